// Host side of PCM outlier rejection: the Pcm<poseT, T> plugin
// (include/KimeraRPGO/outlier/Pcm.h) driving the device kernels.
//
// Bookkeeping stays on the host exactly as the reference keeps it (factor
// classification, groups keyed by ObservationId in a std::unordered_map with
// the reference's hash so that groups are visited in the same order, the
// prefix-trajectory side effects of std::map::operator[]); the trajectories,
// the odometry check, the pairwise test, the adjacency and the clique run on
// the GPU.
#pragma once
#include <cstdint>
#include <functional>
#include <map>
#include <set>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "pcm_kernels.hpp"
#include "stores.hpp"

namespace rpgo {

inline char key_chr(uint64_t k) { return static_cast<char>(static_cast<unsigned char>(k >> 56)); }
// gtsam::Symbol(c, index) as a key
inline uint64_t symbol_key(char c, uint64_t index) {
  return (static_cast<uint64_t>(static_cast<unsigned char>(c)) << 56) | index;
}

// ObservationId (TypeUtils.h:44-58) and its hash (TypeUtils.h:80-88)
struct ObsId {
  char id1, id2;
  bool operator==(const ObsId& o) const {
    return (id1 == o.id1 && id2 == o.id2) || (id2 == o.id1 && id1 == o.id2);
  }
};
struct ObsIdHash {
  size_t operator()(const ObsId& id) const {
    std::hash<char> h;
    return h(id.id1) + h(id.id2) + h(id.id1) * h(id.id2);
  }
};

struct PcmConfig {
  int dim = 3;   // 2 or 3
  int mode = 0;  // 0 Pcm (PoseWithCovariance), 1 PcmSimple (PoseWithNode)
  double odom_threshold = 10.0, lc_threshold = 5.0;
  double odom_trans_threshold = 0.05, odom_rot_threshold = 0.005;
  double dist_trans_threshold = 0.01, dist_rot_threshold = 0.001;
  bool incremental = false;
  std::vector<char> special;  // landmark key prefixes (specialSymbols)
};

struct PcmStats {
  int64_t pair_checks = 0;
  int64_t odom_checks = 0;
};

class PcmEngine {
 public:
  PcmEngine(const PcmConfig& cfg, cudaStream_t st);
  // Pcm::removeOutliers. `values` already holds new_values; factor rows point
  // into `store`. Returns do_optimize; *out is the graph to optimise
  // (odometry, special, inliers).
  bool remove_outliers(const std::vector<FactorRec>& new_factors, const std::set<uint64_t>& new_keys,
                       const ValueStore& values, const FactorStore& store, std::vector<FactorRec>* out);

  size_t num_lc() const { return total_lc_; }
  size_t num_lc_inliers() const { return total_good_lc_; }
  size_t num_odom() const { return nfg_odom_.size(); }
  size_t num_special() const { return nfg_special_.size(); }
  // adjacency of the g-th group in visiting order (host copy, n x words)
  bool adjacency(int g, std::vector<uint32_t>* words, int* n) const;
  const PcmStats& stats() const { return stats_; }
  // For each loop closure of the last graph to optimise (its order): degree
  // in its group's adjacency / (group size - 1), log1p(degree), and the
  // number of its neighbours among the group's consistent set / (set size -
  // 1); zeros where the pairwise check is disabled. 3 floats per closure.
  void closure_stats(std::vector<float>* out);

  // ---- edits (Pcm.h:299-408); each leaves the graph to optimise in *out
  // removeLastLoopClosure(ObservationId): false when the group is unknown or
  // has no closure left; the removed closure's keys in *k1, *k2
  bool remove_last_loop_closure(char prefix_1, char prefix_2, uint64_t* k1, uint64_t* k2,
                                std::vector<FactorRec>* out);
  // removeLastLoopClosure(): the group of the latest accepted closure
  bool remove_last_loop_closure(uint64_t* k1, uint64_t* k2, std::vector<FactorRec>* out);
  void ignore_prefix(char prefix, std::vector<FactorRec>* out);
  void revive_prefix(char prefix, std::vector<FactorRec>* out);
  const std::vector<char>& ignored_prefixes() const { return ignored_; }
  void remove_priors_with_prefix(char prefix, std::vector<FactorRec>* out);

  // ---- multi-robot frame alignment inputs (Pcm.h:1011-1074)
  // robot prefixes in the order their odometry started, sorted in place as
  // the reference sorts robot_order_
  const std::vector<char>& sorted_robot_order();
  // keys of robot `prefix` that its trajectory holds, with their slots
  void robot_slots(char prefix, std::vector<uint64_t>* keys, std::vector<int32_t>* slots) const;
  int32_t find_slot(uint64_t key) const;  // -1 when the trajectory has no entry
  // consistent closures of the group (a, b); false when there is no group
  bool group_closures(char a, char b, std::vector<FactorRec>* out) const;
  const double* traj_pose() const { return traj_pose_.get(); }

 private:
  struct Group {
    std::vector<FactorRec> factors;
    std::vector<int32_t> consistent;  // indices into factors (clique buffer order, duplicates kept)
    int n = 0, words = 0, row_cap = 0;
    // rows of the reference's adj_matrix: 1 for a fresh Measurements
    // (TypeUtils.h:16-33), n after each increment, one less per removal
    int adj_rows = 1;
    DeviceBuffer<uint32_t> adj;  // row_cap x words
    std::vector<int32_t> h_sa, h_sb;
    std::vector<uint8_t> h_flip;
    std::vector<int64_t> h_row;  // factor-store rows of the closures
    DeviceBuffer<int32_t> sa, sb;
    DeviceBuffer<uint8_t> flip;
    DeviceBuffer<double> zp, zc;
    ObsId key{0, 0};
  };
  int32_t slot(uint64_t key);  // trajectory slot, default-initialised when new
  void flush_slots();          // upload defaults / initial poses of new slots
  void ensure_traj_capacity(size_t n);
  TrajView view() const;
  void run_pairwise(Group& g, int old_n, const FactorStore& store);
  // Pcm.h:775-844 for the observations [old_n, n) of landmark `lk`
  void run_landmark_pairwise(Group& g, uint64_t lk, int old_n, const FactorStore& store);
  void grow_adjacency(Group& g, int n);
  bool is_special(char c) const;
  uint64_t landmark_key(const FactorRec& f) const { return is_special(key_chr(f.k1)) ? f.k1 : f.k2; }
  // trajectory slot of `key` as looked up in robot `prefix`'s trajectory: a
  // key of another robot is a default entry of that trajectory
  int32_t slot_in(char prefix, uint64_t key);
  size_t landmark_inliers(Group& g);
  void find_inliers();
  void find_inliers_incremental(const std::unordered_map<ObsId, size_t, ObsIdHash>& num_new);
  // Pcm::buildGraphToOptimize (Pcm.h:977-1005), ignored prefixes left out
  void build_graph(std::vector<FactorRec>* out) const;
  bool remove_last(const ObsId& id, uint64_t* k1, uint64_t* k2, std::vector<FactorRec>* out);
  // clique of the first `rows` closures of a group (indices past the
  // group's closures dropped)
  void clique_of(Group& g, int rows);

  PcmConfig cfg_;
  bool odom_check_ = true, lc_check_ = true;
  cudaStream_t st_;
  int stride_, d_;
  std::unordered_map<uint64_t, int32_t> slots_;
  int32_t num_slots_ = 0;
  size_t traj_cap_ = 0;
  std::vector<std::pair<int32_t, int64_t>> pending_init_;  // slot <- value row (cov zero)
  const ValueStore* values_ = nullptr;
  std::vector<int32_t> pending_default_;
  DeviceBuffer<double> traj_pose_, traj_cov_;
  DeviceBuffer<int32_t> traj_node_;
  DeviceBuffer<uint8_t> traj_rot_;
  std::unordered_set<char> prefix_exists_;
  std::vector<FactorRec> nfg_odom_, nfg_special_;
  std::unordered_map<ObsId, Group, ObsIdHash> groups_;
  std::unordered_map<uint64_t, Group> landmarks_;  // landmarks_ (Pcm.h), keyed by landmark key
  std::map<std::pair<char, uint64_t>, int32_t> foreign_slots_;
  std::vector<ObsId> lc_in_order_;  // loop_closures_in_order_ (Pcm.h:112)
  std::vector<char> ignored_;       // ignored_prefixes_ (Pcm.h:117)
  std::vector<char> robot_order_;   // robot_order_ (Pcm.h:128)
  size_t total_lc_ = 0, total_good_lc_ = 0;
  // scratch
  DeviceBuffer<int32_t> d_src_, d_dst_;
  DeviceBuffer<int64_t> d_rows_;
  DeviceBuffer<double> d_dpose_, d_dcov_, scratch_rec_, scratch_cov_;
  DeviceBuffer<uint8_t> scratch_rot_, d_ok_;
  DeviceBuffer<uint32_t> lower_scratch_;
  CliqueWorkspace clique_ws_;
  PcmStats stats_;
};

}  // namespace rpgo

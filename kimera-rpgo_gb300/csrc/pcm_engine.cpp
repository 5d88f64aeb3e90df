// Pcm<poseT, T>::removeOutliers and friends over device data; see
// pcm_engine.hpp. Reference lines are cited per method.
#include "pcm_engine.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "warm.hpp"

namespace rpgo {

PcmEngine::PcmEngine(const PcmConfig& cfg, cudaStream_t st) : cfg_(cfg), st_(st) {
  stride_ = cfg.dim == 3 ? 12 : 4;
  d_ = cfg.dim == 3 ? 6 : 3;
  // Pcm.h:74-82: a negative threshold disables the check
  if (cfg.odom_threshold < 0 || cfg.odom_rot_threshold < 0 || cfg.odom_trans_threshold < 0) odom_check_ = false;
  if (cfg.lc_threshold < 0 || cfg.dist_rot_threshold < 0 || cfg.dist_trans_threshold < 0) lc_check_ = false;
}

int32_t PcmEngine::slot(uint64_t key) {
  auto it = slots_.find(key);
  if (it != slots_.end()) return it->second;
  const int32_t s = num_slots_++;
  slots_.emplace(key, s);
  pending_default_.push_back(s);
  return s;
}

void PcmEngine::ensure_traj_capacity(size_t n) {
  if (n <= traj_cap_) return;
  size_t c = traj_cap_ ? traj_cap_ : 1024;
  while (c < n) c *= 2;
  const size_t old = traj_cap_;
  auto grow = [&](auto& buf, size_t per) {
    buf.grow(c * per, st_);
    (void)old;
  };
  grow(traj_pose_, stride_);
  grow(traj_cov_, (size_t)d_ * d_);
  grow(traj_node_, 1);
  grow(traj_rot_, 1);
  traj_cap_ = c;
}

TrajView PcmEngine::view() const {
  return TrajView{traj_pose_.get(), traj_cov_.get(), traj_node_.get(), traj_rot_.get()};
}

// std::map::operator[] default entries: identity pose, zero covariance,
// node 0, rotation_info true (GeometryUtils.h:67-73, 203-206); the first pose
// of a new robot prefix takes its value with zero covariance (Pcm.h:534-542).
void PcmEngine::flush_slots() {
  ensure_traj_capacity((size_t)num_slots_);
  if (!pending_default_.empty()) {
    const int32_t lo = *std::min_element(pending_default_.begin(), pending_default_.end());
    const int32_t hi = *std::max_element(pending_default_.begin(), pending_default_.end()) + 1;
    const size_t cnt = (size_t)(hi - lo);
    std::vector<double> pose(cnt * stride_, 0.0), cov(cnt * d_ * d_, 0.0);
    std::vector<int32_t> node(cnt, 0);
    std::vector<uint8_t> rot(cnt, 1);
    for (size_t i = 0; i < cnt; ++i) {
      double* p = &pose[i * stride_];
      if (cfg_.dim == 3) {
        p[0] = p[4] = p[8] = 1.0;
      } else {
        p[0] = 1.0;
      }
    }
    RPGO_CUDA(cudaMemcpyAsync(traj_pose_.get() + (size_t)lo * stride_, pose.data(), pose.size() * sizeof(double),
                              cudaMemcpyHostToDevice, st_));
    RPGO_CUDA(cudaMemcpyAsync(traj_cov_.get() + (size_t)lo * d_ * d_, cov.data(), cov.size() * sizeof(double),
                              cudaMemcpyHostToDevice, st_));
    RPGO_CUDA(cudaMemcpyAsync(traj_node_.get() + lo, node.data(), node.size() * sizeof(int32_t),
                              cudaMemcpyHostToDevice, st_));
    RPGO_CUDA(cudaMemcpyAsync(traj_rot_.get() + lo, rot.data(), rot.size(), cudaMemcpyHostToDevice, st_));
    RPGO_CUDA(cudaStreamSynchronize(st_));
    pending_default_.clear();
  }
  for (auto& pi : pending_init_) {
    const int32_t s = pi.first;
    std::vector<double> cov((size_t)d_ * d_, 0.0);
    int32_t node = 0;
    uint8_t rot = 1;
    RPGO_CUDA(cudaMemcpyAsync(traj_pose_.get() + (size_t)s * stride_, values_->pose() + (size_t)pi.second * stride_,
                              stride_ * sizeof(double), cudaMemcpyDeviceToDevice, st_));
    RPGO_CUDA(cudaMemcpyAsync(traj_cov_.get() + (size_t)s * d_ * d_, cov.data(), cov.size() * sizeof(double),
                              cudaMemcpyHostToDevice, st_));
    RPGO_CUDA(cudaMemcpyAsync(traj_node_.get() + s, &node, sizeof(node), cudaMemcpyHostToDevice, st_));
    RPGO_CUDA(cudaMemcpyAsync(traj_rot_.get() + s, &rot, 1, cudaMemcpyHostToDevice, st_));
    RPGO_CUDA(cudaStreamSynchronize(st_));
  }
  pending_init_.clear();
}

// adjacency capacity: row_cap rows of row_cap/32 + 4 words, zero padded. The
// 16 extra bytes put consecutive row starts in different 128-byte line
// offsets (the clique kernel reads 32 rows side by side; with a power-of-two
// stride they all fall into the same L1 sets) and keep rows 16-byte aligned.
void PcmEngine::grow_adjacency(Group& g, int n) {
  if (n <= g.row_cap) return;
  int cap = g.row_cap ? g.row_cap : 64;
  while (cap < n) cap *= 2;
  const int words = cap / 32 + 4;
  DeviceBuffer<uint32_t> nb((size_t)cap * words);
  nb.zero(st_);
  if (g.n > 0)
    RPGO_CUDA(cudaMemcpy2DAsync(nb.get(), (size_t)words * 4, g.adj.get(), (size_t)g.words * 4, (size_t)g.words * 4,
                                g.n, cudaMemcpyDeviceToDevice, st_));
  g.adj = std::move(nb);
  g.row_cap = cap;
  g.words = words;
}

bool PcmEngine::is_special(char c) const {
  return std::find(cfg_.special.begin(), cfg_.special.end(), c) != cfg_.special.end();
}

int32_t PcmEngine::slot_in(char prefix, uint64_t key) {
  if (key_chr(key) == prefix) return slot(key);
  auto it = foreign_slots_.find({prefix, key});
  if (it != foreign_slots_.end()) return it->second;
  const int32_t s = num_slots_++;
  pending_default_.push_back(s);
  foreign_slots_[{prefix, key}] = s;
  return s;
}

void PcmEngine::run_landmark_pairwise(Group& g, uint64_t lk, int old_n, const FactorStore& store) {
  const int n = (int)g.factors.size();
  if (n <= old_n) return;
  // measurements of every observation (a first observation arrives without
  // a pairwise check, so its row is gathered here); landmark groups are small
  const int add = n - old_n;
  g.zp.resize((size_t)n * stride_);
  g.zc.resize((size_t)n * d_ * d_);
  d_rows_.upload(g.h_row.data(), n, st_);
  gather_rows(n, d_rows_.get(), store.meas(), stride_, g.zp.get(), st_);
  gather_rows(n, d_rows_.get(), store.cov(), d_ * d_, g.zc.get(), st_);
  grow_adjacency(g, n);
  // the new rows and columns start empty
  launch_clear_columns(g.adj.get(), g.words, old_n, old_n, st_);
  RPGO_CUDA(cudaMemsetAsync(g.adj.get() + (size_t)old_n * g.words, 0, sizeof(uint32_t) * (size_t)add * g.words, st_));
  std::vector<int4> desc;
  std::vector<int2> ij;
  for (int j = std::max(old_n, 1); j < n; ++j)
    for (int i = 0; i < j; ++i) {
      const uint64_t ki = g.factors[i].k1, kj = g.factors[j].k1;
      if (ki == lk || kj == lk) continue;  // observation stored landmark -> pose: left inconsistent
      const char p = key_chr(ki);
      if (key_chr(kj) == p) {
        desc.push_back(int4{slot(ki), slot(kj), -1, -1});
      } else {
        const int32_t a0 = slot(symbol_key(p, 0)), sa = slot(ki);
        const int32_t b0 = slot_in(p, symbol_key(key_chr(kj), 0)), sb = slot_in(p, kj);
        desc.push_back(int4{a0, sa, b0, sb});
      }
      ij.push_back(int2{i, j});
    }
  flush_slots();
  if (!desc.empty()) {
    DeviceBuffer<int4> ddesc;
    DeviceBuffer<int2> dij;
    ddesc.upload(desc, st_);
    dij.upload(ij, st_);
    const double th0 = cfg_.mode == 0 ? cfg_.lc_threshold : cfg_.dist_trans_threshold;
    const double th1 = cfg_.mode == 0 ? 0.0 : cfg_.dist_rot_threshold;
    launch_landmark_pairs(cfg_.dim, cfg_.mode, (int)desc.size(), ddesc.get(), dij.get(), g.zp.get(), g.zc.get(),
                          view(), th0, th1, g.adj.get(), g.words, st_);
    RPGO_CUDA(cudaStreamSynchronize(st_));
    stats_.pair_checks += (int64_t)desc.size();
  }
  g.n = n;
  g.adj_rows = n;
}

// findMaxCliqueHeu over a landmark's adjacency (Pcm.h:878-897): always run,
// whatever the loop-closure check setting; a fresh landmark's 1 x 1 zero
// matrix gives its only observation
size_t PcmEngine::landmark_inliers(Group& g) {
  g.consistent.clear();
  const int rows = g.adj_rows;
  std::vector<int32_t> clique;
  int sz = 0;
  if (rows > 0 && g.adj.get() && g.n >= rows) {
    sz = max_clique_heu(rows, g.adj.get(), g.words, 0, -1, &clique, clique_ws_, st_);
  } else if (rows > 0) {
    sz = 1;
    clique.assign(1, 0);
  }
  for (int i = 0; i < sz; ++i)
    if (clique[i] < (int32_t)g.factors.size()) g.consistent.push_back(clique[i]);
  return g.consistent.size();
}

void PcmEngine::run_pairwise(Group& g, int old_n, const FactorStore& store) {
  const int n = (int)g.factors.size();
  if (n <= old_n) return;
  // the new closures' slots (host) and measurements (gathered from the store)
  g.sa.grow(n, st_);
  g.sb.grow(n, st_);
  g.flip.grow(n, st_);
  g.zp.grow((size_t)n * stride_, st_);
  g.zc.grow((size_t)n * d_ * d_, st_);
  const int add = n - old_n;
  RPGO_CUDA(cudaMemcpyAsync(g.sa.get() + old_n, g.h_sa.data() + old_n, add * sizeof(int32_t),
                            cudaMemcpyHostToDevice, st_));
  RPGO_CUDA(cudaMemcpyAsync(g.sb.get() + old_n, g.h_sb.data() + old_n, add * sizeof(int32_t),
                            cudaMemcpyHostToDevice, st_));
  RPGO_CUDA(cudaMemcpyAsync(g.flip.get() + old_n, g.h_flip.data() + old_n, add, cudaMemcpyHostToDevice, st_));
  d_rows_.upload(g.h_row.data() + old_n, add, st_);
  gather_rows(add, d_rows_.get(), store.meas(), stride_, g.zp.get() + (size_t)old_n * stride_, st_);
  gather_rows(add, d_rows_.get(), store.cov(), d_ * d_, g.zc.get() + (size_t)old_n * d_ * d_, st_);
  grow_adjacency(g, n);
  lower_scratch_.resize((size_t)(n - old_n) * g.words);
  const double th0 = cfg_.mode == 0 ? cfg_.lc_threshold : cfg_.dist_trans_threshold;
  const double th1 = cfg_.mode == 0 ? 0.0 : cfg_.dist_rot_threshold;
  launch_pairwise(cfg_.dim, cfg_.mode, n, old_n, g.sa.get(), g.sb.get(), g.flip.get(), g.zp.get(), g.zc.get(),
                  view(), th0, th1, g.adj.get(), g.words, lower_scratch_.get(), st_);
  stats_.pair_checks += (int64_t)n * (n - 1) / 2 - (int64_t)old_n * (old_n - 1) / 2;
  g.n = n;
  g.adj_rows = n;
}

// Pcm.h:851-899
void PcmEngine::find_inliers() {
  total_good_lc_ = 0;
  for (auto& kv : groups_) {
    Group& g = kv.second;
    size_t num;
    if (lc_check_) {
      std::vector<int32_t> clique;
      const int sz = max_clique_heu(g.n, g.adj.get(), g.words, 0, -1, &clique, clique_ws_, st_);
      // after a removal that left fewer than two closures the reference keeps
      // its larger adjacency; indices past the closures are dropped
      g.consistent.clear();
      for (int i = 0; i < sz; ++i)
        if (clique[i] < (int32_t)g.factors.size()) g.consistent.push_back(clique[i]);
      num = g.consistent.size();
    } else {
      g.consistent.resize(g.factors.size());
      for (size_t i = 0; i < g.factors.size(); ++i) g.consistent[i] = (int32_t)i;
      num = g.factors.size();
    }
    total_good_lc_ += num;
  }
  for (auto& kv : landmarks_) total_good_lc_ += landmark_inliers(kv.second);
}

// Pcm.h:906-970 with findMaxCliqueHeuIncremental (GraphUtils.cpp:30-44)
void PcmEngine::find_inliers_incremental(const std::unordered_map<ObsId, size_t, ObsIdHash>& num_new) {
  total_good_lc_ = 0;
  for (const auto& kv : num_new) {
    Group& g = groups_[kv.first];
    const int prev = (int)g.consistent.size();
    std::vector<int32_t> clique;
    int sz;
    if (lc_check_) {
      const int first = g.n - (int)kv.second;
      sz = max_clique_heu(g.n, g.adj.get(), g.words, first, prev, &clique, clique_ws_, st_);
    } else {
      // the adjacency stays the 1x1 zero matrix of a fresh Measurements
      // (TypeUtils.h:16-33): only a first, lone closure can be taken
      sz = prev;
      if (kv.second == 1 && prev < 1) {
        sz = 1;
        clique.assign(1, 0);
      }
    }
    if (sz > prev) {
      g.consistent.clear();
      for (int i = 0; i < sz; ++i)
        if (clique[i] < (int32_t)g.factors.size()) g.consistent.push_back(clique[i]);
    }
  }
  for (const auto& kv : groups_) total_good_lc_ += kv.second.consistent.size();
  for (auto& kv : landmarks_) total_good_lc_ += landmark_inliers(kv.second);
}

bool PcmEngine::remove_outliers(const std::vector<FactorRec>& new_factors, const std::set<uint64_t>& new_keys,
                                const ValueStore& values, const FactorStore& store, std::vector<FactorRec>* out) {
  values_ = &values;
  if (new_factors.empty()) return false;
  bool do_optimize = false;
  // ---- classification (Pcm.h:164-240)
  std::vector<int32_t> src, dst;
  std::vector<int64_t> orows;
  std::vector<const FactorRec*> lcs;
  for (const auto& f : new_factors) {
    if (f.kind == 0) {
      if (is_special(key_chr(f.k1)) || is_special(key_chr(f.k2))) {
        if (new_keys.count(f.k1) || new_keys.count(f.k2)) {
          // first observation of a landmark (Pcm.h:209-220): a fresh
          // Measurements holding it, replacing any earlier one
          Group g;
          g.factors.push_back(f);
          g.consistent.push_back(0);
          g.h_sa.push_back(0);
          g.h_sb.push_back(0);
          g.h_flip.push_back(0);
          g.h_row.push_back(f.row);
          landmarks_[landmark_key(f)] = std::move(g);
          ++total_lc_;
        } else if (f.k1 != f.k2) {
          lcs.push_back(&f);
        }
      } else if (f.k1 + 1 == f.k2 && new_keys.count(f.k2)) {
        // updateOdom (Pcm.h:516-557)
        nfg_odom_.push_back(f);
        const char prefix = key_chr(f.k2);
        if (!prefix_exists_.count(prefix)) {
          prefix_exists_.insert(prefix);
          robot_order_.push_back(prefix);
          const int32_t s0 = slot(f.k1);
          pending_init_.emplace_back(s0, values.row(f.k1));
        }
        src.push_back(slot(f.k1));
        dst.push_back(slot(f.k2));
        orows.push_back(f.row);
      } else if (f.k1 != f.k2) {
        lcs.push_back(&f);
      }
    } else {
      nfg_special_.push_back(f);
      do_optimize = true;
    }
  }
  if (!src.empty()) {
    flush_slots();
    d_src_.upload(src, st_);
    d_dst_.upload(dst, st_);
    d_rows_.upload(orows, st_);
    d_dpose_.resize(orows.size() * stride_);
    d_dcov_.resize(orows.size() * d_ * d_);
    gather_rows((int64_t)orows.size(), d_rows_.get(), store.meas(), stride_, d_dpose_.get(), st_);
    gather_rows((int64_t)orows.size(), d_rows_.get(), store.cov(), d_ * d_, d_dcov_.get(), st_);
    launch_traj_scan(cfg_.dim, cfg_.mode, (int64_t)src.size(), d_src_.get(), d_dst_.get(), d_dpose_.get(),
                     d_dcov_.get(), view(), scratch_rec_, scratch_cov_, scratch_rot_, st_);
  }
  if (!lcs.empty()) {
    // ---- odometry consistency of intra-robot closures (Pcm.h:455-465, 604-629)
    std::vector<int32_t> ci, cj, owner;
    std::vector<int64_t> crow;
    for (size_t k = 0; k < lcs.size(); ++k) {
      const FactorRec& f = *lcs[k];
      if (!values.has(f.k1) || !values.has(f.k2)) continue;
      if (key_chr(f.k1) != key_chr(f.k2) || !odom_check_) continue;
      if (is_special(key_chr(f.k1))) continue;
      prefix_exists_.insert(key_chr(f.k1));
      ci.push_back(slot(f.k1));
      cj.push_back(slot(f.k2));
      owner.push_back((int32_t)k);
      crow.push_back(f.row);
    }
    std::vector<uint8_t> passed(lcs.size(), 1);
    if (!ci.empty()) {
      flush_slots();
      DeviceBuffer<int32_t> di, dj;
      DeviceBuffer<double> dzp(crow.size() * stride_), dzc(crow.size() * d_ * d_);
      di.upload(ci, st_);
      dj.upload(cj, st_);
      d_rows_.upload(crow, st_);
      gather_rows((int64_t)crow.size(), d_rows_.get(), store.meas(), stride_, dzp.get(), st_);
      gather_rows((int64_t)crow.size(), d_rows_.get(), store.cov(), d_ * d_, dzc.get(), st_);
      d_ok_.resize(ci.size());
      const double th0 = cfg_.mode == 0 ? cfg_.odom_threshold : cfg_.odom_trans_threshold;
      const double th1 = cfg_.mode == 0 ? 0.0 : cfg_.odom_rot_threshold;
      launch_odom_check(cfg_.dim, cfg_.mode, (int64_t)ci.size(), di.get(), dj.get(), dzp.get(), dzc.get(), view(),
                        th0, th1, d_ok_.get(), st_);
      std::vector<uint8_t> ok(ci.size());
      d_ok_.download(ok.data(), ok.size(), st_);
      RPGO_CUDA(cudaStreamSynchronize(st_));
      for (size_t q = 0; q < ci.size(); ++q) passed[owner[q]] = ok[q];
      stats_.odom_checks += (int64_t)ci.size();
    }
    // ---- grouping (Pcm.h:466-486)
    std::unordered_map<ObsId, size_t, ObsIdHash> num_new;
    std::vector<std::pair<ObsId, int>> touched;
    std::vector<std::pair<uint64_t, int>> touched_lm;
    for (size_t k = 0; k < lcs.size(); ++k) {
      const FactorRec& f = *lcs[k];
      if (!values.has(f.k1) || !values.has(f.k2)) continue;
      if (is_special(key_chr(f.k1)) || is_special(key_chr(f.k2))) {
        // landmark re-observation (Pcm.h:440-454)
        const uint64_t lk = landmark_key(f);
        Group& lg = landmarks_[lk];
        bool seen = false;
        for (auto& t : touched_lm)
          if (t.first == lk) seen = true;
        if (!seen) touched_lm.emplace_back(lk, (int)lg.factors.size());
        lg.factors.push_back(f);
        lg.h_sa.push_back(0);
        lg.h_sb.push_back(0);
        lg.h_flip.push_back(0);
        lg.h_row.push_back(f.row);
        ++total_lc_;
        continue;
      }
      if (!passed[k]) continue;
      const ObsId id{key_chr(f.k1), key_chr(f.k2)};
      num_new[id]++;
      auto it = groups_.find(id);
      if (it == groups_.end()) {
        it = groups_.emplace(id, Group()).first;
        it->second.key = id;
      }
      Group& g = it->second;
      bool seen = false;
      for (auto& t : touched)
        if (t.first == id) seen = true;
      if (!seen) touched.emplace_back(id, (int)g.factors.size());
      g.factors.push_back(f);
      g.h_sa.push_back(slot(f.k1));
      g.h_sb.push_back(slot(f.k2));
      g.h_flip.push_back(key_chr(f.k1) != g.key.id1 ? 1 : 0);
      g.h_row.push_back(f.row);
      lc_in_order_.push_back(id);
      ++total_lc_;
    }
    if (lc_check_) {
      flush_slots();
      for (auto& t : touched) {
        Group& g = groups_[t.first];
        if (g.factors.size() >= 2) {
          // areLoopsConsistent reads both robots' trajectories (Pcm.h:699-710)
          prefix_exists_.insert(g.key.id1);
          prefix_exists_.insert(g.key.id2);
        }
        run_pairwise(g, t.second, store);
      }
    }
    if (!touched_lm.empty()) flush_slots();
    for (auto& t : touched_lm) run_landmark_pairwise(landmarks_[t.first], t.first, t.second, store);
    if (cfg_.incremental) find_inliers_incremental(num_new);
    else find_inliers();
    do_optimize = true;
  }
  build_graph(out);
  return do_optimize;
}

void PcmEngine::build_graph(std::vector<FactorRec>* out) const {
  out->clear();
  out->insert(out->end(), nfg_odom_.begin(), nfg_odom_.end());
  out->insert(out->end(), nfg_special_.begin(), nfg_special_.end());
  auto ignored = [this](char c) { return std::find(ignored_.begin(), ignored_.end(), c) != ignored_.end(); };
  for (const auto& kv : groups_) {
    if (ignored(kv.first.id1) || ignored(kv.first.id2)) continue;
    for (int32_t idx : kv.second.consistent) out->push_back(kv.second.factors[idx]);
  }
  for (const auto& kv : landmarks_)
    for (int32_t idx : kv.second.consistent) out->push_back(kv.second.factors[idx]);
}

void PcmEngine::clique_of(Group& g, int rows) {
  g.consistent.clear();
  std::vector<int32_t> clique;
  int sz = 0;
  if (lc_check_ && rows > 0 && g.adj.get()) {
    sz = max_clique_heu(rows, g.adj.get(), g.words, 0, -1, &clique, clique_ws_, st_);
  } else if (rows > 0) {
    // the greedy clique of an edgeless graph is its first vertex
    sz = 1;
    clique.assign(1, 0);
  }
  for (int i = 0; i < sz; ++i)
    if (clique[i] < (int32_t)g.factors.size()) g.consistent.push_back(clique[i]);
}

// Pcm.h:299-342. Deviation: a group whose closures are all gone returns
// false (the reference would index its empty factor list).
bool PcmEngine::remove_last(const ObsId& id, uint64_t* k1, uint64_t* k2, std::vector<FactorRec>* out) {
  auto it = groups_.find(id);
  if (it == groups_.end()) return false;
  Group& g = it->second;
  const int num_lc = g.adj_rows;
  if (num_lc <= 0 || g.factors.empty()) return false;
  *k1 = g.factors.back().k1;
  *k2 = g.factors.back().k2;
  g.factors.pop_back();
  g.h_sa.pop_back();
  g.h_sb.pop_back();
  g.h_flip.pop_back();
  g.h_row.pop_back();
  if (g.factors.size() < 2) {
    g.consistent.clear();
    for (size_t i = 0; i < g.factors.size(); ++i) g.consistent.push_back((int32_t)i);
  } else {
    // adj_matrix.block(0, 0, numLC - 1, numLC - 1): the removed closure's
    // column is cleared so that the degrees of the kept rows are exact
    const int m = num_lc - 1;
    if (g.adj.get() && g.n > m) {
      launch_clear_columns(g.adj.get(), g.words, m, m, st_);
      g.n = m;
    }
    g.adj_rows = m;
    clique_of(g, m);
  }
  build_graph(out);
  return true;
}

bool PcmEngine::remove_last_loop_closure(char prefix_1, char prefix_2, uint64_t* k1, uint64_t* k2,
                                         std::vector<FactorRec>* out) {
  return remove_last(ObsId{prefix_1, prefix_2}, k1, k2, out);
}

// Pcm.h:347-353
bool PcmEngine::remove_last_loop_closure(uint64_t* k1, uint64_t* k2, std::vector<FactorRec>* out) {
  if (lc_in_order_.empty()) return false;
  const ObsId id = lc_in_order_.back();
  lc_in_order_.pop_back();
  return remove_last(id, k1, k2, out);
}

// Pcm.h:357-365
void PcmEngine::ignore_prefix(char prefix, std::vector<FactorRec>* out) {
  if (std::find(ignored_.begin(), ignored_.end(), prefix) == ignored_.end()) ignored_.push_back(prefix);
  build_graph(out);
}

// Pcm.h:369-376
void PcmEngine::revive_prefix(char prefix, std::vector<FactorRec>* out) {
  ignored_.erase(std::remove(ignored_.begin(), ignored_.end(), prefix), ignored_.end());
  build_graph(out);
}

// Pcm.h:386-408: priors of keys with this prefix leave the special factors
void PcmEngine::remove_priors_with_prefix(char prefix, std::vector<FactorRec>* out) {
  std::vector<FactorRec> kept;
  for (const auto& f : nfg_special_)
    if (f.kind != 1 || key_chr(f.k1) != prefix) kept.push_back(f);
  nfg_special_.swap(kept);
  build_graph(out);
}

void PcmEngine::closure_stats(std::vector<float>* out) {
  out->clear();
  auto ignored = [this](char c) { return std::find(ignored_.begin(), ignored_.end(), c) != ignored_.end(); };
  for (auto& kv : groups_) {
    Group& g = kv.second;
    const int count = (int)g.consistent.size();
    if (count == 0 || ignored(kv.first.id1) || ignored(kv.first.id2)) continue;
    if (!lc_check_ || g.n == 0 || !g.adj.get()) {
      out->insert(out->end(), (size_t)count * 3, 0.f);
      continue;
    }
    std::vector<uint32_t> mask((size_t)g.words, 0u);
    for (int32_t i : g.consistent) mask[(size_t)i >> 5] |= 1u << (i & 31);
    int members = 0;
    for (uint32_t w : mask) members += __builtin_popcount(w);
    DeviceBuffer<uint32_t> dmask;
    DeviceBuffer<int32_t> drows, ddeg((size_t)count), dsup((size_t)count);
    dmask.upload(mask, st_);
    drows.upload(g.consistent, st_);
    launch_row_stats(g.n, g.adj.get(), g.words, dmask.get(), drows.get(), count, ddeg.get(), dsup.get(), st_);
    std::vector<int32_t> deg((size_t)count), sup((size_t)count);
    ddeg.download(deg.data(), deg.size(), st_);
    dsup.download(sup.data(), sup.size(), st_);
    RPGO_CUDA(cudaStreamSynchronize(st_));
    for (int k = 0; k < count; ++k) {
      out->push_back((float)deg[k] / (float)std::max(1, g.n - 1));
      out->push_back((float)std::log1p((double)deg[k]));
      out->push_back((float)sup[k] / (float)std::max(1, members - 1));
    }
  }
  for (const auto& kv : landmarks_) out->insert(out->end(), kv.second.consistent.size() * 3, 0.f);
}

const std::vector<char>& PcmEngine::sorted_robot_order() {
  std::sort(robot_order_.begin(), robot_order_.end());
  return robot_order_;
}

void PcmEngine::robot_slots(char prefix, std::vector<uint64_t>* keys, std::vector<int32_t>* slots) const {
  keys->clear();
  slots->clear();
  for (const auto& kv : slots_)
    if (key_chr(kv.first) == prefix) {
      keys->push_back(kv.first);
      slots->push_back(kv.second);
    }
}

int32_t PcmEngine::find_slot(uint64_t key) const {
  auto it = slots_.find(key);
  return it == slots_.end() ? -1 : it->second;
}

bool PcmEngine::group_closures(char a, char b, std::vector<FactorRec>* out) const {
  out->clear();
  auto it = groups_.find(ObsId{a, b});
  if (it == groups_.end()) return false;
  for (int32_t idx : it->second.consistent) out->push_back(it->second.factors[idx]);
  return true;
}

bool PcmEngine::adjacency(int gi, std::vector<uint32_t>* words, int* n) const {
  int k = 0;
  for (const auto& kv : groups_) {
    if (k++ != gi) continue;
    const Group& g = kv.second;
    *n = g.n;
    const int w = (g.n + 31) / 32;
    words->assign((size_t)g.n * w, 0u);
    if (g.n == 0) return true;
    RPGO_CUDA(cudaMemcpy2DAsync(words->data(), (size_t)w * 4, g.adj.get(), (size_t)g.words * 4, (size_t)w * 4, g.n,
                                cudaMemcpyDeviceToHost, st_));
    RPGO_CUDA(cudaStreamSynchronize(st_));
    return true;
  }
  return false;
}

}  // namespace rpgo

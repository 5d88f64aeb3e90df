// rpgo_gb300.hpp — C++ facade of the GB300-native Kimera-RPGO robust back-end.
//
// Header-only, GTSAM-free. It keeps the class API of the reference,
//   KimeraRPGO::RobustSolverParams (include/KimeraRPGO/SolverParams.h:33-299)
//   KimeraRPGO::RobustSolver       (include/KimeraRPGO/RobustSolver.h:30-139,
//                                   GenericSolver.h:30-70)
// with the same method names, default arguments and setter semantics, over
// the C ABI of rpgo_gb300.h (link librpgo_gb300.so). GTSAM types become
// plain containers: FactorGraph (structure of arrays, noise models as
// covariance + square-root information) and Values (keys + flat poses in the
// pose layout of rpgo_gb300.h). Where the reference prints a warning and
// exits, or lets a GTSAM exception escape, the facade throws rpgo::Error
// carrying the C ABI status.
#ifndef RPGO_GB300_HPP
#define RPGO_GB300_HPP

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rpgo_gb300.h"

namespace rpgo {

using Key = uint64_t;
// gtsam::Symbol(c, j)
inline Key symbol(char c, uint64_t j) { return (static_cast<uint64_t>(static_cast<unsigned char>(c)) << 56) | j; }
inline char symbolChr(Key k) { return static_cast<char>(static_cast<unsigned char>(k >> 56)); }
inline uint64_t symbolIndex(Key k) { return k & ((uint64_t(1) << 56) - 1); }

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char* call) {
  if (status != RPGO_OK) throw Error(status, std::string(call) + " failed with status " + std::to_string(status));
}

// ---------------------------------------------------------------- parameters
// SolverParams.h:13-31
enum class Solver { LM = RPGO_SOLVER_LM, GN = RPGO_SOLVER_GN };
enum class OutlierRemovalMethod {
  NONE = RPGO_OUTLIER_NONE,
  PCM2D = RPGO_OUTLIER_PCM2D,
  PCM3D = RPGO_OUTLIER_PCM3D,
  PCM_Simple2D = RPGO_OUTLIER_PCM_SIMPLE2D,
  PCM_Simple3D = RPGO_OUTLIER_PCM_SIMPLE3D
};
enum class Verbosity { UPDATE = RPGO_VERBOSITY_UPDATE, QUIET = RPGO_VERBOSITY_QUIET, VERBOSE = RPGO_VERBOSITY_VERBOSE };
enum class MultiRobotAlignMethod { NONE = RPGO_ALIGN_NONE, L2 = RPGO_ALIGN_L2, GNC = RPGO_ALIGN_GNC };

// SolverParams.h:33-56
struct PcmParams {
  double odom_threshold = 10.0;
  double lc_threshold = 5.0;
  double odom_trans_threshold = 0.05;
  double odom_rot_threshold = 0.005;
  double dist_trans_threshold = 0.01;
  double dist_rot_threshold = 0.001;
  bool incremental = false;
};

// SolverParams.h:58-78
struct GncParams {
  enum class GncThresholdMode { COST = 0u, PROBABILITY = 1u };
  GncThresholdMode gnc_threshold_mode_ = GncThresholdMode::PROBABILITY;
  double gnc_inlier_threshold_ = 0.9;
  size_t max_iterations_ = 100;
  double mu_step_ = 1.4;
  double relative_cost_tol_ = 1e-5;
  double weights_tol_ = 1e-4;
  bool fix_prev_inliers_ = false;
  bool bias_odom_ = false;
};

// SolverParams.h:80-299: the same public fields and setters. `dim` is the
// pose dimension used when outlier rejection is off (the reference takes it
// from its template argument); `linear_solver` picks the LM step's solver.
struct RobustSolverParams {
  Solver solver = Solver::LM;
  OutlierRemovalMethod outlierRemovalMethod = OutlierRemovalMethod::PCM3D;
  std::vector<char> specialSymbols;
  Verbosity verbosity = Verbosity::UPDATE;
  bool log_output = false;
  std::string log_folder;
  PcmParams pcm_params;
  GncParams gnc_params;
  bool lm_diagonal_damping = true;
  MultiRobotAlignMethod multirobot_align_method = MultiRobotAlignMethod::NONE;
  double multirobot_align_gnc_prob = 0.99;
  bool use_gnc_ = false;
  int dim = 3;
  int linear_solver = RPGO_LINEAR_CHOLESKY;

  void setNoRejection(Verbosity verbos = Verbosity::UPDATE) {
    outlierRemovalMethod = OutlierRemovalMethod::NONE;
    verbosity = verbos;
  }
  void setIncremental() { pcm_params.incremental = true; }
  void setLmDiagonalDamping(bool diagonal_damping) { lm_diagonal_damping = diagonal_damping; }
  void setPcm2DParams(double odomThreshold, double lcThreshold, Verbosity verbos = Verbosity::UPDATE) {
    outlierRemovalMethod = OutlierRemovalMethod::PCM2D;
    pcm_params.odom_threshold = odomThreshold;
    pcm_params.lc_threshold = lcThreshold;
    verbosity = verbos;
  }
  void setPcm3DParams(double odomThreshold, double lcThreshold, Verbosity verbos = Verbosity::UPDATE) {
    outlierRemovalMethod = OutlierRemovalMethod::PCM3D;
    pcm_params.odom_threshold = odomThreshold;
    pcm_params.lc_threshold = lcThreshold;
    verbosity = verbos;
  }
  void setPcmSimple2DParams(double transThreshold, double rotThreshold, Verbosity verbos = Verbosity::UPDATE) {
    setPcmSimple2DParams(transThreshold, rotThreshold, transThreshold, rotThreshold, verbos);
  }
  void setPcmSimple3DParams(double transThreshold, double rotThreshold, Verbosity verbos = Verbosity::UPDATE) {
    setPcmSimple3DParams(transThreshold, rotThreshold, transThreshold, rotThreshold, verbos);
  }
  void setPcmSimple2DParams(double transOdomThreshold, double rotOdomThreshold, double transPcmThreshold,
                            double rotPcmThreshold, Verbosity verbos = Verbosity::UPDATE) {
    outlierRemovalMethod = OutlierRemovalMethod::PCM_Simple2D;
    setSimple(transOdomThreshold, rotOdomThreshold, transPcmThreshold, rotPcmThreshold, verbos);
  }
  void setPcmSimple3DParams(double transOdomThreshold, double rotOdomThreshold, double transPcmThreshold,
                            double rotPcmThreshold, Verbosity verbos = Verbosity::UPDATE) {
    outlierRemovalMethod = OutlierRemovalMethod::PCM_Simple3D;
    setSimple(transOdomThreshold, rotOdomThreshold, transPcmThreshold, rotPcmThreshold, verbos);
  }
  void setGncInlierCostThresholdsAtProbability(const double& alpha, const size_t& max_iterations = 100,
                                               const double& mu_step = 1.4, const double& rel_cost_tol = 1e-5,
                                               const double& weight_tol = 1e-4, const bool& fix_prev_inliers = false,
                                               const bool& bias_odom = false) {
    setGnc(GncParams::GncThresholdMode::PROBABILITY, alpha, max_iterations, mu_step, rel_cost_tol, weight_tol,
           fix_prev_inliers, bias_odom);
  }
  void setGncInlierCostThresholds(const double& cost, const size_t& max_iterations = 100,
                                  const double& mu_step = 1.4, const double& rel_cost_tol = 1e-5,
                                  const double& weight_tol = 1e-4, const bool& fix_prev_inliers = false,
                                  const bool& bias_odom = false) {
    setGnc(GncParams::GncThresholdMode::COST, cost, max_iterations, mu_step, rel_cost_tol, weight_tol,
           fix_prev_inliers, bias_odom);
  }
  void gncFixInliers() { gnc_params.fix_prev_inliers_ = true; }
  void gncBiasOdom() { gnc_params.bias_odom_ = true; }
  void setMultiRobotAlignMethod(MultiRobotAlignMethod method) { multirobot_align_method = method; }
  void setMultiRobotGncAlignProbability(double probability) { multirobot_align_gnc_prob = probability; }
  void logOutput(const std::string& output_folder) {
    log_output = true;
    log_folder = output_folder;
  }

  // The flat C struct. Throws rpgo::Error(RPGO_ERR_ARG) for values the C ABI
  // cannot represent (too many special symbols, an iteration count beyond
  // int32, a dimension other than 2 or 3).
  rpgo_params toC() const {
    if (specialSymbols.size() > RPGO_MAX_SPECIAL_SYMBOLS)
      throw Error(RPGO_ERR_ARG, "RobustSolverParams: more than RPGO_MAX_SPECIAL_SYMBOLS special symbols");
    if (gnc_params.max_iterations_ > 0x7fffffffu)
      throw Error(RPGO_ERR_ARG, "RobustSolverParams: gnc max_iterations beyond int32");
    if (dim != 2 && dim != 3) throw Error(RPGO_ERR_ARG, "RobustSolverParams: dim must be 2 or 3");
    rpgo_params p;
    rpgo_params_default(&p);
    p.solver = static_cast<int32_t>(solver);
    p.outlier_removal = static_cast<int32_t>(outlierRemovalMethod);
    p.verbosity = static_cast<int32_t>(verbosity);
    p.dim = dim;
    p.odom_threshold = pcm_params.odom_threshold;
    p.lc_threshold = pcm_params.lc_threshold;
    p.odom_trans_threshold = pcm_params.odom_trans_threshold;
    p.odom_rot_threshold = pcm_params.odom_rot_threshold;
    p.dist_trans_threshold = pcm_params.dist_trans_threshold;
    p.dist_rot_threshold = pcm_params.dist_rot_threshold;
    p.incremental = pcm_params.incremental ? 1 : 0;
    p.use_gnc = use_gnc_ ? 1 : 0;
    p.gnc_threshold_mode = static_cast<int32_t>(gnc_params.gnc_threshold_mode_);
    p.gnc_inlier_threshold = gnc_params.gnc_inlier_threshold_;
    p.gnc_max_iterations = static_cast<int32_t>(gnc_params.max_iterations_);
    p.gnc_mu_step = gnc_params.mu_step_;
    p.gnc_relative_cost_tol = gnc_params.relative_cost_tol_;
    p.gnc_weights_tol = gnc_params.weights_tol_;
    p.gnc_fix_prev_inliers = gnc_params.fix_prev_inliers_ ? 1 : 0;
    p.gnc_bias_odom = gnc_params.bias_odom_ ? 1 : 0;
    p.lm_diagonal_damping = lm_diagonal_damping ? 1 : 0;
    p.linear_solver = linear_solver;
    p.num_special_symbols = static_cast<int32_t>(specialSymbols.size());
    for (size_t i = 0; i < specialSymbols.size(); ++i) p.special_symbols[i] = specialSymbols[i];
    p.multirobot_align_method = static_cast<int32_t>(multirobot_align_method);
    p.multirobot_align_gnc_prob = multirobot_align_gnc_prob;
    return p;
  }
  // pose dimension the solver will use (2 for the 2D outlier removers)
  int poseDim() const {
    if (outlierRemovalMethod == OutlierRemovalMethod::PCM2D ||
        outlierRemovalMethod == OutlierRemovalMethod::PCM_Simple2D)
      return 2;
    if (outlierRemovalMethod == OutlierRemovalMethod::NONE) return dim;
    return 3;
  }

 private:
  void setSimple(double to, double ro, double tp, double rp, Verbosity verbos) {
    pcm_params.odom_trans_threshold = to;
    pcm_params.odom_rot_threshold = ro;
    pcm_params.dist_trans_threshold = tp;
    pcm_params.dist_rot_threshold = rp;
    verbosity = verbos;
  }
  void setGnc(GncParams::GncThresholdMode mode, double thr, size_t it, double mu, double rel, double wt, bool fix,
              bool bias) {
    use_gnc_ = true;
    gnc_params.gnc_threshold_mode_ = mode;
    gnc_params.gnc_inlier_threshold_ = thr;
    gnc_params.max_iterations_ = it;
    gnc_params.mu_step_ = mu;
    gnc_params.relative_cost_tol_ = rel;
    gnc_params.weights_tol_ = wt;
    gnc_params.fix_prev_inliers_ = fix;
    gnc_params.bias_odom_ = bias;
  }
};

// ---------------------------------------------------------------- graph containers
inline int poseStride(int dim) { return dim == 3 ? 12 : 4; }

// gtsam::Values: keys and poses (stride 12 for Pose3, 4 for Pose2)
struct Values {
  int dim = 3;
  std::vector<Key> keys;
  std::vector<double> poses;
  explicit Values(int d = 3) : dim(d) {}
  size_t size() const { return keys.size(); }
  bool empty() const { return keys.empty(); }
  void insert(Key k, const double* pose) {
    keys.push_back(k);
    poses.insert(poses.end(), pose, pose + poseStride(dim));
  }
  bool exists(Key k) const {
    for (Key x : keys)
      if (x == k) return true;
    return false;
  }
  // pose of key k (throws rpgo::Error(RPGO_ERR_KEY) when absent)
  std::vector<double> at(Key k) const {
    for (size_t i = 0; i < keys.size(); ++i)
      if (keys[i] == k)
        return std::vector<double>(poses.begin() + (ptrdiff_t)(i * poseStride(dim)),
                                   poses.begin() + (ptrdiff_t)((i + 1) * poseStride(dim)));
    throw Error(RPGO_ERR_KEY, "Values::at: key not found");
  }
  rpgo_value_batch batch() const { return rpgo_value_batch{(int64_t)keys.size(), keys.data(), poses.data()}; }
};

// gtsam::NonlinearFactorGraph of BetweenFactor / PriorFactor with Gaussian
// noise models: per factor the measured pose, the covariance and the
// square-root information R (upper triangular, R^T R = covariance^-1).
struct FactorGraph {
  int dim = 3;
  std::vector<int32_t> kind;
  std::vector<Key> key_front, key_back;
  std::vector<double> measured, covariance, sqrt_information;
  explicit FactorGraph(int d = 3) : dim(d) {}
  size_t size() const { return kind.size(); }
  bool empty() const { return kind.empty(); }
  // BetweenFactor(from, to, measured, Gaussian::Covariance(covariance))
  void addBetween(Key from, Key to, const double* pose, const double* cov) { push(RPGO_FACTOR_BETWEEN, from, to, pose, cov); }
  // PriorFactor(key, measured, Gaussian::Covariance(covariance))
  void addPrior(Key key, const double* pose, const double* cov) { push(RPGO_FACTOR_PRIOR, key, key, pose, cov); }
  void add(const FactorGraph& other) {
    if (other.dim != dim) throw Error(RPGO_ERR_ARG, "FactorGraph::add: dimension differs");
    kind.insert(kind.end(), other.kind.begin(), other.kind.end());
    key_front.insert(key_front.end(), other.key_front.begin(), other.key_front.end());
    key_back.insert(key_back.end(), other.key_back.begin(), other.key_back.end());
    measured.insert(measured.end(), other.measured.begin(), other.measured.end());
    covariance.insert(covariance.end(), other.covariance.begin(), other.covariance.end());
    sqrt_information.insert(sqrt_information.end(), other.sqrt_information.begin(), other.sqrt_information.end());
  }
  rpgo_factor_batch batch() const {
    return rpgo_factor_batch{(int64_t)kind.size(), kind.data(), key_front.data(), key_back.data(),
                             measured.data(), covariance.data(), sqrt_information.data()};
  }

 private:
  void push(int32_t k, Key a, Key b, const double* pose, const double* cov) {
    const int d = dim == 3 ? 6 : 3;
    std::vector<double> R(d * d);
    if (!sqrtInformation(cov, d, R.data())) throw Error(RPGO_ERR_ARG, "FactorGraph: covariance not positive definite");
    kind.push_back(k);
    key_front.push_back(a);
    key_back.push_back(b);
    measured.insert(measured.end(), pose, pose + poseStride(dim));
    covariance.insert(covariance.end(), cov, cov + d * d);
    sqrt_information.insert(sqrt_information.end(), R.begin(), R.end());
  }
  // R upper triangular with R^T R = C^-1: the transposed Cholesky factor of
  // the information C^-1 (the covariance's Cholesky factor inverted).
  static bool sqrtInformation(const double* C, int d, double* R) {
    double Lc[36] = {0}, Li[36] = {0}, I[36] = {0}, Lf[36] = {0};
    if (!chol(C, d, Lc)) return false;
    for (int j = 0; j < d; ++j)  // Li = Lc^-1 (lower)
      for (int i = j; i < d; ++i) {
        double s = (i == j) ? 1.0 : 0.0;
        for (int k = j; k < i; ++k) s -= Lc[i * d + k] * Li[k * d + j];
        Li[i * d + j] = s / Lc[i * d + i];
      }
    for (int i = 0; i < d; ++i)  // information = Li^T Li
      for (int j = 0; j < d; ++j) {
        double s = 0.0;
        for (int k = 0; k < d; ++k) s += Li[k * d + i] * Li[k * d + j];
        I[i * d + j] = s;
      }
    if (!chol(I, d, Lf)) return false;
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) R[i * d + j] = Lf[j * d + i];
    return true;
  }
  static bool chol(const double* A, int d, double* L) {
    for (int i = 0; i < d; ++i)
      for (int j = 0; j <= i; ++j) {
        double s = A[i * d + j];
        for (int k = 0; k < j; ++k) s -= L[i * d + k] * L[j * d + k];
        if (i == j) {
          if (!(s > 0.0)) return false;
          L[i * d + i] = std::sqrt(s);
        } else {
          L[i * d + j] = s / L[j * d + j];
        }
      }
    return true;
  }
};

// TypeUtils.h:35-41
struct Edge {
  Key from_key;
  Key to_key;
};
using EdgePtr = std::unique_ptr<const Edge>;

// ---------------------------------------------------------------- solver
class RobustSolver {
 public:
  explicit RobustSolver(const RobustSolverParams& params) : params_(params), dim_(params.poseDim()) {
    const rpgo_params p = params.toC();
    h_ = rpgo_create(&p);
    if (!h_) throw Error(RPGO_ERR_CUDA, "rpgo_create failed (bad parameters or no usable CUDA device)");
  }
  ~RobustSolver() {
    if (h_) rpgo_destroy(h_);
  }
  RobustSolver(const RobustSolver&) = delete;
  RobustSolver& operator=(const RobustSolver&) = delete;
  RobustSolver(RobustSolver&& o) noexcept : params_(std::move(o.params_)), dim_(o.dim_), h_(o.h_) { o.h_ = nullptr; }

  // RobustSolver::update (RobustSolver.h:65-67)
  void update(const FactorGraph& factors, const Values& values = Values(), bool optimize_graph = true) {
    const rpgo_factor_batch f = factors.batch();
    const rpgo_value_batch v = values.batch();
    check(rpgo_update(h_, &f, &v, optimize_graph ? 1 : 0), "rpgo_update");
  }
  // RobustSolver::forceUpdate (RobustSolver.h:53-55)
  void forceUpdate(const FactorGraph& nfg = FactorGraph(), const Values& values = Values()) {
    const rpgo_factor_batch f = nfg.batch();
    const rpgo_value_batch v = values.batch();
    check(rpgo_force_update(h_, &f, &v), "rpgo_force_update");
  }
  // README.md:114-118: loadGraph / addGraph as update() wrappers
  void loadGraph(const FactorGraph& nfg, const Values& values, const FactorGraph& prior) {
    const rpgo_factor_batch f = nfg.batch(), p = prior.batch();
    const rpgo_value_batch v = values.batch();
    check(rpgo_load_graph(h_, &f, &v, &p), "rpgo_load_graph");
  }
  void addGraph(const FactorGraph& nfg, const Values& values, const FactorGraph& between) {
    const rpgo_factor_batch f = nfg.batch(), b = between.batch();
    const rpgo_value_batch v = values.batch();
    check(rpgo_add_graph(h_, &f, &v, &b), "rpgo_add_graph");
  }

  size_t getNumLC() const { return (size_t)counts().num_lc; }
  size_t getNumLCInliers() const { return (size_t)counts().num_lc_inliers; }
  size_t size() const { return (size_t)counts().num_factors; }

  Values calculateEstimate() const {
    Values v(dim_);
    const int64_t n = counts().num_values;
    v.keys.resize((size_t)n);
    v.poses.resize((size_t)n * poseStride(dim_));
    check(rpgo_get_estimate(h_, v.keys.data(), v.poses.data(), n), "rpgo_get_estimate");
    return v;
  }
  Values calculateBestEstimate() const { return calculateEstimate(); }
  Values getLinearizationPoint() const { return calculateEstimate(); }
  // getFactorsUnsafe(): the graph handed to the optimiser (kinds, keys,
  // measurements; the noise models stay inside the library)
  FactorGraph getFactorsUnsafe() const {
    FactorGraph g(dim_);
    const int64_t n = counts().num_factors;
    g.kind.resize((size_t)n);
    g.key_front.resize((size_t)n);
    g.key_back.resize((size_t)n);
    g.measured.resize((size_t)n * poseStride(dim_));
    check(rpgo_get_factors(h_, g.kind.data(), g.key_front.data(), g.key_back.data(), g.measured.data(), n),
          "rpgo_get_factors");
    return g;
  }
  std::vector<double> getGncWeights() const {
    const int64_t n = counts().num_gnc_weights;
    std::vector<double> w((size_t)n);
    check(rpgo_get_gnc_weights(h_, w.data(), n), "rpgo_get_gnc_weights");
    return w;
  }
  std::vector<double> getGncTempWeights() const {
    int64_t n = 0;
    check(rpgo_get_gnc_temp_weights(h_, nullptr, 0, &n), "rpgo_get_gnc_temp_weights");
    std::vector<double> w((size_t)n);
    check(rpgo_get_gnc_temp_weights(h_, w.data(), n, &n), "rpgo_get_gnc_temp_weights");
    return w;
  }

  // edit API (RobustSolver.h:73-99)
  EdgePtr removeLastLoopClosure(char prefix_1, char prefix_2) { return removeLast(1, prefix_1, prefix_2); }
  EdgePtr removeLastLoopClosure() { return removeLast(0, 0, 0); }
  void ignorePrefix(char prefix) { check(rpgo_ignore_prefix(h_, prefix), "rpgo_ignore_prefix"); }
  void revivePrefix(char prefix) { check(rpgo_revive_prefix(h_, prefix), "rpgo_revive_prefix"); }
  std::vector<char> getIgnoredPrefixes() const {
    int32_t n = 0;
    check(rpgo_get_ignored_prefixes(h_, nullptr, 0, &n), "rpgo_get_ignored_prefixes");
    std::vector<char> out((size_t)n);
    check(rpgo_get_ignored_prefixes(h_, out.data(), n, &n), "rpgo_get_ignored_prefixes");
    return out;
  }
  void removePriorFactorsWithPrefix(const char& prefix, bool optimize_graph = false) {
    check(rpgo_remove_prior_factors_with_prefix(h_, prefix, optimize_graph ? 1 : 0),
          "rpgo_remove_prior_factors_with_prefix");
  }

  // temporary factors and values (GenericSolver.h:46-65)
  void updateTempFactorsValues(const FactorGraph& temp_nfg, const Values& temp_values) {
    const rpgo_factor_batch f = temp_nfg.batch();
    const rpgo_value_batch v = temp_values.batch();
    check(rpgo_update_temp_factors_values(h_, &f, &v), "rpgo_update_temp_factors_values");
  }
  void replaceTempFactorsValues(const FactorGraph& temp_nfg, const Values& temp_values) {
    const rpgo_factor_batch f = temp_nfg.batch();
    const rpgo_value_batch v = temp_values.batch();
    check(rpgo_replace_temp_factors_values(h_, &f, &v), "rpgo_replace_temp_factors_values");
  }
  void clearTempFactorsValues() { check(rpgo_clear_temp_factors_values(h_), "rpgo_clear_temp_factors_values"); }
  Values getTempValues() const {
    int64_t nf = 0, nv = 0;
    check(rpgo_get_temp_sizes(h_, &nf, &nv), "rpgo_get_temp_sizes");
    Values v(dim_);
    v.keys.resize((size_t)nv);
    v.poses.resize((size_t)nv * poseStride(dim_));
    check(rpgo_get_temp_values(h_, v.keys.data(), v.poses.data(), nv), "rpgo_get_temp_values");
    return v;
  }

  // RobustSolver::saveData (RobustSolver.h:133-138)
  void saveData(std::string folder_path) const { check(rpgo_save_data(h_, folder_path.c_str()), "rpgo_save_data"); }

  const RobustSolverParams& params() const { return params_; }
  rpgo_solver* handle() const { return h_; }

 private:
  rpgo_counts counts() const {
    rpgo_counts c;
    check(rpgo_get_counts(h_, &c), "rpgo_get_counts");
    return c;
  }
  EdgePtr removeLast(int by_id, char a, char b) {
    uint64_t k1 = 0, k2 = 0;
    int32_t removed = 0;
    check(rpgo_remove_last_loop_closure(h_, by_id, a, b, &k1, &k2, &removed), "rpgo_remove_last_loop_closure");
    if (!removed) return nullptr;
    return EdgePtr(new Edge{k1, k2});
  }
  RobustSolverParams params_;
  int dim_;
  rpgo_solver* h_ = nullptr;
};

// g2o file (GTSAM readG2o / load3D / load2D semantics) into a FactorGraph and
// Values; throws rpgo::Error on a read failure
inline std::pair<FactorGraph, Values> readG2o(const std::string& path, int dim) {
  int32_t status = RPGO_OK;
  rpgo_g2o* g = rpgo_g2o_read(path.c_str(), dim, &status);
  if (!g) throw Error(status == RPGO_OK ? RPGO_ERR_ARG : status, "rpgo_g2o_read failed: " + path);
  rpgo_factor_batch f;
  rpgo_value_batch v;
  const int rc = rpgo_g2o_view(g, &f, &v);
  if (rc != RPGO_OK) {
    rpgo_g2o_free(g);
    throw Error(rc, "rpgo_g2o_view failed");
  }
  const int d = dim == 3 ? 6 : 3, st = poseStride(dim);
  FactorGraph fg(dim);
  fg.kind.assign(f.kind, f.kind + f.count);
  fg.key_front.assign(f.key_front, f.key_front + f.count);
  fg.key_back.assign(f.key_back, f.key_back + f.count);
  fg.measured.assign(f.measured, f.measured + f.count * st);
  fg.covariance.assign(f.covariance, f.covariance + f.count * d * d);
  fg.sqrt_information.assign(f.sqrt_information, f.sqrt_information + f.count * d * d);
  Values vals(dim);
  vals.keys.assign(v.key, v.key + v.count);
  vals.poses.assign(v.pose, v.pose + v.count * st);
  rpgo_g2o_free(g);
  return {std::move(fg), std::move(vals)};
}

}  // namespace rpgo

#endif  // RPGO_GB300_HPP

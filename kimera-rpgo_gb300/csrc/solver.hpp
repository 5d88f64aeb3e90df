// Host control of the GPU nonlinear least-squares solve: GTSAM's
// LevenbergMarquardtOptimizer / GaussNewtonOptimizer and GncOptimizer<TLS>
// semantics (as RobustSolver::optimize uses them, src/RobustSolver.cpp:115-306)
// over the device kernels of solver_kernels.cu. Only scalars (costs, the
// linearised cost change, convergence flags) cross to the host per iteration.
#pragma once
#include <cstdint>
#include <vector>

#include "pcm_engine.hpp"
#include "solver_kernels.hpp"

namespace rpgo {

struct LmParams {
  bool gauss_newton = false;
  bool diagonal_damping = true;
  int max_iterations = 100;
  double rel_tol = 1e-5, abs_tol = 1e-5, error_tol = 0.0;
  double lambda_initial = 1e-5, lambda_factor = 10.0, lambda_upper = 1e5, lambda_lower = 0.0;
  double min_model_fidelity = 1e-3;
};

struct GncConfig {
  int threshold_mode = 1;  // 0 cost, 1 probability
  double threshold = 0.9;
  int max_iterations = 100;
  double mu_step = 1.4, rel_cost_tol = 1e-5, weights_tol = 1e-4;
};

struct NlsStats {
  int64_t iterations = 0, linear_solves = 0, cg_iterations = 0, gnc_iterations = 0;
  bool failed = false;
};

class GpuNls {
 public:
  // structure from the host factor list; measurements, square-root
  // informations and initial values gathered on the device from the stores
  // direct: sparse Cholesky steps (else whole-GPU PCG)
  GpuNls(int dim, const std::vector<FactorRec>& graph, const FactorStore& store, const ValueStore& values,
         cudaStream_t st, bool direct = true);
  void set_weights(const std::vector<double>& w);
  // LM / GN from the initial values (from_current: from the estimate in
  // dev().x); result left in dev().x
  void optimize(const LmParams& p, NlsStats* st, bool from_current = false);
  double error_at_result();
  // the same, with the current weights copied to w in the same wait
  double error_at_result(std::vector<double>* w);
  // GenericSolver::updateValues: write the result back into the value rows
  void write_back(ValueStore& values) const;
  SolverDev& dev() { return s_; }
  cudaStream_t stream() const { return st_; }
  const std::vector<uint64_t>& keys() const { return keys_; }

 private:
  int dim_;
  cudaStream_t st_;
  SolverDev s_;
  std::vector<uint64_t> keys_;
  DeviceBuffer<int64_t> value_rows_;  // value-store row of each variable (key order)
};

double chi2inv(double alpha, int dof);

// GncOptimizer<GncParams<LM or GN>> with the TLS loss; known inliers are the
// first n_known factors. init_weights (optional) as in setWeights.
// lm_from_previous (no counterpart in the reference): every LM run after the
// first starts from the previous estimate instead of the initial values.
void gnc_tls(GpuNls& nls, size_t n_known, const GncConfig& g, const LmParams& lp,
             const std::vector<double>* init_weights, std::vector<double>* weights_out, NlsStats* st,
             bool lm_from_previous = false);

// Warm-started GNC-TLS (no counterpart in the reference). probs[k]: predicted
// inlier probability of factor k >= n_known. The predicted inliers
// (probs >= 0.5) form the first weights; LM from the initial values; then TLS
// weight updates starting at mu = warm_mu (mu *= mu_step after each), each
// followed by LM from the previous estimate, until an update reproduces the
// binary weights of the last solve (a fixed point of the TLS rule). Returns
// true (certified) when such a fixed point is reached within max_iterations
// and keeps at least kWarmKeep of the predicted inliers; false tells the
// caller to run the plain schedule.
constexpr double kWarmKeep = 0.75;
bool gnc_tls_warm(GpuNls& nls, size_t n_known, const GncConfig& g, const LmParams& lp,
                  const std::vector<double>& probs, double warm_mu, std::vector<double>* weights_out, NlsStats* st);

}  // namespace rpgo

// Host control of the GPU solve; see solver.hpp.
#include "solver.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <unordered_map>

namespace rpgo {

GpuNls::GpuNls(int dim, const std::vector<FactorRec>& graph, const FactorStore& store, const ValueStore& values,
               cudaStream_t st, bool direct)
    : dim_(dim), st_(st) {
  const int stride = dim == 3 ? 12 : 4, d = dim == 3 ? 6 : 3;
  std::unordered_map<uint64_t, int> index;
  index.reserve(values.size());
  std::vector<int64_t> vrows;
  vrows.reserve(values.size());
  for (const auto& kv : values.rows()) {
    index[kv.first] = (int)keys_.size();
    keys_.push_back(kv.first);
    vrows.push_back(kv.second);
  }
  const size_t F = graph.size();
  std::vector<int32_t> kind(F), vi(F), vj(F);
  std::vector<int64_t> frows(F);
  for (size_t f = 0; f < F; ++f) {
    const FactorRec& r = graph[f];
    kind[f] = r.kind;
    vi[f] = index.at(r.k1);
    vj[f] = r.kind == 0 ? index.at(r.k2) : vi[f];
    frows[f] = r.row;
  }
  solver_upload(s_, dim, kind, vi, vj, (int)keys_.size(), st_, direct);
  DeviceBuffer<int64_t> fr;
  fr.upload(frows, st_);
  value_rows_.upload(vrows, st_);
  gather_rows((int64_t)F, fr.get(), store.meas(), stride, s_.z.get(), st_);
  gather_rows((int64_t)F, fr.get(), store.sqrt_info(), d * d, s_.sqrt_info.get(), st_);
  gather_rows((int64_t)vrows.size(), value_rows_.get(), values.pose(), stride, s_.x0.get(), st_);
  set_weights(std::vector<double>(F, 1.0));
  RPGO_CUDA(cudaStreamSynchronize(st_));
}

void GpuNls::set_weights(const std::vector<double>& w) { s_.weights.upload(w, st_); }

double GpuNls::error_at_result() { return solver_error(s_, s_.x.get(), s_.weights.get(), st_); }

double GpuNls::error_at_result(std::vector<double>* w) {
  w->resize((size_t)s_.F);
  if (s_.F == 0) return 0.0;
  double* h = s_.pin.get(1);
  const double* sum = enqueue_error_sum(s_, s_.x.get(), s_.weights.get(), st_);
  RPGO_CUDA(cudaMemcpyAsync(h, sum, sizeof(double), cudaMemcpyDeviceToHost, st_));
  s_.weights.download(w->data(), (size_t)s_.F, st_);
  RPGO_CUDA(cudaStreamSynchronize(st_));
  return h[0];
}

void GpuNls::write_back(ValueStore& values) const {
  scatter_rows((int64_t)keys_.size(), value_rows_.get(), s_.x.get(), dim_ == 3 ? 12 : 4, values.pose(), st_);
  RPGO_CUDA(cudaStreamSynchronize(st_));
}

// NonlinearOptimizer::defaultOptimize with LevenbergMarquardtOptimizer::iterate
// or GaussNewtonOptimizer::iterate (GTSAM, restated).
void GpuNls::optimize(const LmParams& p, NlsStats* st, bool from_current) {
  SolverDev& s = s_;
  if (!from_current)
    RPGO_CUDA(cudaMemcpyAsync(s.x.get(), s.x0.get(), s.x0.size() * sizeof(double), cudaMemcpyDeviceToDevice, st_));
  double cur_err = solver_error(s, s.x.get(), s.weights.get(), st_);
  if (cur_err <= p.error_tol || p.max_iterations <= 0) return;
  double lambda = p.lambda_initial;
  int iters = 0;
  double new_err = cur_err;
  while (true) {
    const double current_error = new_err;
    solver_linearize(s, p.diagonal_damping, st_);
    if (p.gauss_newton) {
      SolveOut o = solver_solve(s, 0.0, st_);
      st->linear_solves++;
      st->cg_iterations += o.cg_iterations;
      if (!o.ok) {
        st->failed = true;
        return;
      }
      solver_retract(s, st_);
      std::swap(s.x, s.xnew);
      cur_err = solver_error(s, s.x.get(), s.weights.get(), st_);
      ++iters;
    } else {
      while (true) {
        double nerr = 0.0;
        SolveOut o = solver_solve_eval(s, lambda, st_, &nerr);
        st->linear_solves++;
        st->cg_iterations += o.cg_iterations;
        bool success = false, stop_search = false;
        if (o.ok && o.lin_change >= 0.0) {
          const double cost_change = cur_err - nerr;
          if (o.lin_change > std::numeric_limits<double>::epsilon() * cur_err)
            success = (cost_change / o.lin_change) > p.min_model_fidelity;
          else
            success = true;
          if (std::fabs(cost_change) < p.rel_tol * cur_err) stop_search = true;
        }
        if (success) {
          std::swap(s.x, s.xnew);
          cur_err = nerr;
          lambda = std::max(p.lambda_lower, lambda / p.lambda_factor);
          ++iters;
          break;
        } else if (!stop_search) {
          lambda *= p.lambda_factor;
          if (lambda >= p.lambda_upper) break;
        } else {
          break;
        }
      }
    }
    new_err = cur_err;
    const double abs_dec = current_error - new_err;
    const double rel_dec = abs_dec / current_error;
    const bool converged =
        (new_err <= p.error_tol) || (p.rel_tol != 0.0 && rel_dec <= p.rel_tol) || (abs_dec <= p.abs_tol);
    if (iters >= p.max_iterations || converged || !std::isfinite(current_error)) break;
  }
  st->iterations += iters;
}

// chi-square quantile by bisection on the closed-form CDF (integer dof)
static double chi2_cdf(double x, int k) {
  if (x <= 0.0) return 0.0;
  const double h = 0.5 * x;
  if (k % 2 == 0) {
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < k / 2; ++i) {
      term *= h / i;
      sum += term;
    }
    return 1.0 - std::exp(-h) * sum;
  }
  double p = std::erf(std::sqrt(h));
  double term = std::sqrt(x) * std::sqrt(2.0 / 3.141592653589793) * std::exp(-h);
  for (int j = 1; j <= (k - 1) / 2; ++j) {
    p -= term;
    term *= x / (2.0 * j + 1.0);
  }
  return p;
}
double chi2inv(double alpha, int k) {
  double lo = 0.0, hi = 1.0;
  while (chi2_cdf(hi, k) < alpha) hi *= 2.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (chi2_cdf(mid, k) < alpha) lo = mid;
    else hi = mid;
  }
  return 0.5 * (lo + hi);
}

// GncOptimizer::optimize (TLS), restated.
void gnc_tls(GpuNls& nls, size_t n_known, const GncConfig& g, const LmParams& lp,
             const std::vector<double>* init_weights, std::vector<double>* weights_out, NlsStats* st,
             bool lm_from_previous) {
  SolverDev& s = nls.dev();
  cudaStream_t stream = nls.stream();
  const size_t F = (size_t)s.F;
  const int dof = s.d;
  std::vector<double> barc(F, g.threshold_mode == 0 ? g.threshold : 0.5 * chi2inv(g.threshold, dof));
  DeviceBuffer<double> barc_dev;
  barc_dev.upload(barc, stream);
  std::vector<double> weights(F, 1.0);
  if (init_weights) weights = *init_weights;
  nls.set_weights(weights);
  nls.optimize(lp, st);
  // mu from the residuals at the initial values
  std::vector<double> r0;
  solver_factor_errors(s, s.x0.get(), &r0, stream);
  double mu = std::numeric_limits<double>::infinity();
  for (size_t k = 0; k < F; ++k)
    if (2.0 * r0[k] - barc[k] > 0.0) mu = std::min(mu, barc[k] / (2.0 * r0[k] - barc[k]));
  if (mu >= 0.0 && mu < 1e-6) mu = 1e-6;
  if (!(mu > 0.0) || std::isinf(mu)) mu = -1.0;
  double prev_cost = nls.error_at_result();
  const size_t n_unknown = F - n_known;
  if (n_unknown == 0 || mu <= 0.0) {
    *weights_out = weights;
    return;
  }
  for (int it = 0; it < g.max_iterations; ++it) {
    st->gnc_iterations++;
    solver_gnc_weights(s, s.x.get(), (int)n_known, barc_dev.get(), mu, stream);
    nls.optimize(lp, st, lm_from_previous);
    const double cost = nls.error_at_result(&weights);
    bool conv = std::fabs(cost - prev_cost) / std::max(prev_cost, 1e-7) < g.rel_cost_tol;
    if (!conv) {
      conv = true;
      for (size_t k = 0; k < F; ++k)
        if (std::fabs(weights[k] - std::round(weights[k])) > g.weights_tol) {
          conv = false;
          break;
        }
    }
    if (conv) break;
    mu *= g.mu_step;
    prev_cost = cost;
  }
  s.weights.download(weights.data(), F, stream);
  RPGO_CUDA(cudaStreamSynchronize(stream));
  *weights_out = weights;
}

bool gnc_tls_warm(GpuNls& nls, size_t n_known, const GncConfig& g, const LmParams& lp,
                  const std::vector<double>& probs, double warm_mu, std::vector<double>* weights_out, NlsStats* st) {
  SolverDev& s = nls.dev();
  cudaStream_t stream = nls.stream();
  const size_t F = (size_t)s.F;
  std::vector<double> barc(F, g.threshold_mode == 0 ? g.threshold : 0.5 * chi2inv(g.threshold, s.d));
  DeviceBuffer<double> barc_dev;
  barc_dev.upload(barc, stream);
  std::vector<double> weights(F, 1.0), wnew(F, 1.0);
  size_t predicted = 0;
  for (size_t k = n_known; k < F; ++k) {
    weights[k] = (k < probs.size() && probs[k] >= 0.5) ? 1.0 : 0.0;
    predicted += weights[k] == 1.0;
  }
  const std::vector<double> first = weights;
  nls.set_weights(weights);
  nls.optimize(lp, st);
  double mu = warm_mu;
  bool fixed_point = F == n_known;
  for (int it = 0; it < g.max_iterations && !fixed_point; ++it) {
    st->gnc_iterations++;
    solver_gnc_weights(s, s.x.get(), (int)n_known, barc_dev.get(), mu, stream);
    s.weights.download(wnew.data(), F, stream);
    RPGO_CUDA(cudaStreamSynchronize(stream));
    bool same = true;
    for (size_t k = n_known; k < F && same; ++k)
      if (std::fabs(wnew[k] - std::round(wnew[k])) > g.weights_tol || std::round(wnew[k]) != weights[k]) same = false;
    if (same) {
      fixed_point = true;
      nls.set_weights(weights);
      break;
    }
    weights = wnew;
    nls.optimize(lp, st, true);
    mu *= g.mu_step;
  }
  size_t kept = 0;
  for (size_t k = n_known; k < F; ++k) kept += (first[k] == 1.0 && weights[k] == 1.0);
  *weights_out = weights;
  return fixed_point && (double)kept >= kWarmKeep * (double)predicted;
}

}  // namespace rpgo

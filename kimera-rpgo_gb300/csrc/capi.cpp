// extern "C" boundary of the library (include/rpgo_gb300.h).
//
// rpgo_solver mirrors KimeraRPGO::RobustSolver (include/KimeraRPGO/RobustSolver.h,
// src/RobustSolver.cpp) and GenericSolver (src/GenericSolver.cpp): it owns
// the values and the graph to optimise, hands new factors to the PCM plugin
// (pcm_engine.cpp) and runs the GPU GNC / LM / GN solve (solver.cpp). Where
// the reference calls exit() or lets an exception escape, a status code is
// returned instead.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <memory>
#include <mutex>
#include <numeric>
#include <set>
#include <string>
#include <vector>

#include "../../include/rpgo_gb300.h"
#include "pcm_engine.hpp"
#include "solver.hpp"
#include "warm.hpp"
#include "align.hpp"
#include "batch_joint.hpp"

using namespace rpgo;

struct rpgo_solver {
  rpgo_params p;
  int dim = 3, stride = 12, d = 6;
  cudaStream_t st = nullptr;
  std::unique_ptr<ValueStore> values;  // GenericSolver::values_ (device rows)
  std::unique_ptr<FactorStore> store;  // every factor measurement ever added (device rows)
  std::vector<FactorRec> nfg;          // GenericSolver::nfg_ (kinds, keys, store rows)
  std::vector<FactorRec> temp_nfg;     // GenericSolver::temp_nfg_ (measurements in `store`)
  std::unique_ptr<ValueStore> temp_values;  // GenericSolver::temp_values_
  std::vector<double> gnc_temp_weights;     // RobustSolver::gnc_temp_weights_
  std::unique_ptr<PcmEngine> pcm;
  std::vector<double> gnc_weights;
  size_t gnc_num_inliers = 0, latest_num_lc = 0;
  bool last_do_optimize = false;
  rpgo_timing timing{};
  std::vector<double> warm_probs;  // rpgo_set_warm_start_probs, consumed by the next GNC solve
  int coop_ctas = 0;                // CTAs of the cooperative direct solve (0: one per SM)
  DeviceBuffer<float> model;        // closure network parameters (rpgo_set_warm_start_model)
  bool has_model = false;
  std::vector<float> features;      // closure features of the last GNC solve (warm modes)
};

namespace rpgo {
void set_coop_ctas(rpgo_solver* s, int ctas) { s->coop_ctas = ctas; }
}  // namespace rpgo

namespace {

double ms_since(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// Append a batch's measurements to the factor store (host or device arrays)
// and return the factor records.
std::vector<FactorRec> ingest(rpgo_solver* s, const rpgo_factor_batch* f, bool on_device) {
  std::vector<FactorRec> out;
  if (!f || f->count <= 0) return out;
  const int64_t first = s->store->append(f->count, f->measured, f->covariance, f->sqrt_information, on_device, s->st);
  out.resize((size_t)f->count);
  for (int64_t k = 0; k < f->count; ++k) {
    FactorRec& r = out[k];
    r.kind = f->kind[k];
    r.k1 = f->key_front[k];
    r.k2 = (r.kind == RPGO_FACTOR_BETWEEN) ? f->key_back[k] : f->key_front[k];
    r.row = first + k;
  }
  return out;
}

// Features of the closures of the graph to optimise (factors n_known..) at
// the initial values, kept for rpgo_get_closure_features; with an installed
// closure network and no caller-given probabilities, its predictions become
// the warm start's inlier probabilities.
void closure_features_and_probs(rpgo_solver* s, GpuNls& nls, const std::vector<FactorRec>& full, size_t n_known) {
  const size_t F = full.size();
  const int64_t nlc = (int64_t)F - (int64_t)n_known;
  s->features.clear();
  if (nlc <= 0) return;
  std::vector<float> pcm_stats;
  if (s->pcm) s->pcm->closure_stats(&pcm_stats);
  std::vector<float> aux((size_t)nlc * 4, 0.f);
  for (int64_t q = 0; q < nlc; ++q) {
    const FactorRec& f = full[n_known + q];
    const uint64_t kmask = (1ull << 56) - 1;
    if (key_chr(f.k1) == key_chr(f.k2)) {
      const uint64_t a = f.k1 & kmask, b = f.k2 & kmask;
      aux[q * 4] = (float)(a > b ? a - b : b - a);
    }
    if (pcm_stats.size() == (size_t)nlc * 3)
      for (int c = 0; c < 3; ++c) aux[q * 4 + 1 + c] = pcm_stats[q * 3 + c];
  }
  DeviceBuffer<float> daux, dfeat((size_t)nlc * kFeat);
  daux.upload(aux, s->st);
  closure_features(nls.dev(), (int)n_known, daux.get(), dfeat.get(), s->st);
  s->features.resize((size_t)nlc * kFeat);
  dfeat.download(s->features.data(), s->features.size(), s->st);
  if ((s->p.gnc_warm_start == RPGO_WARM_ON || s->p.gnc_warm_start == RPGO_WARM_CONTINUATION) && s->has_model &&
      s->warm_probs.size() != F) {
    DeviceBuffer<float> dprob((size_t)nlc);
    mlp_forward(s->model.get(), nlc, dfeat.get(), dprob.get(), s->st);
    std::vector<float> prob((size_t)nlc);
    dprob.download(prob.data(), prob.size(), s->st);
    RPGO_CUDA(cudaStreamSynchronize(s->st));
    s->warm_probs.assign(F, 1.0);
    for (int64_t q = 0; q < nlc; ++q) s->warm_probs[n_known + q] = prob[q];
  }
  RPGO_CUDA(cudaStreamSynchronize(s->st));
}

// Pcm::multirobotValueInitialization (Pcm.h:1011-1074) with
// gncRobustPoseAveraging (1093-1131): robot r0 (smallest prefix) keeps its
// odometry poses; every other robot's poses are moved by the GNC-TLS (or L2)
// average of the frame offsets its consistent closures with r0 imply, solved
// on the GPU as priors on one pose from the identity with GTSAM's default LM
// parameters. Only the robot's own keys are written (the reference would also
// move other robots' keys that a cross-robot lookup left in a trajectory).
void multirobot_align(rpgo_solver* s) {
  if (!s->pcm || s->p.multirobot_align_method == RPGO_ALIGN_NONE) return;
  const std::vector<char> order = s->pcm->sorted_robot_order();
  if (order.size() < 2) return;
  const int stride = s->stride, d = s->d;
  std::vector<uint64_t> keys;
  std::vector<int32_t> slots;
  auto apply = [&](char r, const double* T_dev) {
    s->pcm->robot_slots(r, &keys, &slots);
    std::vector<int32_t> sl;
    std::vector<int64_t> rows;
    for (size_t k = 0; k < keys.size(); ++k)
      if (s->values->has(keys[k])) {
        sl.push_back(slots[k]);
        rows.push_back(s->values->row(keys[k]));
      }
    if (sl.empty()) return;
    DeviceBuffer<int32_t> dsl;
    DeviceBuffer<int64_t> drows;
    dsl.upload(sl, s->st);
    drows.upload(rows, s->st);
    launch_transform_rows(s->dim, (int)sl.size(), T_dev, dsl.get(), s->pcm->traj_pose(), drows.get(),
                          s->values->pose(), s->st);
    RPGO_CUDA(cudaStreamSynchronize(s->st));
  };
  std::vector<double> ident(stride, 0.0);
  if (s->dim == 3) ident[0] = ident[4] = ident[8] = 1.0;
  else ident[0] = 1.0;
  DeviceBuffer<double> dident;
  dident.upload(ident, s->st);
  const char r0 = order[0];
  apply(r0, dident.get());
  for (size_t i = 1; i < order.size(); ++i) {
    const char ri = order[i];
    std::vector<FactorRec> lcs;
    if (!s->pcm->group_closures(r0, ri, &lcs)) continue;
    std::vector<int32_t> front, back;
    std::vector<uint8_t> swap;
    std::vector<int64_t> rows;
    bool ok = true;
    for (const auto& f : lcs) {
      uint64_t a = f.k1, b = f.k2;
      const bool sw = key_chr(a) != r0;
      if (sw) std::swap(a, b);
      const int32_t sa = s->pcm->find_slot(a), sb = s->pcm->find_slot(b);
      if (sa < 0 || sb < 0 || key_chr(a) != r0 || key_chr(b) != ri) {
        ok = false;
        break;
      }
      front.push_back(sa);
      back.push_back(sb);
      swap.push_back(sw ? 1 : 0);
      rows.push_back(f.row);
    }
    if (!ok) continue;
    const int K = (int)lcs.size();
    if (K == 0) {  // an empty average stays at its initial value, the identity
      apply(ri, dident.get());
      continue;
    }
    std::vector<double> meas((size_t)K * stride);
    if (K > 0) {
      DeviceBuffer<int32_t> dfr, dbk;
      DeviceBuffer<uint8_t> dsw;
      DeviceBuffer<int64_t> drw;
      DeviceBuffer<double> dout((size_t)K * stride);
      dfr.upload(front, s->st);
      dbk.upload(back, s->st);
      dsw.upload(swap, s->st);
      drw.upload(rows, s->st);
      launch_frame_offsets(s->dim, K, dfr.get(), dbk.get(), dsw.get(), drw.get(), s->pcm->traj_pose(),
                           s->store->meas(), dout.get(), s->st);
      dout.download(meas.data(), meas.size(), s->st);
      RPGO_CUDA(cudaStreamSynchronize(s->st));
    }
    // priors on one pose: sigmas 0.1 on the first rotation-dimension entries
    // of the tangent, 0.5 on the rest (Pcm.h:1100-1106)
    const int rdim = s->dim == 3 ? 3 : 1;
    std::vector<double> cov((size_t)K * d * d, 0.0), sq((size_t)K * d * d, 0.0);
    for (int k = 0; k < K; ++k)
      for (int e = 0; e < d; ++e) {
        const double sg = e < rdim ? 0.1 : 0.5;
        cov[(size_t)k * d * d + d * e + e] = sg * sg;
        sq[(size_t)k * d * d + d * e + e] = 1.0 / sg;
      }
    FactorStore fs(stride, d);
    ValueStore vs(stride);
    std::vector<FactorRec> graph((size_t)K);
    if (K > 0) {
      const int64_t first = fs.append(K, meas.data(), cov.data(), sq.data(), false, s->st);
      for (int k = 0; k < K; ++k) graph[k] = FactorRec{RPGO_FACTOR_PRIOR, 0, 0, first + k};
    }
    const uint64_t key0 = 0;
    vs.append(1, &key0, ident.data(), false, s->st);
    GpuNls nls(s->dim, graph, fs, vs, s->st, true);
    nls.dev().coop_ctas = s->coop_ctas;
    GncConfig g;
    if (s->p.multirobot_align_method == RPGO_ALIGN_L2) {
      g.threshold_mode = RPGO_GNC_COST;
      g.threshold = std::numeric_limits<double>::max();
    } else {
      g.threshold_mode = RPGO_GNC_PROBABILITY;
      g.threshold = s->p.multirobot_align_gnc_prob;
    }
    LmParams lp;
    lp.diagonal_damping = false;
    std::vector<double> w;
    NlsStats nst;
    gnc_tls(nls, 0, g, lp, nullptr, &w, &nst);
    apply(ri, nls.dev().x.get());
  }
}

// keys of a value store in row order
std::vector<uint64_t> keys_by_row(const ValueStore& v) {
  std::vector<uint64_t> k(v.size());
  for (const auto& kv : v.rows()) k[(size_t)kv.second] = kv.first;
  return k;
}

// The values the optimiser sees (RobustSolver.cpp:117-120: values_ merged
// with temp_values_): the graph's store itself, or a merged copy whose rows
// are the graph's rows followed by the temporary ones.
struct SolveValues {
  rpgo_solver* s;
  std::unique_ptr<ValueStore> merged;
  explicit SolveValues(rpgo_solver* sv) : s(sv) {
    if (s->temp_values->size() == 0) return;
    merged = std::make_unique<ValueStore>(s->stride);
    const std::vector<uint64_t> k0 = keys_by_row(*s->values), k1 = keys_by_row(*s->temp_values);
    merged->append((int64_t)k0.size(), k0.data(), s->values->pose(), true, s->st);
    merged->append((int64_t)k1.size(), k1.data(), s->temp_values->pose(), true, s->st);
  }
  ValueStore& get() { return merged ? *merged : *s->values; }
  // GenericSolver::updateValues (src/GenericSolver.cpp:37-45): results back
  // into the graph's and the temporary values
  void write_back(GpuNls& nls) {
    nls.write_back(get());
    if (!merged) return;
    const size_t n0 = s->values->size(), n1 = s->temp_values->size(), st = (size_t)s->stride;
    RPGO_CUDA(cudaMemcpyAsync(s->values->pose(), merged->pose(), n0 * st * sizeof(double), cudaMemcpyDeviceToDevice,
                              s->st));
    RPGO_CUDA(cudaMemcpyAsync(s->temp_values->pose(), merged->pose() + n0 * st, n1 * st * sizeof(double),
                              cudaMemcpyDeviceToDevice, s->st));
    RPGO_CUDA(cudaStreamSynchronize(s->st));
  }
};

// RobustSolver::optimize (src/RobustSolver.cpp:115-306)
int optimize(rpgo_solver* s) {
  LmParams lp;
  lp.gauss_newton = s->p.solver == RPGO_SOLVER_GN;
  lp.diagonal_damping = s->p.lm_diagonal_damping != 0;
  std::vector<FactorRec> full = s->nfg;
  full.insert(full.end(), s->temp_nfg.begin(), s->temp_nfg.end());
  SolveValues sv(s);
  NlsStats st;
  const size_t num_lc = s->pcm ? s->pcm->num_lc() : 0;
  if (s->p.use_gnc && s->pcm && !(s->p.gnc_fix_prev_inliers && num_lc == s->latest_num_lc)) {
    GncConfig g;
    g.threshold_mode = s->p.gnc_threshold_mode;
    g.threshold = s->p.gnc_inlier_threshold;
    g.max_iterations = s->p.gnc_max_iterations;
    g.mu_step = s->p.gnc_mu_step;
    g.rel_cost_tol = s->p.gnc_relative_cost_tol;
    g.weights_tol = s->p.gnc_weights_tol;
    const size_t n_known = s->pcm->num_odom() + s->pcm->num_special();
    std::vector<double> init;
    if (s->p.gnc_bias_odom) {
      init.assign(full.size(), 0.0);
      for (size_t i = 0; i < n_known && i < init.size(); ++i) init[i] = 1.0;
    }
    GpuNls nls(s->dim, full, *s->store, sv.get(), s->st, s->p.linear_solver != RPGO_LINEAR_PCG);
    nls.dev().coop_ctas = s->coop_ctas;
    const int wm = s->p.gnc_warm_start;
    if (wm == RPGO_WARM_ON || wm == RPGO_WARM_RECORD || wm == RPGO_WARM_CONTINUATION)
      closure_features_and_probs(s, nls, full, n_known);
    std::vector<double> w;
    bool warm_done = false;
    if (wm == RPGO_WARM_ON && s->warm_probs.size() == full.size()) {
      s->timing.warm_runs++;
      warm_done = gnc_tls_warm(nls, n_known, g, lp, s->warm_probs, s->p.gnc_warm_mu, &w, &st);
      if (!warm_done) s->timing.warm_fallbacks++;
    }
    if (wm == RPGO_WARM_CONTINUATION) {
      // plain continuation; first weights from the prediction, LM from the
      // previous estimate
      std::vector<double> first(full.size(), 1.0);
      if (s->warm_probs.size() == full.size())
        for (size_t k = n_known; k < full.size(); ++k) first[k] = s->warm_probs[k] >= 0.5 ? 1.0 : 0.0;
      s->timing.warm_runs++;
      gnc_tls(nls, n_known, g, lp, &first, &w, &st, true);
      warm_done = true;
    }
    s->warm_probs.clear();
    if (!warm_done) gnc_tls(nls, n_known, g, lp, s->p.gnc_bias_odom ? &init : nullptr, &w, &st);
    sv.write_back(nls);
    s->gnc_weights.assign(w.begin(), w.begin() + std::min(w.size(), s->nfg.size()));
    s->gnc_temp_weights.assign(w.begin() + std::min(w.size(), s->nfg.size()), w.end());
    const double sum = std::accumulate(s->gnc_weights.begin(), s->gnc_weights.end(), 0.0);
    s->gnc_num_inliers = static_cast<size_t>(sum) - n_known;
  } else {
    if (s->p.gnc_fix_prev_inliers && s->pcm) {
      const size_t prev_k = s->gnc_weights.size() - std::min(s->latest_num_lc, s->gnc_weights.size());
      const size_t k = s->pcm->num_odom() + s->pcm->num_special();
      full.assign(s->nfg.begin(), s->nfg.begin() + std::min(k, s->nfg.size()));
      for (size_t i = 0; i < s->latest_num_lc; ++i)
        if (prev_k + i < s->gnc_weights.size() && s->gnc_weights[prev_k + i] > 0.5 && k + i < s->nfg.size())
          full.push_back(s->nfg[k + i]);
      full.insert(full.end(), s->temp_nfg.begin(), s->temp_nfg.end());
    }
    GpuNls nls(s->dim, full, *s->store, sv.get(), s->st, s->p.linear_solver != RPGO_LINEAR_PCG);
    nls.dev().coop_ctas = s->coop_ctas;
    nls.optimize(lp, &st);
    if (st.failed) return RPGO_ERR_SOLVER;
    sv.write_back(nls);
    s->gnc_temp_weights.assign(s->temp_nfg.size(), 1.0);
    const size_t tail = std::min(s->latest_num_lc, s->gnc_weights.size());
    std::vector<double> lcw(s->gnc_weights.end() - tail, s->gnc_weights.end());
    s->gnc_weights.assign(s->nfg.size(), 1.0);
    const size_t t2 = std::min(tail, s->gnc_weights.size());
    for (size_t i = 0; i < t2; ++i) s->gnc_weights[s->gnc_weights.size() - t2 + i] = lcw[lcw.size() - t2 + i];
  }
  s->timing.lm_iterations += st.iterations;
  s->timing.linear_solves += st.linear_solves;
  s->timing.cg_iterations += st.cg_iterations;
  s->timing.gnc_iterations += st.gnc_iterations;
  if (s->pcm) s->latest_num_lc = s->pcm->num_lc();
  return RPGO_OK;
}

}  // namespace

namespace rpgo {

// The problem RobustSolver::optimize would solve now, for the joint batch:
// kJointSolve with *jp filled, kJointNone when the last update asked for no
// optimisation, kJointOwn when this solve needs the solver's own path
// (temporary values, a warm start, the fixed-previous-inliers subset, the
// PCG solver, an empty graph).
int joint_prepare(rpgo_solver* s, JointProblem* jp) {
  if (!s->last_do_optimize) return kJointNone;
  if (s->temp_values->size() != 0 || s->p.linear_solver == RPGO_LINEAR_PCG) return kJointOwn;
  std::vector<FactorRec> full = s->nfg;
  full.insert(full.end(), s->temp_nfg.begin(), s->temp_nfg.end());
  if (full.empty() || s->values->size() == 0) return kJointOwn;
  jp->lm = LmParams{};
  jp->lm.gauss_newton = s->p.solver == RPGO_SOLVER_GN;
  jp->lm.diagonal_damping = s->p.lm_diagonal_damping != 0;
  const size_t num_lc = s->pcm ? s->pcm->num_lc() : 0;
  jp->init_weights.clear();
  if (s->p.use_gnc && s->pcm && !(s->p.gnc_fix_prev_inliers && num_lc == s->latest_num_lc)) {
    if (s->p.gnc_warm_start != RPGO_WARM_OFF) return kJointOwn;
    jp->gnc = true;
    jp->gnc_cfg.threshold_mode = s->p.gnc_threshold_mode;
    jp->gnc_cfg.threshold = s->p.gnc_inlier_threshold;
    jp->gnc_cfg.max_iterations = s->p.gnc_max_iterations;
    jp->gnc_cfg.mu_step = s->p.gnc_mu_step;
    jp->gnc_cfg.rel_cost_tol = s->p.gnc_relative_cost_tol;
    jp->gnc_cfg.weights_tol = s->p.gnc_weights_tol;
    jp->n_known = s->pcm->num_odom() + s->pcm->num_special();
    if (s->p.gnc_bias_odom) {
      jp->init_weights.assign(full.size(), 0.0);
      for (size_t i = 0; i < jp->n_known && i < full.size(); ++i) jp->init_weights[i] = 1.0;
    }
  } else {
    if (s->p.gnc_fix_prev_inliers && s->pcm) return kJointOwn;
    jp->gnc = false;
    jp->n_known = full.size();
  }
  jp->graph = std::move(full);
  jp->store = s->store.get();
  jp->values = s->values.get();
  return kJointSolve;
}

// RobustSolver::optimize's bookkeeping after the joint batch solved *jp
// (the estimate is already in the solver's values)
int joint_commit(rpgo_solver* s, const JointProblem& jp, double solve_ms) {
  const NlsStats& st = jp.stats;
  if (jp.gnc) {
    const std::vector<double>& w = jp.weights;
    s->gnc_weights.assign(w.begin(), w.begin() + std::min(w.size(), s->nfg.size()));
    s->gnc_temp_weights.assign(w.begin() + std::min(w.size(), s->nfg.size()), w.end());
    const double sum = std::accumulate(s->gnc_weights.begin(), s->gnc_weights.end(), 0.0);
    s->gnc_num_inliers = static_cast<size_t>(sum) - jp.n_known;
  } else {
    if (st.failed) return RPGO_ERR_SOLVER;
    s->gnc_temp_weights.assign(s->temp_nfg.size(), 1.0);
    const size_t tail = std::min(s->latest_num_lc, s->gnc_weights.size());
    std::vector<double> lcw(s->gnc_weights.end() - tail, s->gnc_weights.end());
    s->gnc_weights.assign(s->nfg.size(), 1.0);
    const size_t t2 = std::min(tail, s->gnc_weights.size());
    for (size_t i = 0; i < t2; ++i) s->gnc_weights[s->gnc_weights.size() - t2 + i] = lcw[lcw.size() - t2 + i];
  }
  s->timing.solve_ms = solve_ms;
  s->timing.lm_iterations += st.iterations;
  s->timing.linear_solves += st.linear_solves;
  s->timing.gnc_iterations += st.gnc_iterations;
  if (s->pcm) s->latest_num_lc = s->pcm->num_lc();
  return RPGO_OK;
}

// the solver's own optimisation (joint_prepare answered kJointOwn)
int joint_optimize_own(rpgo_solver* s, double* solve_ms) {
  cudaEvent_t e0, e1;
  RPGO_CUDA(cudaEventCreate(&e0));
  RPGO_CUDA(cudaEventCreate(&e1));
  RPGO_CUDA(cudaEventRecord(e0, s->st));
  const int rc = optimize(s);
  RPGO_CUDA(cudaEventRecord(e1, s->st));
  RPGO_CUDA(cudaEventSynchronize(e1));
  *solve_ms = ms_since(e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

}  // namespace rpgo

namespace {

// RobustSolver::update / forceUpdate on prepared factor records; value
// arrays are host or device pointers.
int update_impl(rpgo_solver* s, std::vector<FactorRec> nf, const rpgo_value_batch* vb, bool values_on_device,
                int optimize_graph, bool force) {
  std::set<uint64_t> new_keys;
  if (vb) {
    for (int64_t k = 0; k < vb->count; ++k) {
      if (s->values->has(vb->key[k]) || s->temp_values->has(vb->key[k]) || new_keys.count(vb->key[k]))
        return RPGO_ERR_KEY;
      new_keys.insert(vb->key[k]);
    }
    s->values->append(vb->count, vb->key, vb->pose, values_on_device, s->st);
  }
  s->timing = rpgo_timing{};  // the figures describe the last update
  cudaEvent_t e0, e1, e2;
  RPGO_CUDA(cudaEventCreate(&e0));
  RPGO_CUDA(cudaEventCreate(&e1));
  RPGO_CUDA(cudaEventCreate(&e2));
  const int64_t launches0 = thread_launch_counter();
  const int64_t pairs0 = s->pcm ? s->pcm->stats().pair_checks : 0;
  const KernelTimes kt0 = kernel_times();
  RPGO_CUDA(cudaEventRecord(e0, s->st));
  bool do_opt;
  if (s->pcm) {
    do_opt = s->pcm->remove_outliers(nf, new_keys, *s->values, *s->store, &s->nfg);
    if (!nf.empty()) multirobot_align(s);
  } else {
    // GenericSolver::addAndCheckIfOptimize (src/GenericSolver.cpp:47-65)
    s->nfg.insert(s->nfg.end(), nf.begin(), nf.end());
    do_opt = true;
    if (nf.size() == 1 && nf[0].kind == RPGO_FACTOR_BETWEEN && new_keys.size() == 1) do_opt = false;
    if (nf.empty() && new_keys.empty()) do_opt = false;
  }
  s->last_do_optimize = do_opt;
  RPGO_CUDA(cudaEventRecord(e1, s->st));
  int rc = RPGO_OK;
  for (const auto& f : s->nfg)
    if (!s->values->has(f.k1) || !s->values->has(f.k2)) rc = RPGO_ERR_KEY;
  auto known = [s](uint64_t k) { return s->values->has(k) || s->temp_values->has(k); };
  for (const auto& f : s->temp_nfg)
    if (!known(f.k1) || !known(f.k2)) rc = RPGO_ERR_KEY;
  if (rc == RPGO_OK && ((do_opt && optimize_graph) || force)) rc = optimize(s);
  RPGO_CUDA(cudaEventRecord(e2, s->st));
  RPGO_CUDA(cudaEventSynchronize(e2));
  s->timing.pcm_ms = ms_since(e0, e1);
  s->timing.solve_ms = ms_since(e1, e2);
  s->timing.pair_checks = (s->pcm ? s->pcm->stats().pair_checks : 0) - pairs0;
  s->timing.kernel_launches = thread_launch_counter() - launches0;
  const KernelTimes& kt = kernel_times();
  s->timing.pcg_kernel_ms = kt.pcg_ms - kt0.pcg_ms;
  s->timing.pcg_kernel_launches = kt.pcg_launches - kt0.pcg_launches;
  s->timing.pcg_kernel_bytes = kt.pcg_bytes - kt0.pcg_bytes;
  s->timing.chol_kernel_ms = kt.chol_ms - kt0.chol_ms;
  s->timing.chol_kernel_launches = kt.chol_launches - kt0.chol_launches;
  s->timing.chol_kernel_flops = kt.chol_flops - kt0.chol_flops;
  s->timing.chol_kernel_bytes = kt.chol_bytes - kt0.chol_bytes;
  s->timing.chol_levels = kt.chol_launches > kt0.chol_launches ? kt.chol_levels : 0;
  s->timing.chol_tail = kt.chol_launches > kt0.chol_launches ? kt.chol_tail : 0;
  s->timing.pair_kernel_ms = kt.pair_ms - kt0.pair_ms;
  s->timing.pair_kernel_launches = kt.pair_launches - kt0.pair_launches;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  return rc;
}

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const CudaError& e) {
    std::fprintf(stderr, "rpgo_gb300: %s\n", e.what());
    return RPGO_ERR_CUDA;
  } catch (const std::out_of_range&) {
    return RPGO_ERR_KEY;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "rpgo_gb300: %s\n", e.what());
    return RPGO_ERR_ARG;
  }
}

// The device's default memory pool backs every DeviceBuffer. It keeps up to
// kPoolKeepBytes of freed memory for reuse instead of returning it to the
// driver at each synchronisation.
constexpr uint64_t kPoolKeepBytes = 8ull << 30;

int device_ready() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return 0;
  static std::once_flag once;
  static bool pool_ok = false;
  std::call_once(once, [] {
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = kPoolKeepBytes;
      pool_ok = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess;
    }
  });
  return pool_ok ? 1 : 0;
}

}  // namespace

int save_data_impl_(const rpgo_solver* s, const char* folder) {
  // writeG2o (src/Logger.cpp:64-164) and gnc_weights.csv (src/RobustSolver.cpp:448-465)
  const std::string base(folder);
  std::ofstream g2o(base + "/result.g2o");
  if (!g2o) return RPGO_ERR_ARG;
  auto quat = [](const double* R, double q[4]) {
    const double tr = R[0] + R[4] + R[8];
    if (tr > 0) {
      const double w = std::sqrt(tr + 1.0) * 2;
      q[0] = 0.25 * w; q[1] = (R[7] - R[5]) / w; q[2] = (R[2] - R[6]) / w; q[3] = (R[3] - R[1]) / w;
    } else if (R[0] > R[4] && R[0] > R[8]) {
      const double w = std::sqrt(1.0 + R[0] - R[4] - R[8]) * 2;
      q[0] = (R[7] - R[5]) / w; q[1] = 0.25 * w; q[2] = (R[1] + R[3]) / w; q[3] = (R[2] + R[6]) / w;
    } else if (R[4] > R[8]) {
      const double w = std::sqrt(1.0 + R[4] - R[0] - R[8]) * 2;
      q[0] = (R[2] - R[6]) / w; q[1] = (R[1] + R[3]) / w; q[2] = 0.25 * w; q[3] = (R[5] + R[7]) / w;
    } else {
      const double w = std::sqrt(1.0 + R[8] - R[0] - R[4]) * 2;
      q[0] = (R[3] - R[1]) / w; q[1] = (R[2] + R[6]) / w; q[2] = (R[5] + R[7]) / w; q[3] = 0.25 * w;
    }
  };
  std::vector<uint64_t> vkeys;
  std::vector<double> vposes;
  s->values->download_sorted(&vkeys, &vposes, s->st);
  for (size_t vi = 0; vi < vkeys.size(); ++vi) {
    const double* p = &vposes[vi * s->stride];
    const uint64_t vkey = vkeys[vi];
    if (s->dim == 2) {
      g2o << "VERTEX_SE2 " << vkey << " " << p[2] << " " << p[3] << " " << std::atan2(p[1], p[0]) << "\n";
    } else {
      double q[4];
      quat(p, q);
      g2o << "VERTEX_SE3:QUAT " << vkey << " " << p[9] << " " << p[10] << " " << p[11] << " " << q[1] << " "
          << q[2] << " " << q[3] << " " << q[0] << "\n";
    }
  }
  std::vector<int64_t> rows;
  for (const auto& f : s->nfg) rows.push_back(f.row);
  std::vector<double> allm, allr;
  s->store->download_meas(rows, &allm, s->st);
  s->store->download_sqrt(rows, &allr, s->st);
  for (size_t fi = 0; fi < s->nfg.size(); ++fi) {
    const FactorRec& f = s->nfg[fi];
    if (f.kind != RPGO_FACTOR_BETWEEN) continue;
    const int d = s->d;
    const double* sqrt_info = &allr[fi * d * d];
    double info[36];
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) {
        double acc = 0.0;
        for (int k = 0; k < d; ++k) acc += sqrt_info[d * k + i] * sqrt_info[d * k + j];
        info[d * i + j] = acc;
      }
    const double* m = &allm[fi * s->stride];
    if (s->dim == 2) {
      g2o << "EDGE_SE2 " << f.k1 << " " << f.k2 << " " << m[2] << " " << m[3] << " " << std::atan2(m[1], m[0]);
      for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) g2o << " " << info[3 * i + j];
    } else {
      double q[4];
      quat(m, q);
      g2o << "EDGE_SE3:QUAT " << f.k1 << " " << f.k2 << " " << m[9] << " " << m[10] << " " << m[11] << " " << q[1]
          << " " << q[2] << " " << q[3] << " " << q[0];
      // diagonal blocks swapped to [t; R], off-diagonal blocks copied in place (Logger.cpp:148-152)
      double gi[36];
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
          const bool di = i < 3, dj = j < 3;
          int si = i, sj = j;
          if (di && dj) { si = i + 3; sj = j + 3; }
          else if (!di && !dj) { si = i - 3; sj = j - 3; }
          gi[6 * i + j] = info[6 * si + sj];
        }
      for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) g2o << " " << gi[6 * i + j];
    }
    g2o << "\n";
  }
  if (s->p.use_gnc) {
    std::ofstream w(base + "/gnc_weights.csv");
    w.precision(17);
    for (size_t i = 0; i < s->gnc_weights.size(); ++i) w << s->gnc_weights[i] << (i + 1 < s->gnc_weights.size() ? "\n" : "");
  }
  return RPGO_OK;
}


extern "C" {

void rpgo_params_default(rpgo_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->solver = RPGO_SOLVER_LM;
  p->outlier_removal = RPGO_OUTLIER_PCM3D;
  p->verbosity = RPGO_VERBOSITY_UPDATE;
  p->dim = 3;
  p->odom_threshold = 10.0;
  p->lc_threshold = 5.0;
  p->odom_trans_threshold = 0.05;
  p->odom_rot_threshold = 0.005;
  p->dist_trans_threshold = 0.01;
  p->dist_rot_threshold = 0.001;
  p->incremental = 0;
  p->use_gnc = 0;
  p->gnc_threshold_mode = RPGO_GNC_PROBABILITY;
  p->gnc_inlier_threshold = 0.9;
  p->gnc_max_iterations = 100;
  p->gnc_mu_step = 1.4;
  p->gnc_relative_cost_tol = 1e-5;
  p->gnc_weights_tol = 1e-4;
  p->gnc_fix_prev_inliers = 0;
  p->gnc_bias_odom = 0;
  p->lm_diagonal_damping = 1;
  p->linear_solver = RPGO_LINEAR_CHOLESKY;
  p->gnc_warm_start = RPGO_WARM_OFF;
  p->gnc_warm_mu = 100.0;
  p->multirobot_align_method = RPGO_ALIGN_NONE;
  p->multirobot_align_gnc_prob = 0.99;
}
void rpgo_params_set_multirobot_align(rpgo_params* p, int32_t method, double prob) {
  p->multirobot_align_method = method;
  p->multirobot_align_gnc_prob = prob;
}
void rpgo_params_set_no_rejection(rpgo_params* p, int32_t v) {
  p->outlier_removal = RPGO_OUTLIER_NONE;
  p->verbosity = v;
}
void rpgo_params_set_pcm2d(rpgo_params* p, double o, double l, int32_t v) {
  p->outlier_removal = RPGO_OUTLIER_PCM2D;
  p->dim = 2;
  p->odom_threshold = o;
  p->lc_threshold = l;
  p->verbosity = v;
}
void rpgo_params_set_pcm3d(rpgo_params* p, double o, double l, int32_t v) {
  p->outlier_removal = RPGO_OUTLIER_PCM3D;
  p->dim = 3;
  p->odom_threshold = o;
  p->lc_threshold = l;
  p->verbosity = v;
}
void rpgo_params_set_pcm_simple2d(rpgo_params* p, double to, double ro, double tp, double rp, int32_t v) {
  p->outlier_removal = RPGO_OUTLIER_PCM_SIMPLE2D;
  p->dim = 2;
  p->odom_trans_threshold = to;
  p->odom_rot_threshold = ro;
  p->dist_trans_threshold = tp;
  p->dist_rot_threshold = rp;
  p->verbosity = v;
}
void rpgo_params_set_pcm_simple3d(rpgo_params* p, double to, double ro, double tp, double rp, int32_t v) {
  p->outlier_removal = RPGO_OUTLIER_PCM_SIMPLE3D;
  p->dim = 3;
  p->odom_trans_threshold = to;
  p->odom_rot_threshold = ro;
  p->dist_trans_threshold = tp;
  p->dist_rot_threshold = rp;
  p->verbosity = v;
}
static void set_gnc(rpgo_params* p, int mode, double t, int32_t it, double mu, double rc, double wt, int32_t fix,
                    int32_t bias) {
  p->use_gnc = 1;
  p->gnc_threshold_mode = mode;
  p->gnc_inlier_threshold = t;
  p->gnc_max_iterations = it;
  p->gnc_mu_step = mu;
  p->gnc_relative_cost_tol = rc;
  p->gnc_weights_tol = wt;
  p->gnc_fix_prev_inliers = fix;
  p->gnc_bias_odom = bias;
}
void rpgo_params_set_gnc_probability(rpgo_params* p, double a, int32_t it, double mu, double rc, double wt,
                                     int32_t fix, int32_t bias) {
  set_gnc(p, RPGO_GNC_PROBABILITY, a, it, mu, rc, wt, fix, bias);
}
void rpgo_params_set_gnc_cost(rpgo_params* p, double c, int32_t it, double mu, double rc, double wt, int32_t fix,
                              int32_t bias) {
  set_gnc(p, RPGO_GNC_COST, c, it, mu, rc, wt, fix, bias);
}

rpgo_solver* rpgo_create(const rpgo_params* p) {
  if (!p) return nullptr;
  const int m = p->outlier_removal;
  if (m < RPGO_OUTLIER_NONE || m > RPGO_OUTLIER_PCM_SIMPLE3D) return nullptr;
  if (p->solver != RPGO_SOLVER_LM && p->solver != RPGO_SOLVER_GN) return nullptr;
  if (p->multirobot_align_method < RPGO_ALIGN_NONE || p->multirobot_align_method > RPGO_ALIGN_GNC) return nullptr;
  int dim = (m == RPGO_OUTLIER_PCM2D || m == RPGO_OUTLIER_PCM_SIMPLE2D) ? 2 : (m == RPGO_OUTLIER_NONE ? p->dim : 3);
  if (dim != 2 && dim != 3) return nullptr;
  if (!device_ready()) return nullptr;
  auto s = std::make_unique<rpgo_solver>();
  s->p = *p;
  s->dim = dim;
  s->stride = dim == 3 ? 12 : 4;
  s->d = dim == 3 ? 6 : 3;
  try {
    RPGO_CUDA(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
    AllocStreamScope scope(s->st);
    s->values = std::make_unique<ValueStore>(s->stride);
    s->temp_values = std::make_unique<ValueStore>(s->stride);
    s->store = std::make_unique<FactorStore>(s->stride, s->d);
    if (m != RPGO_OUTLIER_NONE) {
      PcmConfig c;
      c.dim = dim;
      c.mode = (m == RPGO_OUTLIER_PCM_SIMPLE2D || m == RPGO_OUTLIER_PCM_SIMPLE3D) ? 1 : 0;
      c.odom_threshold = p->odom_threshold;
      c.lc_threshold = p->lc_threshold;
      c.odom_trans_threshold = p->odom_trans_threshold;
      c.odom_rot_threshold = p->odom_rot_threshold;
      c.dist_trans_threshold = p->dist_trans_threshold;
      c.dist_rot_threshold = p->dist_rot_threshold;
      c.incremental = p->incremental != 0;
      for (int i = 0; i < p->num_special_symbols && i < RPGO_MAX_SPECIAL_SYMBOLS; ++i)
        c.special.push_back(p->special_symbols[i]);
      s->pcm = std::make_unique<PcmEngine>(c, s->st);
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "rpgo_gb300: %s\n", e.what());
    return nullptr;
  }
  return s.release();
}

void rpgo_destroy(rpgo_solver* s) {
  if (!s) return;
  cudaStream_t st = s->st;
  {
    AllocStreamScope scope(st);
    s->pcm.reset();
    s->values.reset();
    s->store.reset();
    delete s;
  }
  if (st) cudaStreamDestroy(st);
}

int rpgo_update(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v, int32_t optimize_graph) {
  if (!s) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] { return update_impl(s, ingest(s, f, false), v, false, optimize_graph, false); });
}
int rpgo_update_dev(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v, int32_t optimize_graph) {
  if (!s) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] { return update_impl(s, ingest(s, f, true), v, true, optimize_graph, false); });
}
int rpgo_force_update(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v) {
  if (!s) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] { return update_impl(s, ingest(s, f, false), v, false, 1, true); });
}

static int update_with_extra(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v,
                             const rpgo_factor_batch* extra) {
  if (!s) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    auto all = ingest(s, f, false);
    auto more = ingest(s, extra, false);
    all.insert(all.end(), more.begin(), more.end());
    return update_impl(s, std::move(all), v, false, 1, false);
  });
}
int rpgo_load_graph(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v,
                    const rpgo_factor_batch* prior) {
  return update_with_extra(s, f, v, prior);
}
int rpgo_add_graph(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v,
                   const rpgo_factor_batch* between) {
  return update_with_extra(s, f, v, between);
}

int rpgo_get_counts(const rpgo_solver* s, rpgo_counts* c) {
  if (!s || !c) return RPGO_ERR_ARG;
  c->num_factors = (int64_t)s->nfg.size();
  c->num_values = (int64_t)s->values->size();
  c->num_lc = s->pcm ? (int64_t)s->pcm->num_lc() : 0;
  c->num_lc_inliers = s->p.use_gnc ? (int64_t)s->gnc_num_inliers : (s->pcm ? (int64_t)s->pcm->num_lc_inliers() : 0);
  c->num_odom = s->pcm ? (int64_t)s->pcm->num_odom() : 0;
  c->num_special = s->pcm ? (int64_t)s->pcm->num_special() : 0;
  c->num_gnc_weights = (int64_t)s->gnc_weights.size();
  c->last_do_optimize = s->last_do_optimize ? 1 : 0;
  return RPGO_OK;
}
int rpgo_get_estimate(const rpgo_solver* s, uint64_t* keys, double* poses, int64_t cap) {
  if (!s || (int64_t)s->values->size() > cap) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    std::vector<uint64_t> k;
    std::vector<double> p;
    s->values->download_sorted(&k, &p, s->st);
    std::memcpy(keys, k.data(), k.size() * sizeof(uint64_t));
    std::memcpy(poses, p.data(), p.size() * sizeof(double));
    return (int)RPGO_OK;
  });
}
int rpgo_get_gnc_weights(const rpgo_solver* s, double* w, int64_t cap) {
  if (!s || (int64_t)s->gnc_weights.size() > cap) return RPGO_ERR_ARG;
  std::memcpy(w, s->gnc_weights.data(), sizeof(double) * s->gnc_weights.size());
  return RPGO_OK;
}
int rpgo_get_factors(const rpgo_solver* s, int32_t* kind, uint64_t* k1, uint64_t* k2, double* meas, int64_t cap) {
  if (!s || (int64_t)s->nfg.size() > cap) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    for (size_t i = 0; i < s->nfg.size(); ++i) {
      if (kind) kind[i] = s->nfg[i].kind;
      if (k1) k1[i] = s->nfg[i].k1;
      if (k2) k2[i] = s->nfg[i].k2;
    }
    if (meas) {
      std::vector<int64_t> rows;
      for (const auto& f : s->nfg) rows.push_back(f.row);
      std::vector<double> m;
      s->store->download_meas(rows, &m, s->st);
      std::memcpy(meas, m.data(), m.size() * sizeof(double));
    }
    return (int)RPGO_OK;
  });
}
int rpgo_get_adjacency(const rpgo_solver* s, int32_t group, uint32_t* words, int64_t cap, int64_t* n) {
  if (!s || !n) return RPGO_ERR_ARG;
  if (!s->pcm) return RPGO_ERR_UNSUPPORTED;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    std::vector<uint32_t> w;
    int nn = 0;
    if (!s->pcm->adjacency(group, &w, &nn)) return (int)RPGO_ERR_ARG;
    *n = nn;
    if (!words) return (int)RPGO_OK;
    if ((int64_t)w.size() > cap) return (int)RPGO_ERR_ARG;
    std::memcpy(words, w.data(), w.size() * sizeof(uint32_t));
    return (int)RPGO_OK;
  });
}
int rpgo_set_warm_start_probs(rpgo_solver* s, const double* probs, int64_t n) {
  if (!s || n < 0 || (n > 0 && !probs)) return RPGO_ERR_ARG;
  s->warm_probs.assign(probs, probs + n);
  return RPGO_OK;
}
// ---- edit API (src/RobustSolver.cpp:371-446)
static int edit_optimize(rpgo_solver* s) {
  for (const auto& f : s->nfg)
    if (!s->values->has(f.k1) || !s->values->has(f.k2)) return RPGO_ERR_KEY;
  return optimize(s);
}

int rpgo_remove_last_loop_closure(rpgo_solver* s, int32_t by_id, char prefix_1, char prefix_2, uint64_t* key_front,
                                  uint64_t* key_back, int32_t* removed) {
  if (!s || !removed) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    uint64_t a = 0, b = 0;
    bool ok;
    if (s->pcm) {
      ok = by_id ? s->pcm->remove_last_loop_closure(prefix_1, prefix_2, &a, &b, &s->nfg)
                 : s->pcm->remove_last_loop_closure(&a, &b, &s->nfg);
    } else {
      // GenericSolver::removeLastFactor (src/GenericSolver.cpp:122-128);
      // an empty graph removes nothing (the reference indexes it)
      ok = !s->nfg.empty();
      if (ok) {
        a = s->nfg.back().k1;
        b = s->nfg.back().k2;
        s->nfg.pop_back();
      }
    }
    *removed = ok ? 1 : 0;
    if (key_front) *key_front = a;
    if (key_back) *key_back = b;
    return edit_optimize(s);
  });
}

int rpgo_ignore_prefix(rpgo_solver* s, char prefix) {
  if (!s) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    if (s->pcm) s->pcm->ignore_prefix(prefix, &s->nfg);
    else if (s->p.verbosity != RPGO_VERBOSITY_QUIET)
      std::fprintf(stderr, "rpgo_gb300: 'ignorePrefix' currently not implemented for no outlier rejection case\n");
    return edit_optimize(s);
  });
}

int rpgo_revive_prefix(rpgo_solver* s, char prefix) {
  if (!s) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    if (s->pcm) s->pcm->revive_prefix(prefix, &s->nfg);
    else if (s->p.verbosity != RPGO_VERBOSITY_QUIET)
      std::fprintf(stderr, "rpgo_gb300: 'revivePrefix' currently not implemented for no outlier rejection case\n");
    return edit_optimize(s);
  });
}

int rpgo_get_ignored_prefixes(const rpgo_solver* s, char* out, int32_t cap, int32_t* n) {
  if (!s || !n) return RPGO_ERR_ARG;
  static const std::vector<char> none;
  const std::vector<char>& v = s->pcm ? s->pcm->ignored_prefixes() : none;
  *n = (int32_t)v.size();
  if (!out) return RPGO_OK;
  if ((int32_t)v.size() > cap) return RPGO_ERR_ARG;
  for (size_t i = 0; i < v.size(); ++i) out[i] = v[i];
  return RPGO_OK;
}

int rpgo_remove_prior_factors_with_prefix(rpgo_solver* s, char prefix, int32_t optimize_graph) {
  if (!s) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    if (s->pcm) {
      s->pcm->remove_priors_with_prefix(prefix, &s->nfg);
    } else {
      // GenericSolver::removePriorsWithPrefix (src/GenericSolver.cpp:130-160)
      std::vector<FactorRec> kept;
      for (const auto& f : s->nfg)
        if (f.kind != RPGO_FACTOR_PRIOR || key_chr(f.k1) != prefix) kept.push_back(f);
      s->nfg.swap(kept);
    }
    return optimize_graph ? edit_optimize(s) : (int)RPGO_OK;
  });
}

int rpgo_set_warm_start_model(rpgo_solver* s, const float* params) {
  if (!s) return RPGO_ERR_ARG;
  if (!params) {
    s->has_model = false;
    return RPGO_OK;
  }
  AllocStreamScope scope(s->st);
  return guarded([&] {
    s->model.upload(params, kMlpParams, s->st);
    RPGO_CUDA(cudaStreamSynchronize(s->st));
    s->has_model = true;
    return (int)RPGO_OK;
  });
}
int rpgo_get_closure_features(const rpgo_solver* s, float* out, int64_t cap, int64_t* n) {
  if (!s || !n) return RPGO_ERR_ARG;
  *n = (int64_t)(s->features.size() / kFeat);
  if (!out) return RPGO_OK;
  if ((int64_t)s->features.size() > cap * kFeat) return RPGO_ERR_ARG;
  std::memcpy(out, s->features.data(), sizeof(float) * s->features.size());
  return RPGO_OK;
}
int rpgo_mlp_forward_dev(const float* params, int64_t n, const float* features, float* prob, void* stream) {
  if (n < 0 || (n > 0 && (!params || !features || !prob))) return RPGO_ERR_ARG;
  AllocStreamScope scope((cudaStream_t)stream);
  return guarded([&] {
    mlp_forward(params, n, features, prob, (cudaStream_t)stream);
    RPGO_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return (int)RPGO_OK;
  });
}
int rpgo_mlp_train_step_dev(float* params, float* adam_m, float* adam_v, int64_t step, float lr, int64_t n,
                            const float* features, const float* labels, float* grad, double* loss, void* stream) {
  if (n < 0 || !params || !grad || (lr > 0.f && (!adam_m || !adam_v || step < 1)) ||
      (n > 0 && (!features || !labels)))
    return RPGO_ERR_ARG;
  AllocStreamScope scope((cudaStream_t)stream);
  return guarded([&] {
    const double l = mlp_train_step(params, adam_m, adam_v, step, lr, n, features, labels, grad, (cudaStream_t)stream);
    if (loss) *loss = l;
    return (int)RPGO_OK;
  });
}
int rpgo_get_timing(const rpgo_solver* s, rpgo_timing* t) {
  if (!s || !t) return RPGO_ERR_ARG;
  *t = s->timing;
  return RPGO_OK;
}

// GenericSolver::updateTempFactorsValues / replaceTempFactorsValues
// (include/KimeraRPGO/GenericSolver.h:50-61)
static int set_temp(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v, bool replace) {
  if (!s) return RPGO_ERR_ARG;
  if (f && f->count > 0 && (!f->kind || !f->key_front || !f->measured || !f->covariance || !f->sqrt_information))
    return RPGO_ERR_ARG;
  if (v && v->count > 0 && (!v->key || !v->pose)) return RPGO_ERR_ARG;
  if (f)
    for (int64_t k = 0; k < f->count; ++k) {
      if (f->kind[k] != RPGO_FACTOR_BETWEEN && f->kind[k] != RPGO_FACTOR_PRIOR) return RPGO_ERR_ARG;
      if (f->kind[k] == RPGO_FACTOR_BETWEEN && !f->key_back) return RPGO_ERR_ARG;
    }
  AllocStreamScope scope(s->st);
  return guarded([&] {
    std::set<uint64_t> keys;
    if (v)
      for (int64_t k = 0; k < v->count; ++k) {
        const uint64_t key = v->key[k];
        if (s->values->has(key) || (!replace && s->temp_values->has(key)) || !keys.insert(key).second)
          return (int)RPGO_ERR_KEY;
      }
    if (replace) {
      s->temp_nfg.clear();
      s->temp_values = std::make_unique<ValueStore>(s->stride);
    }
    std::vector<FactorRec> nf = ingest(s, f, false);
    s->temp_nfg.insert(s->temp_nfg.end(), nf.begin(), nf.end());
    if (v && v->count > 0) s->temp_values->append(v->count, v->key, v->pose, false, s->st);
    RPGO_CUDA(cudaStreamSynchronize(s->st));
    return (int)RPGO_OK;
  });
}

int rpgo_update_temp_factors_values(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v) {
  return set_temp(s, f, v, false);
}

int rpgo_replace_temp_factors_values(rpgo_solver* s, const rpgo_factor_batch* f, const rpgo_value_batch* v) {
  return set_temp(s, f, v, true);
}

// GenericSolver::clearTempFactorsValues (GenericSolver.h:62-65)
int rpgo_clear_temp_factors_values(rpgo_solver* s) {
  if (!s) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    s->temp_nfg.clear();
    s->temp_values = std::make_unique<ValueStore>(s->stride);
    return (int)RPGO_OK;
  });
}

int rpgo_get_temp_sizes(const rpgo_solver* s, int64_t* nf, int64_t* nv) {
  if (!s) return RPGO_ERR_ARG;
  if (nf) *nf = (int64_t)s->temp_nfg.size();
  if (nv) *nv = (int64_t)s->temp_values->size();
  return RPGO_OK;
}

// GenericSolver::getTempValues (GenericSolver.h:46)
int rpgo_get_temp_values(const rpgo_solver* s, uint64_t* keys, double* poses, int64_t cap) {
  if (!s || (int64_t)s->temp_values->size() > cap) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] {
    std::vector<uint64_t> k;
    std::vector<double> p;
    s->temp_values->download_sorted(&k, &p, s->st);
    if (!k.empty()) {
      std::memcpy(keys, k.data(), k.size() * sizeof(uint64_t));
      std::memcpy(poses, p.data(), p.size() * sizeof(double));
    }
    return (int)RPGO_OK;
  });
}

// RobustSolver::getGncTempWeights (include/KimeraRPGO/RobustSolver.h:108)
int rpgo_get_gnc_temp_weights(const rpgo_solver* s, double* w, int64_t cap, int64_t* n) {
  if (!s) return RPGO_ERR_ARG;
  if (n) *n = (int64_t)s->gnc_temp_weights.size();
  if ((int64_t)s->gnc_temp_weights.size() > cap) return RPGO_ERR_ARG;
  if (!s->gnc_temp_weights.empty()) std::memcpy(w, s->gnc_temp_weights.data(), sizeof(double) * s->gnc_temp_weights.size());
  return RPGO_OK;
}

int rpgo_save_data(const rpgo_solver* s, const char* folder) {
  if (!s || !folder) return RPGO_ERR_ARG;
  AllocStreamScope scope(s->st);
  return guarded([&] { return save_data_impl_(s, folder); });
}
// ------------------------------------------------------------------ stage entry points (device pointers)
int rpgo_trajectory_scan_dev(int32_t dim, int32_t mode, int64_t count, const int32_t* src, const int32_t* dst,
                             const double* delta_pose, const double* delta_cov, double* traj_pose, double* traj_cov,
                             int32_t* traj_node, uint8_t* traj_rot_info, void* stream) {
  if ((dim != 2 && dim != 3) || (mode != 0 && mode != 1) || count < 0) return RPGO_ERR_ARG;
  AllocStreamScope scope((cudaStream_t)stream);
  return guarded([&] {
    DeviceBuffer<double> rec, cov;
    DeviceBuffer<uint8_t> rot;
    TrajView tv{traj_pose, traj_cov, traj_node, traj_rot_info};
    launch_traj_scan(dim, mode, count, src, dst, delta_pose, delta_cov, tv, rec, cov, rot, (cudaStream_t)stream);
    RPGO_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return (int)RPGO_OK;
  });
}
int rpgo_odometry_check_dev(int32_t dim, int32_t mode, int64_t count, const int32_t* si, const int32_t* sj,
                            const double* zp, const double* zc, const double* tp, const double* tc, const int32_t* tn,
                            const uint8_t* tr, double th0, double th1, uint8_t* ok, void* stream) {
  if ((dim != 2 && dim != 3) || (mode != 0 && mode != 1) || count < 0) return RPGO_ERR_ARG;
  AllocStreamScope scope((cudaStream_t)stream);
  return guarded([&] {
    TrajView tv{const_cast<double*>(tp), const_cast<double*>(tc), const_cast<int32_t*>(tn),
                const_cast<uint8_t*>(tr)};
    launch_odom_check(dim, mode, count, si, sj, zp, zc, tv, th0, th1, ok, (cudaStream_t)stream);
    RPGO_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return (int)RPGO_OK;
  });
}
int rpgo_pairwise_adjacency_dev(int32_t dim, int32_t mode, int32_t n, int32_t row_begin, const int32_t* sa,
                                const int32_t* sb, const uint8_t* flip, const double* zp, const double* zc,
                                const double* tp, const double* tc, const int32_t* tn, const uint8_t* tr, double th0,
                                double th1, uint32_t* adj, int32_t words, void* stream) {
  if ((dim != 2 && dim != 3) || (mode != 0 && mode != 1) || n < 0 || row_begin < 0 || row_begin > n ||
      words < (n + 31) / 32)
    return RPGO_ERR_ARG;
  AllocStreamScope scope((cudaStream_t)stream);
  return guarded([&] {
    TrajView tv{const_cast<double*>(tp), const_cast<double*>(tc), const_cast<int32_t*>(tn),
                const_cast<uint8_t*>(tr)};
    DeviceBuffer<uint32_t> lower((size_t)(n - row_begin) * words + 1);
    launch_pairwise(dim, mode, n, row_begin, sa, sb, flip, zp, zc, tv, th0, th1, adj, words, lower.get(),
                    (cudaStream_t)stream);
    RPGO_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return (int)RPGO_OK;
  });
}
int rpgo_max_clique_heu_dev(int32_t n, const uint32_t* adj, int32_t words, int32_t first, int32_t seed,
                            int32_t* clique_out, int32_t* size_out, void* stream) {
  if (n < 0 || words < (n + 31) / 32 || !size_out) return RPGO_ERR_ARG;
  AllocStreamScope scope((cudaStream_t)stream);
  return guarded([&] {
    CliqueWorkspace ws;
    std::vector<int32_t> cl;
    const int sz = max_clique_heu(n, adj, words, first, seed, &cl, ws, (cudaStream_t)stream);
    *size_out = sz;
    if (clique_out)
      for (size_t i = 0; i < cl.size(); ++i) clique_out[i] = cl[i];
    return (int)RPGO_OK;
  });
}

// ------------------------------------------------------------------ stage entry points (host arrays)
int rpgo_pairwise_adjacency(int32_t dim, int32_t mode, int32_t n, const int32_t* sa, const int32_t* sb,
                            const uint8_t* flip, const double* zp, const double* zc, int32_t num_slots,
                            const double* tp, const double* tc, const int32_t* tn, const uint8_t* tr, double th0,
                            double th1, uint32_t* adj) {
  if ((dim != 2 && dim != 3) || (mode != 0 && mode != 1) || n < 0 || num_slots < 0) return RPGO_ERR_ARG;
  if (!device_ready()) return RPGO_ERR_CUDA;
  AllocStreamScope scope(nullptr);
  return guarded([&] {
    const int stride = dim == 3 ? 12 : 4, d = dim == 3 ? 6 : 3;
    const int words = (n + 31) / 32;
    cudaStream_t st = 0;
    DeviceBuffer<int32_t> dsa, dsb, dtn;
    DeviceBuffer<uint8_t> dfl, dtr;
    DeviceBuffer<double> dzp, dzc, dtp, dtc;
    DeviceBuffer<uint32_t> dadj((size_t)n * words + 1), lower((size_t)n * words + 1);
    dsa.upload(sa, n, st);
    dsb.upload(sb, n, st);
    dfl.upload(flip, n, st);
    dzp.upload(zp, (size_t)n * stride, st);
    dzc.upload(zc, (size_t)n * d * d, st);
    dtp.upload(tp, (size_t)num_slots * stride, st);
    if (mode == 0) dtc.upload(tc, (size_t)num_slots * d * d, st);
    else dtn.upload(tn, num_slots, st);
    dtr.upload(tr, num_slots, st);
    dadj.zero(st);
    TrajView tv{dtp.get(), dtc.get(), dtn.get(), dtr.get()};
    launch_pairwise(dim, mode, n, 0, dsa.get(), dsb.get(), dfl.get(), dzp.get(), dzc.get(), tv, th0, th1,
                    dadj.get(), words, lower.get(), st);
    dadj.download(adj, (size_t)n * words, st);
    RPGO_CUDA(cudaStreamSynchronize(st));
    return (int)RPGO_OK;
  });
}
int rpgo_max_clique_heu(int32_t n, const uint32_t* adj, int32_t first, int32_t seed, int32_t* clique_out,
                        int32_t* size_out) {
  if (n < 0 || !size_out) return RPGO_ERR_ARG;
  if (!device_ready()) return RPGO_ERR_CUDA;
  AllocStreamScope scope(nullptr);
  return guarded([&] {
    const int words = (n + 31) / 32;
    cudaStream_t st = 0;
    DeviceBuffer<uint32_t> dadj;
    dadj.upload(adj, (size_t)n * words, st);
    CliqueWorkspace ws;
    std::vector<int32_t> cl;
    const int sz = max_clique_heu(n, dadj.get(), words, first, seed, &cl, ws, st);
    *size_out = sz;
    if (clique_out)
      for (size_t i = 0; i < cl.size(); ++i) clique_out[i] = cl[i];
    return (int)RPGO_OK;
  });
}

int rpgo_device_info(char* name, int32_t cap, int32_t* sm_count) {
  if (!device_ready()) return RPGO_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess) return RPGO_ERR_CUDA;
  if (name && cap > 0) {
    std::strncpy(name, prop.name, (size_t)cap - 1);
    name[cap - 1] = 0;
  }
  if (sm_count) *sm_count = prop.multiProcessorCount;
  return RPGO_OK;
}

int64_t rpgo_kernel_launch_count(void) { return launch_counter().load(); }
double rpgo_set_direct_solve_guard(double flops, int32_t prefer) {
  return set_direct_solve_guard(flops, prefer < 0 || prefer > 2 ? 0 : prefer);
}
int64_t rpgo_buffer_alloc_count(void) { return alloc_counter().load(); }

}  // extern "C"

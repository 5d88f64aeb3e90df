// CPU FP64 oracle — TEST INFRASTRUCTURE ONLY (ctypes entry points).
//
// RobustSolver restatement: src/RobustSolver.cpp:29-103 (constructor),
// 105-113 (known inliers), 115-306 (optimize), 337-369 (update);
// src/GenericSolver.cpp:37-65 (updateValues, addAndCheckIfOptimize).
// The structs of the public C ABI header are reused for the argument layout.
#include <omp.h>
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <memory>
#include <numeric>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../include/rpgo_gb300.h"
#include "oracle_solver.hpp"

using namespace oracle;

namespace {

struct SolverBase {
  virtual ~SolverBase() = default;
  virtual int update(const rpgo_factor_batch* f, const rpgo_value_batch* v, int opt) = 0;
  virtual void counts(rpgo_counts* c) const = 0;
  virtual int estimate(uint64_t* keys, double* poses, int64_t cap) const = 0;
  virtual int weights(double* w, int64_t cap) const = 0;
  virtual int factors(int32_t* kind, uint64_t* k1, uint64_t* k2, double* meas, int64_t cap) const = 0;
  virtual int adjacency(int32_t group, uint32_t* words, int64_t cap, int64_t* n) const = 0;
  virtual void stats(int64_t* lm_iters, int64_t* solves, int64_t* gnc_iters) const = 0;
  virtual void set_warm_probs(const double* p, int64_t n) = 0;
  virtual int force_optimize() = 0;
  // edit API (src/RobustSolver.cpp:371-446)
  virtual int remove_last_loop_closure(int by_id, char p1, char p2, uint64_t* k1, uint64_t* k2, int* removed) = 0;
  virtual int ignore_prefix(char c, bool revive) = 0;
  virtual int ignored_prefixes(char* out, int cap) const = 0;
  virtual int remove_priors_with_prefix(char c, int optimize_graph) = 0;
  // temporary factors and values (GenericSolver.h:46-65)
  virtual int set_temp(const rpgo_factor_batch* f, const rpgo_value_batch* v, bool replace) = 0;
  virtual void clear_temp() = 0;
  virtual void temp_sizes(int64_t* nf, int64_t* nv) const = 0;
  virtual int temp_values_out(uint64_t* keys, double* poses, int64_t cap) const = 0;
  virtual int temp_weights(double* w, int64_t cap, int64_t* n) const = 0;
  // checks at large sizes (no reference counterpart): sampled rows of the
  // first group's consistency matrix, and the solve stage alone on a given
  // factor list with its first n_known factors as GNC known inliers
  virtual int pcm_rows(const rpgo_factor_batch* f, const rpgo_value_batch* v, const int32_t* rows, int n_rows,
                       uint32_t* out, int64_t cap, int64_t* n, int64_t* src, int64_t src_cap, bool lower_only) = 0;
  virtual int solve_graph(const rpgo_factor_batch* f, const rpgo_value_batch* v, int64_t n_known) = 0;
  int64_t warm_runs = 0, warm_fallbacks = 0;
  // wall-clock seconds spent in outlier rejection and in the solve (sums)
  double pcm_seconds = 0.0, solve_seconds = 0.0;
};

template <class S, class U>
struct RobustSolverO final : SolverBase {
  using L = typename S::L;
  using Pose = typename S::Pose;
  static constexpr int d = S::d;
  rpgo_params p;
  std::map<uint64_t, Pose> values;
  std::vector<Factor<L>> nfg;
  std::unique_ptr<Pcm<L, U>> pcm;
  std::vector<double> gnc_weights;
  std::map<uint64_t, Pose> temp_values;  // GenericSolver::temp_values_
  std::vector<Factor<L>> temp_nfg;       // GenericSolver::temp_nfg_
  std::vector<double> gnc_temp_weights;  // RobustSolver::gnc_temp_weights_
  size_t gnc_num_inliers = 0, latest_num_lc = 0;
  int64_t lm_iters = 0, solves = 0, gnc_iters = 0;
  bool last_do_opt = false;
  std::vector<double> warm_probs;  // consumed by the next warm-started GNC solve

  explicit RobustSolverO(const rpgo_params& prm, bool with_pcm) : p(prm) {
    if (with_pcm) {
      PcmParamsO pp;
      pp.odom_threshold = p.odom_threshold;
      pp.lc_threshold = p.lc_threshold;
      pp.odom_trans_threshold = p.odom_trans_threshold;
      pp.odom_rot_threshold = p.odom_rot_threshold;
      pp.dist_trans_threshold = p.dist_trans_threshold;
      pp.dist_rot_threshold = p.dist_rot_threshold;
      pp.incremental = p.incremental != 0;
      for (int i = 0; i < p.num_special_symbols && i < RPGO_MAX_SPECIAL_SYMBOLS; ++i)
        pp.special.push_back(p.special_symbols[i]);
      pcm.reset(new Pcm<L, U>(pp));
    }
  }
  std::vector<Factor<L>> convert(const rpgo_factor_batch* f) const {
    std::vector<Factor<L>> out;
    if (!f) return out;
    for (int64_t k = 0; k < f->count; ++k) {
      Factor<L> x;
      x.kind = f->kind[k];
      x.k1 = f->key_front[k];
      x.k2 = (x.kind == 0) ? f->key_back[k] : f->key_front[k];
      x.measured = L::load(f->measured + k * L::stride);
      std::memcpy(x.cov, f->covariance + k * d * d, sizeof(double) * d * d);
      std::memcpy(x.sqrt_info, f->sqrt_information + k * d * d, sizeof(double) * d * d);
      x.src = k;
      out.push_back(x);
    }
    return out;
  }
  int update(const rpgo_factor_batch* fb, const rpgo_value_batch* vb, int optimize_graph) override {
    try {
      return update_impl(fb, vb, optimize_graph);
    } catch (const std::out_of_range&) {
      return RPGO_ERR_KEY;
    }
  }
  int update_impl(const rpgo_factor_batch* fb, const rpgo_value_batch* vb, int optimize_graph) {
    auto nf = convert(fb);
    std::set<uint64_t> new_keys;
    if (vb) {
      for (int64_t k = 0; k < vb->count; ++k) {
        if (values.count(vb->key[k]) || temp_values.count(vb->key[k]) || new_keys.count(vb->key[k]))
          return RPGO_ERR_KEY;
        new_keys.insert(vb->key[k]);
      }
      for (int64_t k = 0; k < vb->count; ++k) values[vb->key[k]] = L::load(vb->pose + k * L::stride);
    }
    bool do_opt;
    if (pcm) {
      const auto t0 = std::chrono::steady_clock::now();
      do_opt = pcm->remove_outliers(nf, new_keys, values, &nfg);
      if (!nf.empty()) multirobot_align();
      this->pcm_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    } else {
      nfg.insert(nfg.end(), nf.begin(), nf.end());
      do_opt = true;
      if (nf.size() == 1 && nf[0].kind == 0 && new_keys.size() == 1) do_opt = false;
      if (nf.empty() && new_keys.empty()) do_opt = false;
    }
    last_do_opt = do_opt;
    for (const auto& f : nfg) {
      if (!values.count(f.k1) || !values.count(f.k2)) return RPGO_ERR_KEY;
    }
    auto known = [this](uint64_t k) { return values.count(k) || temp_values.count(k); };
    for (const auto& f : temp_nfg)
      if (!known(f.k1) || !known(f.k2)) return RPGO_ERR_KEY;
    if (do_opt && optimize_graph) {
      const auto t0 = std::chrono::steady_clock::now();
      const int rc = optimize();
      this->solve_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      return rc;
    }
    return RPGO_OK;
  }
  // Pcm.h:1093-1131: GNC (TLS at probability p, or L2) average of poses
  // measured as priors on one pose, from the identity; GTSAM's default
  // LevenbergMarquardtParams (no diagonal damping)
  Pose pose_average(const std::vector<Pose>& meas) const {
    std::vector<Factor<L>> graph;
    for (const Pose& m : meas) {
      Factor<L> f;
      f.kind = 1;
      f.k1 = f.k2 = 0;
      f.measured = m;
      for (int i = 0; i < d * d; ++i) f.cov[i] = f.sqrt_info[i] = 0.0;
      for (int i = 0; i < d; ++i) {
        const double sg = i < L::rdim ? 0.1 : 0.5;
        f.cov[d * i + i] = sg * sg;
        f.sqrt_info[d * i + i] = 1.0 / sg;
      }
      graph.push_back(f);
    }
    std::map<uint64_t, Pose> init{{0, L::identity()}};
    GncParamsO gp;
    if (p.multirobot_align_method == RPGO_ALIGN_L2) {
      gp.threshold_mode = 0;
      gp.threshold = std::numeric_limits<double>::max();
    } else {
      gp.threshold_mode = 1;
      gp.threshold = p.multirobot_align_gnc_prob;
    }
    LmParamsO lp;
    lp.diagonal_damping = false;
    return gnc_tls<S>(graph, init, 0, gp, lp).values.at(0);
  }
  // Pcm.h:1011-1074 (robot keys only: the reference would also move other
  // robots' keys that a cross-robot lookup left in a trajectory)
  void multirobot_align() {
    if (p.multirobot_align_method == RPGO_ALIGN_NONE || pcm->robot_order.size() < 2) return;
    std::sort(pcm->robot_order.begin(), pcm->robot_order.end());
    const char r0 = pcm->robot_order[0];
    auto apply = [&](char r, const Pose& T) {
      for (const auto& kv : pcm->trajectories[r].poses)
        if (key_chr(kv.first) == r && values.count(kv.first)) values[kv.first] = L::compose(T, kv.second.pose);
    };
    apply(r0, L::identity());
    for (size_t i = 1; i < pcm->robot_order.size(); ++i) {
      const char ri = pcm->robot_order[i];
      auto it = pcm->loop_closures.find(ObsId{r0, ri});
      if (it == pcm->loop_closures.end()) continue;
      std::vector<Pose> meas;
      bool ok = true;
      auto& t0 = pcm->trajectories[r0].poses;
      auto& ti = pcm->trajectories[ri].poses;
      for (const auto& f : it->second.consistent) {
        uint64_t front = f.k1, back = f.k2;
        Pose z = f.measured;
        if (key_chr(front) != r0) {
          std::swap(front, back);
          z = L::inverse(z);
        }
        auto a = t0.find(front);
        auto b = ti.find(back);
        if (a == t0.end() || b == ti.end()) {
          ok = false;
          break;
        }
        meas.push_back(L::compose(L::compose(a->second.pose, z), L::inverse(b->second.pose)));
      }
      if (ok) apply(ri, pose_average(meas));
    }
  }
  int optimize(int64_t n_known_override = -1) {
    LmParamsO lp;
    lp.gauss_newton = (p.solver == RPGO_SOLVER_GN);
    lp.diagonal_damping = p.lm_diagonal_damping != 0;
    std::vector<Factor<L>> full = nfg;
    full.insert(full.end(), temp_nfg.begin(), temp_nfg.end());
    std::map<uint64_t, Pose> full_values = values;
    full_values.insert(temp_values.begin(), temp_values.end());
    std::map<uint64_t, Pose> result;
    SolveStats st;
    const size_t num_lc = pcm ? pcm->total_lc : 0;
    if (p.use_gnc && (pcm || n_known_override >= 0) && !(p.gnc_fix_prev_inliers && num_lc == latest_num_lc)) {
      GncParamsO gp;
      gp.threshold_mode = p.gnc_threshold_mode;
      gp.threshold = p.gnc_inlier_threshold;
      gp.max_iterations = p.gnc_max_iterations;
      gp.mu_step = p.gnc_mu_step;
      gp.rel_cost_tol = p.gnc_relative_cost_tol;
      gp.weights_tol = p.gnc_weights_tol;
      const size_t n_known = n_known_override >= 0 ? (size_t)n_known_override
                                                   : pcm->nfg_odom.size() + pcm->nfg_special.size();
      std::vector<double> init;
      if (p.gnc_bias_odom) {
        init.assign(full.size(), 0.0);
        for (size_t i = 0; i < n_known; ++i) init[i] = 1.0;
      }
      GncResult<S> r;
      bool warm_done = false;
      if (p.gnc_warm_start == RPGO_WARM_ON && warm_probs.size() == full.size()) {
        bool certified = false;
        r = gnc_tls_warm<S>(full, full_values, n_known, gp, lp, warm_probs, p.gnc_warm_mu, &certified);
        ++warm_runs;
        if (certified) warm_done = true;
        else ++warm_fallbacks;
        warm_probs.clear();
      }
      if (p.gnc_warm_start == RPGO_WARM_CONTINUATION) {
        // plain continuation, first weights from the prediction (all ones
        // without one), every later LM from the previous estimate
        std::vector<double> first(full.size(), 1.0);
        if (warm_probs.size() == full.size())
          for (size_t k = n_known; k < full.size(); ++k) first[k] = warm_probs[k] >= 0.5 ? 1.0 : 0.0;
        warm_probs.clear();
        ++warm_runs;
        r = gnc_tls<S>(full, full_values, n_known, gp, lp, &first, -1, true);
        warm_done = true;
      }
      if (!warm_done) {
        SolveStats before = r.stats;
        const int outer_before = r.outer_iterations;
        r = gnc_tls<S>(full, full_values, n_known, gp, lp, p.gnc_bias_odom ? &init : nullptr);
        r.stats.iterations += before.iterations;
        r.stats.linear_solves += before.linear_solves;
        r.outer_iterations += outer_before;
      }
      result = r.values;
      st = r.stats;
      gnc_iters += r.outer_iterations;
      gnc_weights.assign(r.weights.begin(), r.weights.begin() + nfg.size());
      gnc_temp_weights.assign(r.weights.begin() + nfg.size(), r.weights.end());
      const double sum = std::accumulate(gnc_weights.begin(), gnc_weights.end(), 0.0);
      gnc_num_inliers = static_cast<size_t>(sum) - n_known;
    } else {
      if (p.gnc_fix_prev_inliers && pcm) {
        const size_t prev_k = gnc_weights.size() - std::min(latest_num_lc, gnc_weights.size());
        const size_t k = pcm->nfg_odom.size() + pcm->nfg_special.size();
        full.assign(nfg.begin(), nfg.begin() + std::min(k, nfg.size()));
        for (size_t i = 0; i < latest_num_lc; ++i)
          if (prev_k + i < gnc_weights.size() && gnc_weights[prev_k + i] > 0.5 && k + i < nfg.size())
            full.push_back(nfg[k + i]);
        full.insert(full.end(), temp_nfg.begin(), temp_nfg.end());
      }
      NLS<S> nls;
      nls.graph = &full;
      result = nls.optimize(full_values, lp, &st);
      if (st.failed) return RPGO_ERR_SOLVER;
      const size_t tail = std::min(latest_num_lc, gnc_weights.size());
      std::vector<double> lcw(gnc_weights.end() - tail, gnc_weights.end());
      gnc_weights.assign(nfg.size(), 1.0);
      const size_t t2 = std::min(tail, gnc_weights.size());
      for (size_t i = 0; i < t2; ++i) gnc_weights[gnc_weights.size() - t2 + i] = lcw[lcw.size() - t2 + i];
      gnc_temp_weights.assign(temp_nfg.size(), 1.0);
    }
    lm_iters += st.iterations;
    solves += st.linear_solves;
    // GenericSolver::updateValues (src/GenericSolver.cpp:37-45)
    for (auto& kv : result) {
      if (values.count(kv.first)) values[kv.first] = kv.second;
      else if (temp_values.count(kv.first)) temp_values[kv.first] = kv.second;
    }
    if (pcm) latest_num_lc = pcm->total_lc;
    return RPGO_OK;
  }
  void counts(rpgo_counts* c) const override {
    c->num_factors = (int64_t)nfg.size();
    c->num_values = (int64_t)values.size();
    c->num_lc = pcm ? (int64_t)pcm->total_lc : 0;
    c->num_lc_inliers = p.use_gnc ? (int64_t)gnc_num_inliers : (pcm ? (int64_t)pcm->total_good_lc : 0);
    c->num_odom = pcm ? (int64_t)pcm->nfg_odom.size() : 0;
    c->num_special = pcm ? (int64_t)pcm->nfg_special.size() : 0;
    c->num_gnc_weights = (int64_t)gnc_weights.size();
    c->last_do_optimize = last_do_opt ? 1 : 0;
  }
  int estimate(uint64_t* keys, double* poses, int64_t cap) const override {
    if ((int64_t)values.size() > cap) return RPGO_ERR_ARG;
    int64_t i = 0;
    for (auto& kv : values) {
      keys[i] = kv.first;
      L::store(kv.second, poses + i * L::stride);
      ++i;
    }
    return RPGO_OK;
  }
  int weights(double* w, int64_t cap) const override {
    if ((int64_t)gnc_weights.size() > cap) return RPGO_ERR_ARG;
    for (size_t i = 0; i < gnc_weights.size(); ++i) w[i] = gnc_weights[i];
    return RPGO_OK;
  }
  int factors(int32_t* kind, uint64_t* k1, uint64_t* k2, double* meas, int64_t cap) const override {
    if ((int64_t)nfg.size() > cap) return RPGO_ERR_ARG;
    for (size_t i = 0; i < nfg.size(); ++i) {
      kind[i] = nfg[i].kind;
      k1[i] = nfg[i].k1;
      k2[i] = nfg[i].k2;
      if (meas) L::store(nfg[i].measured, meas + i * L::stride);
    }
    return RPGO_OK;
  }
  int adjacency(int32_t group, uint32_t* words, int64_t cap, int64_t* n) const override {
    if (!pcm) return RPGO_ERR_UNSUPPORTED;
    int32_t gi = 0;
    for (auto& kv : pcm->loop_closures) {
      if (gi++ != group) continue;
      const auto& g = kv.second;
      *n = g.n;
      if (!words) return RPGO_OK;
      if ((int64_t)g.bits.size() > cap) return RPGO_ERR_ARG;
      for (size_t i = 0; i < g.bits.size(); ++i) words[i] = g.bits[i];
      return RPGO_OK;
    }
    return RPGO_ERR_ARG;
  }
  void set_warm_probs(const double* pr, int64_t n) override { warm_probs.assign(pr, pr + n); }
  int optimize_timed() {
    for (const auto& f : nfg)
      if (!values.count(f.k1) || !values.count(f.k2)) return RPGO_ERR_KEY;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = optimize();
    this->solve_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
  }
  int remove_last_loop_closure(int by_id, char p1, char p2, uint64_t* k1, uint64_t* k2, int* removed) override {
    bool ok;
    if (pcm) {
      ok = by_id ? pcm->remove_last(ObsId{p1, p2}, k1, k2, &nfg) : pcm->remove_last_in_order(k1, k2, &nfg);
    } else {
      ok = !nfg.empty();
      if (ok) {
        *k1 = nfg.back().k1;
        *k2 = nfg.back().k2;
        nfg.pop_back();
      }
    }
    *removed = ok ? 1 : 0;
    return optimize_timed();
  }
  int ignore_prefix(char c, bool revive) override {
    if (pcm) {
      if (revive) pcm->revive_prefix(c, &nfg);
      else pcm->ignore_prefix(c, &nfg);
    }
    return optimize_timed();
  }
  int ignored_prefixes(char* out, int cap) const override {
    if (!pcm) return 0;
    const int n = (int)pcm->ignored.size();
    for (int i = 0; i < n && i < cap; ++i) out[i] = pcm->ignored[i];
    return n;
  }
  int remove_priors_with_prefix(char c, int optimize_graph) override {
    if (pcm) {
      pcm->remove_priors_with_prefix(c, &nfg);
    } else {
      std::vector<Factor<L>> kept;
      for (const auto& f : nfg)
        if (f.kind != 1 || key_chr(f.k1) != c) kept.push_back(f);
      nfg.swap(kept);
    }
    return optimize_graph ? optimize_timed() : RPGO_OK;
  }
  // RobustSolver::forceUpdate with no new factors or values: optimize()
  int set_temp(const rpgo_factor_batch* f, const rpgo_value_batch* v, bool replace) override {
    std::set<uint64_t> keys;
    if (v)
      for (int64_t k = 0; k < v->count; ++k)
        if (values.count(v->key[k]) || (!replace && temp_values.count(v->key[k])) || !keys.insert(v->key[k]).second)
          return RPGO_ERR_KEY;
    if (replace) clear_temp();
    const auto nf = convert(f);
    temp_nfg.insert(temp_nfg.end(), nf.begin(), nf.end());
    if (v)
      for (int64_t k = 0; k < v->count; ++k) temp_values[v->key[k]] = L::load(v->pose + k * L::stride);
    return RPGO_OK;
  }
  void clear_temp() override {
    temp_nfg.clear();
    temp_values.clear();
  }
  void temp_sizes(int64_t* nf, int64_t* nv) const override {
    *nf = (int64_t)temp_nfg.size();
    *nv = (int64_t)temp_values.size();
  }
  int temp_values_out(uint64_t* keys, double* poses, int64_t cap) const override {
    if ((int64_t)temp_values.size() > cap) return RPGO_ERR_ARG;
    int64_t i = 0;
    for (const auto& kv : temp_values) {
      keys[i] = kv.first;
      L::store(kv.second, poses + i * L::stride);
      ++i;
    }
    return RPGO_OK;
  }
  int temp_weights(double* w, int64_t cap, int64_t* n) const override {
    *n = (int64_t)gnc_temp_weights.size();
    if (*n > cap) return RPGO_ERR_ARG;
    std::copy(gnc_temp_weights.begin(), gnc_temp_weights.end(), w);
    return RPGO_OK;
  }
  int force_optimize() override {
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = optimize();
    this->solve_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
  }
  int pcm_rows(const rpgo_factor_batch* fb, const rpgo_value_batch* vb, const int32_t* rows, int n_rows,
               uint32_t* out, int64_t cap, int64_t* n, int64_t* src, int64_t src_cap, bool lower_only) override {
    if (!pcm || !fb || !vb) return RPGO_ERR_UNSUPPORTED;
    std::set<uint64_t> new_keys;
    for (int64_t k = 0; k < vb->count; ++k) {
      if (values.count(vb->key[k]) || !new_keys.insert(vb->key[k]).second) return RPGO_ERR_KEY;
      values[vb->key[k]] = L::load(vb->pose + k * L::stride);
    }
    pcm->defer_lc = true;
    try {
      pcm->remove_outliers(convert(fb), new_keys, values, &nfg);
    } catch (const std::out_of_range&) {
      return RPGO_ERR_KEY;
    }
    if (pcm->loop_closures.empty()) {
      *n = 0;
      return RPGO_OK;
    }
    auto& g = pcm->loop_closures.begin()->second;
    *n = (int64_t)g.factors.size();
    const int words = (int)((g.factors.size() + 31) / 32);
    std::vector<int> rv;
    for (int i = 0; i < n_rows; ++i) {
      if (rows[i] < 0 || rows[i] >= (int)g.factors.size()) return RPGO_ERR_ARG;
      rv.push_back(rows[i]);
    }
    if (src) {
      if (src_cap < *n) return RPGO_ERR_ARG;
      for (size_t i = 0; i < g.factors.size(); ++i) src[i] = g.factors[i].src;
    }
    if (out) {
      if (cap < (int64_t)rv.size() * words) return RPGO_ERR_ARG;
      std::vector<uint32_t> bits;
      pcm->sample_rows(g, rv, &bits, lower_only);
      std::copy(bits.begin(), bits.end(), out);
    }
    return RPGO_OK;
  }
  int solve_graph(const rpgo_factor_batch* fb, const rpgo_value_batch* vb, int64_t n_known) override {
    if (!fb || !vb || n_known < 0 || n_known > fb->count) return RPGO_ERR_ARG;
    for (int64_t k = 0; k < vb->count; ++k) {
      if (values.count(vb->key[k])) return RPGO_ERR_KEY;
      values[vb->key[k]] = L::load(vb->pose + k * L::stride);
    }
    nfg = convert(fb);
    for (const auto& f : nfg)
      if (!values.count(f.k1) || !values.count(f.k2)) return RPGO_ERR_KEY;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = optimize(n_known);
    this->solve_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
  }
  void stats(int64_t* a, int64_t* b, int64_t* c) const override {
    *a = lm_iters;
    *b = solves;
    *c = gnc_iters;
  }
};

template <class L>
void load_pwc(const double* pose, const double* cov, int rot_info, PWC<L>* x) {
  x->pose = L::load(pose);
  std::memcpy(x->cov, cov, sizeof(double) * L::dim * L::dim);
  x->rot_info = rot_info != 0;
}
template <class L>
void store_pwc(const PWC<L>& x, double* pose, double* cov, int* rot_info) {
  L::store(x.pose, pose);
  std::memcpy(cov, x.cov, sizeof(double) * L::dim * L::dim);
  if (rot_info) *rot_info = x.rot_info ? 1 : 0;
}

}  // namespace

extern "C" {

void* oracle_create(const rpgo_params* p) {
  const int m = p->outlier_removal;
  const int dim = (m == RPGO_OUTLIER_PCM2D || m == RPGO_OUTLIER_PCM_SIMPLE2D) ? 2
                  : (m == RPGO_OUTLIER_NONE) ? p->dim : 3;
  SolverBase* s = nullptr;
  switch (m) {
    case RPGO_OUTLIER_NONE:
      if (dim == 2) s = new RobustSolverO<Sol2, PWC<Lie2>>(*p, false);
      else if (dim == 3) s = new RobustSolverO<Sol3, PWC<Lie3>>(*p, false);
      break;
    case RPGO_OUTLIER_PCM2D: s = new RobustSolverO<Sol2, PWC<Lie2>>(*p, true); break;
    case RPGO_OUTLIER_PCM3D: s = new RobustSolverO<Sol3, PWC<Lie3>>(*p, true); break;
    case RPGO_OUTLIER_PCM_SIMPLE2D: s = new RobustSolverO<Sol2, PWN<Lie2>>(*p, true); break;
    case RPGO_OUTLIER_PCM_SIMPLE3D: s = new RobustSolverO<Sol3, PWN<Lie3>>(*p, true); break;
    default: break;
  }
  return s;
}
void oracle_destroy(void* s) { delete static_cast<SolverBase*>(s); }
int oracle_update(void* s, const rpgo_factor_batch* f, const rpgo_value_batch* v, int32_t opt) {
  return static_cast<SolverBase*>(s)->update(f, v, opt);
}
int oracle_get_counts(void* s, rpgo_counts* c) {
  static_cast<SolverBase*>(s)->counts(c);
  return 0;
}
int oracle_get_estimate(void* s, uint64_t* k, double* p, int64_t cap) {
  return static_cast<SolverBase*>(s)->estimate(k, p, cap);
}
int oracle_get_gnc_weights(void* s, double* w, int64_t cap) { return static_cast<SolverBase*>(s)->weights(w, cap); }
int oracle_get_factors(void* s, int32_t* kind, uint64_t* k1, uint64_t* k2, double* meas, int64_t cap) {
  return static_cast<SolverBase*>(s)->factors(kind, k1, k2, meas, cap);
}
int oracle_get_adjacency(void* s, int32_t g, uint32_t* w, int64_t cap, int64_t* n) {
  return static_cast<SolverBase*>(s)->adjacency(g, w, cap, n);
}
int oracle_get_stats(void* s, int64_t* lm, int64_t* solves, int64_t* gnc) {
  static_cast<SolverBase*>(s)->stats(lm, solves, gnc);
  return 0;
}
// warm-started GNC: inlier probabilities of the next solve's factors (graph
// order; known inliers ignored), and the warm counters
int oracle_set_warm_probs(void* s, const double* probs, int64_t n) {
  static_cast<SolverBase*>(s)->set_warm_probs(probs, n);
  return 0;
}
int oracle_force_optimize(void* s) { return static_cast<SolverBase*>(s)->force_optimize(); }
// OpenMP threads of the pair tests (0: keep); returns the current count
int oracle_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}
int oracle_set_temp(void* s, const rpgo_factor_batch* f, const rpgo_value_batch* v, int replace) {
  return static_cast<SolverBase*>(s)->set_temp(f, v, replace != 0);
}
int oracle_clear_temp(void* s) {
  static_cast<SolverBase*>(s)->clear_temp();
  return RPGO_OK;
}
int oracle_temp_sizes(void* s, int64_t* nf, int64_t* nv) {
  static_cast<SolverBase*>(s)->temp_sizes(nf, nv);
  return RPGO_OK;
}
int oracle_temp_values(void* s, uint64_t* k, double* p, int64_t cap) {
  return static_cast<SolverBase*>(s)->temp_values_out(k, p, cap);
}
int oracle_temp_weights(void* s, double* w, int64_t cap, int64_t* n) {
  return static_cast<SolverBase*>(s)->temp_weights(w, cap, n);
}
int oracle_remove_last_loop_closure(void* s, int by_id, char p1, char p2, uint64_t* k1, uint64_t* k2, int* removed) {
  return static_cast<SolverBase*>(s)->remove_last_loop_closure(by_id, p1, p2, k1, k2, removed);
}
int oracle_ignore_prefix(void* s, char c, int revive) { return static_cast<SolverBase*>(s)->ignore_prefix(c, revive); }
int oracle_ignored_prefixes(void* s, char* out, int cap) {
  return static_cast<SolverBase*>(s)->ignored_prefixes(out, cap);
}
int oracle_remove_priors_with_prefix(void* s, char c, int optimize_graph) {
  return static_cast<SolverBase*>(s)->remove_priors_with_prefix(c, optimize_graph);
}
int oracle_get_warm_stats(void* s, int64_t* runs, int64_t* fallbacks) {
  *runs = static_cast<SolverBase*>(s)->warm_runs;
  *fallbacks = static_cast<SolverBase*>(s)->warm_fallbacks;
  return 0;
}
int oracle_get_times(void* s, double* pcm_seconds, double* solve_seconds) {
  *pcm_seconds = static_cast<SolverBase*>(s)->pcm_seconds;
  *solve_seconds = static_cast<SolverBase*>(s)->solve_seconds;
  return 0;
}

// ---- geometry known-answer hooks (GeometryUtils.h)
// op: 0 compose, 1 between, 2 inverse (b ignored)
int oracle_pwc_op(int dim, int op, const double* pa, const double* ca, int ria, const double* pb, const double* cb,
                  int rib, double* pout, double* cout, int* riout) {
  if (dim == 3) {
    PWC<Lie3> a, b, r;
    load_pwc(pa, ca, ria, &a);
    if (op != 2) load_pwc(pb, cb, rib, &b);
    r = op == 0 ? a.compose(b) : op == 1 ? a.between(b) : a.inverse();
    store_pwc(r, pout, cout, riout);
  } else {
    PWC<Lie2> a, b, r;
    load_pwc(pa, ca, ria, &a);
    if (op != 2) load_pwc(pb, cb, rib, &b);
    r = op == 0 ? a.compose(b) : op == 1 ? a.between(b) : a.inverse();
    store_pwc(r, pout, cout, riout);
  }
  return 0;
}
double oracle_pwc_mahalanobis(int dim, const double* pose, const double* cov, int rot_info) {
  if (dim == 3) {
    PWC<Lie3> a;
    load_pwc(pose, cov, rot_info, &a);
    return a.mahalanobis_norm();
  }
  PWC<Lie2> a;
  load_pwc(pose, cov, rot_info, &a);
  return a.mahalanobis_norm();
}
// PoseWithNode norms: out[0] = avg_trans_norm, out[1] = avg_rot_norm
int oracle_pwn_norms(int dim, const double* pose, int node, int rot_info, double* out) {
  if (dim == 3) {
    PWN<Lie3> a;
    a.pose = Lie3::load(pose);
    a.node = node;
    a.rot_info = rot_info != 0;
    out[0] = a.avg_trans_norm();
    out[1] = a.avg_rot_norm();
  } else {
    PWN<Lie2> a;
    a.pose = Lie2::load(pose);
    a.node = node;
    a.rot_info = rot_info != 0;
    out[0] = a.avg_trans_norm();
    out[1] = a.avg_rot_norm();
  }
  return 0;
}
int oracle_logmap(int dim, const double* pose, double* xi) {
  if (dim == 3) p3_logmap(Lie3::load(pose), xi);
  else p2_logmap(Lie2::load(pose), xi);
  return 0;
}
double oracle_atan2(double y, double x) { return r_atan2(y, x); }
double oracle_chi2inv(double alpha, int k) { return chi2inv(alpha, k); }

// Pairwise adjacency of n closures against a trajectory given by slots
// (the stage restated without the solver state). mode 0 PoseWithCovariance,
// 1 PoseWithNode. adj: n x ceil(n/32) words (cleared here).
int oracle_pairwise_adjacency(int dim, int mode, int n, const int32_t* slot_a, const int32_t* slot_b,
                              const uint8_t* flip, const double* z_pose, const double* z_cov,
                              const double* traj_pose, const double* traj_cov, const int32_t* traj_node,
                              const uint8_t* traj_rot, double th0, double th1, uint32_t* adj) {
  const int words = (n + 31) / 32;
  std::memset(adj, 0, sizeof(uint32_t) * (size_t)n * words);
  auto body = [&](auto lie, auto kind) {
    using L = decltype(lie);
    constexpr bool simple = decltype(kind)::value;
    constexpr int dd = L::dim;
    auto traj = [&](int s) {
      if constexpr (simple) {
        PWN<L> x;
        x.pose = L::load(traj_pose + (size_t)s * L::stride);
        x.node = traj_node[s];
        x.rot_info = traj_rot[s] != 0;
        return x;
      } else {
        PWC<L> x;
        x.pose = L::load(traj_pose + (size_t)s * L::stride);
        std::memcpy(x.cov, traj_cov + (size_t)s * dd * dd, sizeof(double) * dd * dd);
        x.rot_info = traj_rot[s] != 0;
        return x;
      }
    };
    using U = decltype(traj(0));
    for (int j = 1; j < n; ++j)
      for (int i = 0; i < j; ++i) {
        U zab = U::from_factor(L::load(z_pose + (size_t)i * L::stride), z_cov + (size_t)i * dd * dd);
        U zcd = U::from_factor(L::load(z_pose + (size_t)j * L::stride), z_cov + (size_t)j * dd * dd);
        int sa = slot_a[i], sb = slot_b[i], sc = slot_a[j], sd = slot_b[j];
        if (flip[i] != flip[j]) std::swap(sc, sd);
        U a_odom_c = traj(sa).between(traj(sc));
        U b_odom_d = traj(sb).between(traj(sd));
        U loop = a_odom_c.compose(zcd).inverse().compose(zab).compose(b_odom_d);
        bool ok;
        if constexpr (simple) ok = loop.avg_trans_norm() < th0 && loop.avg_rot_norm() < th1;
        else ok = loop.mahalanobis_norm() < th0;
        if (ok) {
          adj[(size_t)i * words + (j >> 5)] |= 1u << (j & 31);
          adj[(size_t)j * words + (i >> 5)] |= 1u << (i & 31);
        }
      }
  };
  if (dim == 3) {
    if (mode == 0) body(Lie3{}, std::false_type{});
    else body(Lie3{}, std::true_type{});
  } else {
    if (mode == 0) body(Lie2{}, std::false_type{});
    else body(Lie2{}, std::true_type{});
  }
  return 0;
}

// 0: the reference's linear-search greedy clique (default), 1: the
// membership-stamp form, 2: the bit-row form (both with identical results);
// returns the previous value
int oracle_set_clique_impl(int impl) {
  const int old = g_clique_impl;
  g_clique_impl = impl;
  return old;
}
// On a fresh solver: classify, odometry-check and group the closures of one
// batch (no consistency matrix); the first group's size n, the input-batch
// index of each of its closures (src, n entries) and the requested rows of
// its consistency matrix (out: n_rows x ceil(n / 32) words; lower_only:
// columns below the diagonal only)
int oracle_pcm_rows(void* s, const rpgo_factor_batch* f, const rpgo_value_batch* v, const int32_t* rows,
                    int32_t n_rows, uint32_t* out, int64_t cap, int64_t* n, int64_t* src, int64_t src_cap,
                    int lower_only) {
  return static_cast<SolverBase*>(s)->pcm_rows(f, v, rows, n_rows, out, cap, n, src, src_cap, lower_only != 0);
}
// linear-search iterations of the reference's greedy clique on a bit-packed
// adjacency (n x ceil(n/32) words): counted exactly (exact != 0, O(|S| +
// deg) per round), or estimated on bit rows (positions of the kept elements
// in the neighbour list to their 64-bit word; OpenMP)
double oracle_clique_scan_ops(int n, const uint32_t* adj, int exact) {
  const int words = (n + 31) / 32;
  std::vector<uint32_t> bits(adj, adj + (size_t)n * words);
  if (exact) return fmc_scan_ops(csr_from_bits(bits, n, words), 0, -1);
  std::vector<int> best;
  double ops = 0.0;
  fmc_heuristic_bits(BitRows(bits, n, words), 0, -1, &best, &ops);
  return ops;
}
// iterations cap of every LM / GN run (-1: the solver's own); returns the old
int oracle_set_lm_max_iterations(int n) {
  const int old = g_lm_max_iterations;
  g_lm_max_iterations = n;
  return old;
}
// On a fresh solver: RobustSolver::optimize over the given factor list and
// values, GNC known inliers = factors [0, n_known)
int oracle_solve_graph(void* s, const rpgo_factor_batch* f, const rpgo_value_batch* v, int64_t n_known) {
  return static_cast<SolverBase*>(s)->solve_graph(f, v, n_known);
}

// Greedy max clique on a bit-packed adjacency (n x ceil(n/32) words).
int oracle_max_clique_heu(int n, const uint32_t* adj, int first, int seed, int32_t* clique_out, int32_t* size_out) {
  const int words = (n + 31) / 32;
  std::vector<uint32_t> bits(adj, adj + (size_t)n * words);
  std::vector<int> best;
  int sz = fmc_from_bits(bits, n, words, first, seed, &best);
  *size_out = sz;
  for (int i = 0; i < sz && i < (int)best.size(); ++i) clique_out[i] = best[i];
  return 0;
}

}  // extern "C"

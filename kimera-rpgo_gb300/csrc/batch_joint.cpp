// Joint batch (batch_joint.hpp): lock-step GNC-TLS / LM over many graphs.
#include "batch_joint.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <map>
#include <stdexcept>
#include <thread>

#include "chol.hpp"
#include "chol_plan.hpp"

namespace rpgo {

namespace {

std::atomic<bool> g_joint_graphs{true};         // capture the round as a CUDA graph
std::atomic<int64_t> g_joint_graph_rounds{0};   // rounds replayed from a graph (process-wide)

struct Local {  // one graph in the union's numbering
  std::vector<int32_t> kind, vi, vj;
  std::vector<int64_t> frows, vrows;
  CholPlan plan;
};

// variables in key order of the value store, factors in list order (as GpuNls)
void localise(int d, const JointProblem& p, Local* out) {
  std::map<uint64_t, int> index;
  for (const auto& kv : p.values->rows()) {
    index[kv.first] = (int)out->vrows.size();
    out->vrows.push_back(kv.second);
  }
  const size_t F = p.graph.size();
  out->kind.resize(F);
  out->vi.resize(F);
  out->vj.resize(F);
  out->frows.resize(F);
  for (size_t f = 0; f < F; ++f) {
    const FactorRec& r = p.graph[f];
    out->kind[f] = r.kind;
    out->vi[f] = index.at(r.k1);
    out->vj[f] = r.kind == 0 ? index.at(r.k2) : out->vi[f];
    out->frows[f] = r.row;
  }
  out->plan = make_chol_plan((int)out->vrows.size(), d, out->kind, out->vi, out->vj, false);
}

// Host state of one graph: GpuNls::optimize's LM / GN loop and gnc_tls's
// outer loop, cut at every damped solve.
struct Graph {
  JointProblem* p = nullptr;
  enum Phase { kLmStart, kLmStep, kDone } phase = kLmStart;
  // LM
  double lambda = 0.0, cur_err = 0.0, new_err = 0.0, current_error = 0.0;
  int iters = 0;
  bool accept_pending = false;  // x <- xnew at the start of the next round
  // GNC
  bool in_gnc = false;    // the GNC loop has started (after the first LM run)
  int gnc_it = 0;
  double mu = -1.0, mu0 = -1.0, prev_cost = 0.0;
  bool gnc_pending = false;     // TLS weights at the start of the next round
  bool need_weights = false;    // download this graph's weights after the next round
  std::vector<double> w;        // host copy of the weights of the current GNC stage
};

}  // namespace

int solve_joint(int dim, std::vector<JointProblem*>& probs, cudaStream_t st, int coop_ctas) {
  const int G = (int)probs.size();
  if (G == 0) return 0;
  const int d = dim == 3 ? 6 : 3, stride = dim == 3 ? 12 : 4;
  // per-graph numbering and plans (no dense tails), on host threads
  std::vector<Local> loc(G);
  {
    std::atomic<int> next{0};
    std::vector<std::exception_ptr> err(G);
    auto work = [&] {
      for (int g; (g = next.fetch_add(1)) < G;) {
        try {
          localise(d, *probs[g], &loc[g]);
        } catch (...) {
          err[g] = std::current_exception();
        }
      }
    };
    const int nt = std::max(1, std::min<int>(G, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    for (auto& e : err)
      if (e) std::rethrow_exception(e);
  }
  // the union problem
  BatchDev b;
  b.G = G;
  b.h_voff.assign(G + 1, 0);
  b.h_foff.assign(G + 1, 0);
  for (int g = 0; g < G; ++g) {
    b.h_voff[g + 1] = b.h_voff[g] + (int32_t)loc[g].vrows.size();
    b.h_foff[g + 1] = b.h_foff[g] + (int32_t)loc[g].kind.size();
  }
  const int N = b.h_voff[G], F = b.h_foff[G];
  std::vector<int32_t> kind(F), vi(F), vj(F), vsys(N), fsys(F), nknown(G);
  std::vector<double> barc(F);
  for (int g = 0; g < G; ++g) {
    const int v0 = b.h_voff[g], f0 = b.h_foff[g];
    const Local& l = loc[g];
    for (size_t f = 0; f < l.kind.size(); ++f) {
      kind[f0 + f] = l.kind[f];
      vi[f0 + f] = l.vi[f] + v0;
      vj[f0 + f] = l.vj[f] + v0;
      fsys[f0 + f] = g;
    }
    for (int v = v0; v < b.h_voff[g + 1]; ++v) vsys[v] = g;
    nknown[g] = (int32_t)probs[g]->n_known;
    const GncConfig& c = probs[g]->gnc_cfg;
    const double bc = c.threshold_mode == 0 ? c.threshold : 0.5 * chi2inv(c.threshold, d);
    std::fill(barc.begin() + f0, barc.begin() + b.h_foff[g + 1], bc);
  }
  std::vector<CholPlan> plans(G);
  for (int g = 0; g < G; ++g) plans[g] = std::move(loc[g].plan);
  CholPlan merged = merge_chol_plans(plans, b.h_foff);
  plans.clear();
  SolverDev u;
  u.coop_ctas = coop_ctas;
  solver_upload(u, dim, kind, vi, vj, N, st, true, &merged);
  if (!u.chol) throw std::runtime_error("joint batch: the merged factor exceeds the direct solver's memory budget");
  std::vector<DeviceBuffer<int64_t>> vrows(G);
  for (int g = 0; g < G; ++g) {
    const Local& l = loc[g];
    const int v0 = b.h_voff[g], f0 = b.h_foff[g];
    DeviceBuffer<int64_t> fr;
    fr.upload(l.frows, st);
    vrows[g].upload(l.vrows, st);
    gather_rows((int64_t)l.frows.size(), fr.get(), probs[g]->store->meas(), stride, u.z.get() + (size_t)f0 * stride,
                st);
    gather_rows((int64_t)l.frows.size(), fr.get(), probs[g]->store->sqrt_info(), d * d,
                u.sqrt_info.get() + (size_t)f0 * d * d, st);
    gather_rows((int64_t)l.vrows.size(), vrows[g].get(), probs[g]->values->pose(), stride,
                u.x0.get() + (size_t)v0 * stride, st);
    RPGO_CUDA(cudaStreamSynchronize(st));  // (fr is freed at the end of this scope)
  }
  RPGO_CUDA(cudaMemcpyAsync(u.x.get(), u.x0.get(), (size_t)N * stride * sizeof(double), cudaMemcpyDeviceToDevice, st));
  RPGO_CUDA(cudaMemcpyAsync(u.xnew.get(), u.x0.get(), (size_t)N * stride * sizeof(double), cudaMemcpyDeviceToDevice,
                            st));
  b.vsys.upload(vsys, st);
  b.fsys.upload(fsys, st);
  b.voff.upload(b.h_voff, st);
  b.foff.upload(b.h_foff, st);
  b.nknown.upload(nknown, st);
  b.barc.upload(barc, st);
  b.ctl.resize(G);
  b.vmask.resize(N);
  b.fmask.resize(F);
  b.lam.resize(G);
  b.mu.resize(G);
  b.status.resize(G);
  b.out.resize((size_t)2 * G);
  b.term.resize((size_t)2 * N);
  b.err.resize((size_t)2 * G);
  // first weights
  std::vector<double> w0(F, 1.0);
  for (int g = 0; g < G; ++g) {
    const auto& iw = probs[g]->init_weights;
    if (probs[g]->gnc && !iw.empty())
      for (size_t k = 0; k < iw.size() && b.h_foff[g] + (int)k < b.h_foff[g + 1]; ++k) w0[b.h_foff[g] + k] = iw[k];
  }
  u.weights.upload(w0, st);
  // mu from the unweighted residuals at the initial values (gnc_tls)
  std::vector<double> r0;
  solver_factor_errors(u, u.x0.get(), &r0, st);
  std::vector<Graph> gs(G);
  for (int g = 0; g < G; ++g) {
    Graph& x = gs[g];
    x.p = probs[g];
    x.p->stats = NlsStats{};
    x.p->failed = false;
    double mu = std::numeric_limits<double>::infinity();
    for (int f = b.h_foff[g]; f < b.h_foff[g + 1]; ++f)
      if (2.0 * r0[f] - barc[f] > 0.0) mu = std::min(mu, barc[f] / (2.0 * r0[f] - barc[f]));
    if (mu >= 0.0 && mu < 1e-6) mu = 1e-6;
    if (!(mu > 0.0) || std::isinf(mu)) mu = -1.0;
    x.mu0 = mu;
    x.w.assign(w0.begin() + b.h_foff[g], w0.begin() + b.h_foff[g + 1]);
  }

  PinnedBuffer<uint8_t> hctl;
  PinnedBuffer<double> hlam, hmu, hres, hw;
  uint8_t* ctl = hctl.get(G);
  double* lam = hlam.get(G);
  double* mus = hmu.get(G);
  double* res = hres.get((size_t)4 * G);  // err (2G), then out (2G)
  const double eps = std::numeric_limits<double>::epsilon();

  // an LM run from the initial values starts in the next round: x <- x0, the
  // error at x0, and a solve with the initial lambda (used unless the error
  // at x0 already ends the run)
  auto lm_begin = [&](Graph& x) {
    x.phase = Graph::kLmStart;
    x.lambda = x.p->lm.gauss_newton ? 0.0 : x.p->lm.lambda_initial;
  };
  auto finish = [&](Graph& x) { x.phase = Graph::kDone; };
  // the LM run of graph x ended: GNC's outer loop (gnc_tls)
  auto lm_end = [&](Graph& x) {
    JointProblem& P = *x.p;
    if (!P.gnc) return finish(x);
    if (!x.in_gnc) {
      x.in_gnc = true;
      x.mu = x.mu0;
      x.prev_cost = x.cur_err;
      if (P.graph.size() == P.n_known || x.mu <= 0.0 || P.gnc_cfg.max_iterations <= 0) return finish(x);
      x.gnc_it = 0;
    } else {
      const double cost = x.cur_err;
      bool conv = std::fabs(cost - x.prev_cost) / std::max(x.prev_cost, 1e-7) < P.gnc_cfg.rel_cost_tol;
      if (!conv) {
        conv = true;
        for (double wk : x.w)
          if (std::fabs(wk - std::round(wk)) > P.gnc_cfg.weights_tol) {
            conv = false;
            break;
          }
      }
      if (conv) return finish(x);
      x.mu *= P.gnc_cfg.mu_step;
      x.prev_cost = cost;
      if (++x.gnc_it >= P.gnc_cfg.max_iterations) return finish(x);
    }
    P.stats.gnc_iterations++;
    x.gnc_pending = true;
    x.need_weights = true;
    lm_begin(x);
  };
  // end of an outer LM iteration (new_err = cur_err; convergence test)
  auto outer_end = [&](Graph& x) {
    const LmParams& lp = x.p->lm;
    x.new_err = x.cur_err;
    const double abs_dec = x.current_error - x.new_err;
    const double rel_dec = abs_dec / x.current_error;
    const bool converged =
        (x.new_err <= lp.error_tol) || (lp.rel_tol != 0.0 && rel_dec <= lp.rel_tol) || (abs_dec <= lp.abs_tol);
    if (x.iters >= lp.max_iterations || converged || !std::isfinite(x.current_error)) {
      x.p->stats.iterations += x.iters;
      return lm_end(x);
    }
    x.current_error = x.new_err;
    x.phase = Graph::kLmStep;
  };
  // the result of this round's damped solve at x with lambda
  auto consume_step = [&](Graph& x, bool ok, double lin_change, double nerr) {
    const LmParams& lp = x.p->lm;
    x.p->stats.linear_solves++;
    if (lp.gauss_newton) {
      if (!ok) {  // the GN run ends (GpuNls::optimize returns); GNC goes on
        x.p->failed = true;
        x.p->stats.failed = true;
        return lm_end(x);
      }
      x.accept_pending = true;
      x.cur_err = nerr;
      ++x.iters;
      return outer_end(x);
    }
    bool success = false, stop_search = false;
    if (ok && lin_change >= 0.0) {
      const double cost_change = x.cur_err - nerr;
      if (lin_change > eps * x.cur_err) success = (cost_change / lin_change) > lp.min_model_fidelity;
      else success = true;
      if (std::fabs(cost_change) < lp.rel_tol * x.cur_err) stop_search = true;
    }
    if (success) {
      x.accept_pending = true;
      x.cur_err = nerr;
      x.lambda = std::max(lp.lambda_lower, x.lambda / lp.lambda_factor);
      ++x.iters;
      return outer_end(x);
    }
    if (!stop_search) {
      x.lambda *= lp.lambda_factor;
      if (x.lambda >= lp.lambda_upper) return outer_end(x);
      return;  // same x, larger lambda: solve again next round
    }
    outer_end(x);
  };

  int rounds = 0;
  // One round's device work: the control words, dampings and mu in, the
  // stages before the direct solve; the direct solve; the stages after it and
  // the per-graph results out. The stages before and after are replayed
  // from two captured CUDA graphs once the buffers have their sizes (after
  // the first round; the host arrays are page-locked and fixed); the direct
  // solve, a cooperative launch, is launched on its own between them. If a
  // capture or instantiation is refused, the stages launch one by one.
  auto enqueue_pre = [&](bool any_active) {
    RPGO_CUDA(cudaMemcpyAsync(b.ctl.get(), ctl, G, cudaMemcpyHostToDevice, st));
    RPGO_CUDA(cudaMemcpyAsync(b.lam.get(), lam, G * sizeof(double), cudaMemcpyHostToDevice, st));
    RPGO_CUDA(cudaMemcpyAsync(b.mu.get(), mus, G * sizeof(double), cudaMemcpyHostToDevice, st));
    batch_round_pre(u, b, probs[0]->lm.diagonal_damping, any_active, st);
  };
  auto enqueue_post = [&] {
    batch_round_post(u, b, st);
    RPGO_CUDA(cudaMemcpyAsync(res, b.err.get(), 2 * G * sizeof(double), cudaMemcpyDeviceToHost, st));
    RPGO_CUDA(cudaMemcpyAsync(res + 2 * G, b.out.get(), 2 * G * sizeof(double), cudaMemcpyDeviceToHost, st));
  };
  cudaGraphExec_t exec_pre = nullptr, exec_post = nullptr;
  bool use_graph = g_joint_graphs.load();
  int64_t graph_launches = 0;
  auto capture = [&](auto&& enqueue) -> cudaGraphExec_t {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t e = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      (void)cudaGetLastError();
      return nullptr;
    }
    bool ok = true;
    try {
      enqueue();
    } catch (const CudaError&) {
      ok = false;
    }
    const cudaError_t ec = cudaStreamEndCapture(st, &graph);
    ok = ok && ec == cudaSuccess && graph != nullptr;
    if (ok && cudaGraphInstantiate(&e, graph, 0) != cudaSuccess) {
      ok = false;
      e = nullptr;
    }
    if (graph) cudaGraphDestroy(graph);
    (void)cudaGetLastError();
    return ok ? e : nullptr;
  };
  // the set of graphs whose items the direct solve's compacted lists hold
  std::vector<uint8_t> listed(G, 2);
  auto recompact = [&] {
    bool changed = false;
    for (int g = 0; g < G; ++g) {
      const uint8_t on = ctl[g] & kBatchActive;
      if (on != listed[g]) changed = true;
      listed[g] = on;
    }
    return changed;
  };
  auto run_round = [&](bool any_active) {
    if (any_active && use_graph && rounds >= 1 && !exec_pre) {
      exec_pre = capture([&] { enqueue_pre(true); });
      exec_post = exec_pre ? capture(enqueue_post) : nullptr;
      if (!exec_pre || !exec_post) {
        use_graph = false;
        if (exec_pre) cudaGraphExecDestroy(exec_pre);
        if (exec_post) cudaGraphExecDestroy(exec_post);
        exec_pre = exec_post = nullptr;
      }
    }
    if (any_active && exec_pre) {
      RPGO_CUDA(cudaGraphLaunch(exec_pre, st));
      batch_round_solve(u, b, recompact(), st);
      RPGO_CUDA(cudaGraphLaunch(exec_post, st));
      ++graph_launches;
    } else {
      enqueue_pre(any_active);
      if (any_active) {
        batch_round_solve(u, b, recompact(), st);
        enqueue_post();
      }
    }
  };

  for (Graph& x : gs) lm_begin(x);
  for (;;) {
    bool any_active = false, any_ctl = false, any_w = false;
    for (int g = 0; g < G; ++g) {
      Graph& x = gs[g];
      uint8_t c = 0;
      if (x.accept_pending) c |= kBatchAccept;
      if (x.phase != Graph::kDone) {
        if (x.gnc_pending) c |= kBatchGnc;
        if (x.phase == Graph::kLmStart) {
          // LM from the initial values: every run of plain GNC and the first
          c |= kBatchReset | kBatchError;
        }
        c |= kBatchActive;
        any_active = true;
      }
      ctl[g] = c;
      lam[g] = x.lambda;
      mus[g] = x.mu;
      any_ctl = any_ctl || c != 0;
      any_w = any_w || x.need_weights;
    }
    if (!any_ctl) break;
    run_round(any_active);
    double* hwp = nullptr;
    if (any_w) {  // the weight slices of the graphs that start a GNC stage
      hwp = hw.get(F);
      for (int g = 0; g < G; ++g)
        if (gs[g].need_weights)
          RPGO_CUDA(cudaMemcpyAsync(hwp + b.h_foff[g], u.weights.get() + b.h_foff[g],
                                    (size_t)(b.h_foff[g + 1] - b.h_foff[g]) * sizeof(double), cudaMemcpyDeviceToHost,
                                    st));
    }
    RPGO_CUDA(cudaStreamSynchronize(st));
    if (any_active) {
      ++rounds;
      kernel_times().chol_ms += chol_last_ms(*u.chol);
      kernel_times().chol_launches += 1;
      kernel_times().chol_flops += u.chol->plan.flops;
      kernel_times().chol_bytes += u.chol->plan.bytes;
      kernel_times().chol_levels = u.chol->levels;
      kernel_times().chol_tail = 0;
    }
    for (int g = 0; g < G; ++g) {
      Graph& x = gs[g];
      const uint8_t c = ctl[g];
      if (c & kBatchAccept) x.accept_pending = false;
      if (c & kBatchGnc) x.gnc_pending = false;
      if (x.need_weights && hwp) {
        x.w.assign(hwp + b.h_foff[g], hwp + b.h_foff[g + 1]);
        x.need_weights = false;
      }
      if (!(c & kBatchActive)) continue;
      const double errx = res[g], nerr = res[G + g], lin_change = res[2 * G + 2 * g];
      const bool ok = res[2 * G + 2 * g + 1] == 0.0;
      if (x.phase == Graph::kLmStart) {
        x.cur_err = errx;
        const LmParams& lp = x.p->lm;
        if (x.cur_err <= lp.error_tol || lp.max_iterations <= 0) {
          lm_end(x);
          continue;
        }
        x.iters = 0;
        x.new_err = x.cur_err;
        x.current_error = x.new_err;
        x.lambda = lp.gauss_newton ? 0.0 : lp.lambda_initial;
        x.phase = Graph::kLmStep;
      }
      consume_step(x, ok, lin_change, nerr);
    }
  }
  // results: estimates into the value stores, weights
  std::vector<double> wf(F);
  u.weights.download(wf.data(), F, st);
  for (int g = 0; g < G; ++g) {
    const int v0 = b.h_voff[g];
    scatter_rows((int64_t)loc[g].vrows.size(), vrows[g].get(), u.x.get() + (size_t)v0 * stride, stride,
                 probs[g]->values->pose(), st);
    probs[g]->weights.assign(wf.begin() + b.h_foff[g], wf.begin() + b.h_foff[g + 1]);
  }
  RPGO_CUDA(cudaStreamSynchronize(st));
  if (exec_pre) cudaGraphExecDestroy(exec_pre);
  if (exec_post) cudaGraphExecDestroy(exec_post);
  g_joint_graph_rounds.fetch_add(graph_launches);
  return rounds;
}

bool set_joint_graphs(bool on) { return g_joint_graphs.exchange(on); }
int64_t joint_graph_rounds() { return g_joint_graph_rounds.load(); }

}  // namespace rpgo

// Batched solve of independent graphs (rpgo_solve_batch and
// rpgo_solve_batch_joint, include/rpgo_gb300.h).
//
// rpgo_solve_batch: each graph is an ordinary rpgo_solver (RobustSolver look-alike) on its own
// non-blocking stream; `workers` host threads take graphs from a shared
// counter. The GPU runs the workers' kernels concurrently: the per-graph
// kernels of PCM (trajectory scan, odometry and pairwise checks, clique) are
// small, latency-bound launches, and each cooperative direct solve is limited
// to `coop_ctas` CTAs so that several fit on the device at once. Device memory
// is stream-ordered (no device-wide synchronisation on free), so the workers
// do not serialise each other.
//
// rpgo_solve_batch_joint: every graph's PCM on its own solver (worker
// threads), then the GNC / LM solves of all graphs in lock-step rounds with
// one launch per stage over all of them (batch_joint.cpp).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <exception>
#include <thread>
#include <vector>

#include "../../include/rpgo_gb300.h"
#include "batch_joint.hpp"
#include "common.cuh"

namespace rpgo {
void set_coop_ctas(rpgo_solver* s, int ctas);
}

namespace {

constexpr int kDefaultWorkers = 16;
// concurrent lock-step groups of the joint batch
constexpr int kDefaultJointStreams = 4;
// host threads of the joint batch's per-graph stages (PCM, outputs)
constexpr int kJointHostThreads = 32;
// co-resident CTAs of the direct solve per SM (256 threads x 128 registers)
constexpr int kCholCtasPerSm = 2;

// the estimate, weights and timing of solver s into the batch outputs
int write_outputs(rpgo_solver* s, int rc, const rpgo_factor_batch& f, const rpgo_value_batch& v, double* poses,
                  int64_t stride, double* weights, int64_t* num_weights, rpgo_timing* timing) {
  if (rc == RPGO_OK) {
    rpgo_counts c;
    rpgo_get_counts(s, &c);
    std::vector<uint64_t> keys((size_t)c.num_values);
    if (c.num_values == v.count) {
      rc = rpgo_get_estimate(s, keys.data(), poses, c.num_values);
    } else {
      std::vector<double> tmp((size_t)c.num_values * stride);
      rc = rpgo_get_estimate(s, keys.data(), tmp.data(), c.num_values);
      std::memcpy(poses, tmp.data(), sizeof(double) * (size_t)std::min<int64_t>(c.num_values, v.count) * stride);
    }
    if (rc == RPGO_OK && weights) {
      const int64_t nw = std::min<int64_t>(c.num_gnc_weights, f.count);
      std::vector<double> w((size_t)c.num_gnc_weights);
      rc = rpgo_get_gnc_weights(s, w.data(), c.num_gnc_weights);
      std::memcpy(weights, w.data(), sizeof(double) * (size_t)nw);
      if (num_weights) *num_weights = nw;
    } else if (num_weights) {
      *num_weights = 0;
    }
  }
  if (timing) rpgo_get_timing(s, timing);
  return rc;
}

void solve_one(const rpgo_params* p, const rpgo_factor_batch& f, const rpgo_value_batch& v, int ctas,
               double* poses, int64_t stride, double* weights, int64_t* num_weights, int32_t* status,
               rpgo_timing* timing) {
  rpgo_solver* s = rpgo_create(p);
  if (!s) {
    *status = RPGO_ERR_CUDA;
    return;
  }
  rpgo::set_coop_ctas(s, ctas);
  const int rc = rpgo_update(s, &f, &v, 1);
  *status = write_outputs(s, rc, f, v, poses, stride, weights, num_weights, timing);
  rpgo_destroy(s);
}

// the batch's pose dimension (all graphs share the parameters)
int batch_dim(const rpgo_params* p) {
  const int m = p->outlier_removal;
  return (m == RPGO_OUTLIER_PCM2D || m == RPGO_OUTLIER_PCM_SIMPLE2D) ? 2 : (m == RPGO_OUTLIER_NONE ? p->dim : 3);
}

// run work(i) for i in [0, n) on up to `threads` host threads
template <class Fn>
void parallel_for(int n, int threads, Fn&& work) {
  std::atomic<int> next{0};
  auto loop = [&] {
    for (int i; (i = next.fetch_add(1)) < n;) work(i);
  };
  const int nt = std::max(1, std::min(n, threads));
  std::vector<std::thread> pool;
  pool.reserve((size_t)nt - 1);
  for (int t = 1; t < nt; ++t) pool.emplace_back(loop);
  loop();
  for (auto& t : pool) t.join();
}

}  // namespace

extern "C" int rpgo_solve_batch(const rpgo_params* p, int32_t n, const rpgo_factor_batch* factors,
                                const rpgo_value_batch* values, int32_t workers, int32_t coop_ctas,
                                rpgo_batch_out* out) {
  if (!p || n < 0 || (n > 0 && (!factors || !values || !out || !out->poses || !out->status))) return RPGO_ERR_ARG;
  if (n == 0) return RPGO_OK;
  const int dim = batch_dim(p);
  const int64_t stride = dim == 3 ? 12 : 4;
  std::vector<int64_t> voff((size_t)n + 1, 0), foff((size_t)n + 1, 0);
  for (int g = 0; g < n; ++g) {
    voff[g + 1] = voff[g] + values[g].count;
    foff[g + 1] = foff[g] + factors[g].count;
  }
  int sms = 0;
  try {
    sms = rpgo::device_sm_count();
  } catch (const rpgo::CudaError&) {
    return RPGO_ERR_CUDA;
  }
  const int nw = std::max(1, std::min<int>(workers > 0 ? workers : kDefaultWorkers, n));
  const int ctas = coop_ctas > 0 ? coop_ctas : std::max(1, kCholCtasPerSm * sms / nw);
  std::atomic<int> next{0};
  auto work = [&] {
    for (;;) {
      const int g = next.fetch_add(1);
      if (g >= n) break;
      solve_one(p, factors[g], values[g], ctas, out->poses + voff[g] * stride, stride,
                out->gnc_weights ? out->gnc_weights + foff[g] : nullptr,
                out->num_weights ? out->num_weights + g : nullptr, out->status + g,
                out->timing ? out->timing + g : nullptr);
    }
  };
  std::vector<std::thread> pool;
  pool.reserve((size_t)nw - 1);
  for (int t = 1; t < nw; ++t) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  return RPGO_OK;
}

extern "C" int rpgo_solve_batch_joint(const rpgo_params* p, int32_t n, const rpgo_factor_batch* factors,
                                      const rpgo_value_batch* values, int32_t group, int32_t streams,
                                      rpgo_batch_out* out) {
  if (!p || n < 0 || (n > 0 && (!factors || !values || !out || !out->poses || !out->status))) return RPGO_ERR_ARG;
  if (n == 0) return RPGO_OK;
  const int dim = batch_dim(p);
  const int64_t stride = dim == 3 ? 12 : 4;
  std::vector<int64_t> voff((size_t)n + 1, 0), foff((size_t)n + 1, 0);
  for (int g = 0; g < n; ++g) {
    voff[g + 1] = voff[g] + values[g].count;
    foff[g + 1] = foff[g] + factors[g].count;
  }
  // host threads of the per-graph stages: they mostly wait on their own
  // streams' short kernels, so more threads than cores keep the GPU busier
  const int threads = std::min<int>(n, kJointHostThreads);
  // 1. every graph's PCM (and classification) on its own solver, concurrently
  std::vector<rpgo_solver*> sv((size_t)n, nullptr);
  std::vector<int> rc((size_t)n, RPGO_OK), kind((size_t)n, rpgo::kJointNone);
  std::vector<rpgo::JointProblem> jp((size_t)n);
  std::vector<double> solve_ms((size_t)n, 0.0);
  parallel_for(n, threads, [&](int g) {
    sv[g] = rpgo_create(p);
    if (!sv[g]) {
      rc[g] = RPGO_ERR_CUDA;
      return;
    }
    rc[g] = rpgo_update(sv[g], &factors[g], &values[g], 0);
    if (rc[g] != RPGO_OK) return;
    try {
      kind[g] = rpgo::joint_prepare(sv[g], &jp[g]);
    } catch (const std::exception& e) {
      std::fprintf(stderr, "rpgo_solve_batch_joint: graph %d: %s\n", g, e.what());
      rc[g] = RPGO_ERR_CUDA;
    }
  });
  // 2. graphs that need their solver's own path
  parallel_for(n, threads, [&](int g) {
    if (rc[g] == RPGO_OK && kind[g] == rpgo::kJointOwn) {
      try {
        rc[g] = rpgo::joint_optimize_own(sv[g], &solve_ms[g]);
      } catch (const std::exception& e) {
        std::fprintf(stderr, "rpgo_solve_batch_joint: graph %d: %s\n", g, e.what());
        rc[g] = RPGO_ERR_CUDA;
      }
    }
  });
  // 3. the rest in lock-step groups of graphs of similar size (similar
  // numbers of rounds), several groups concurrently, each on its own stream
  // and a share of the SMs for its direct solve
  std::vector<int> joint;
  for (int g = 0; g < n; ++g)
    if (rc[g] == RPGO_OK && kind[g] == rpgo::kJointSolve) joint.push_back(g);
  std::stable_sort(joint.begin(), joint.end(), [&](int a, int b) { return values[a].count > values[b].count; });
  const int nj = (int)joint.size();
  const int ns = std::max(1, std::min(nj, streams > 0 ? (int)streams : kDefaultJointStreams));
  const int gsz = group > 0 ? (int)group : std::max(1, (nj + ns - 1) / ns);
  const int ngroups = nj > 0 ? (nj + gsz - 1) / gsz : 0;
  int sms = 0;
  try {
    sms = rpgo::device_sm_count();
  } catch (const rpgo::CudaError&) {
    for (int g : joint) rc[g] = RPGO_ERR_CUDA;
  }
  const int conc = std::min(ns, std::max(1, ngroups));
  const int ctas = conc > 1 ? std::max(1, kCholCtasPerSm * sms / conc) : 0;
  parallel_for(sms > 0 ? ngroups : 0, conc, [&](int k) {
    const int b0 = k * gsz, b1 = std::min(nj, b0 + gsz);
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      for (int i = b0; i < b1; ++i) rc[joint[i]] = RPGO_ERR_CUDA;
      return;
    }
    std::vector<rpgo::JointProblem*> probs;
    for (int i = b0; i < b1; ++i) probs.push_back(&jp[joint[i]]);
    try {
      const auto t0 = std::chrono::steady_clock::now();
      rpgo::solve_joint(dim, probs, st, ctas);
      const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      for (int i = b0; i < b1; ++i) solve_ms[joint[i]] = ms;
    } catch (const std::exception& e) {
      std::fprintf(stderr, "rpgo_solve_batch_joint: group of %d graphs failed: %s\n", b1 - b0, e.what());
      for (int i = b0; i < b1; ++i) rc[joint[i]] = RPGO_ERR_CUDA;
    }
    cudaStreamDestroy(st);
  });
  // 4. bookkeeping and outputs
  parallel_for(n, threads, [&](int g) {
    if (!sv[g]) {
      out->status[g] = rc[g];
      return;
    }
    if (rc[g] == RPGO_OK && kind[g] == rpgo::kJointSolve) rc[g] = rpgo::joint_commit(sv[g], jp[g], solve_ms[g]);
    out->status[g] = write_outputs(sv[g], rc[g], factors[g], values[g], out->poses + voff[g] * stride, stride,
                                   out->gnc_weights ? out->gnc_weights + foff[g] : nullptr,
                                   out->num_weights ? out->num_weights + g : nullptr,
                                   out->timing ? out->timing + g : nullptr);
    rpgo_destroy(sv[g]);
  });
  return RPGO_OK;
}

extern "C" int32_t rpgo_set_joint_graphs(int32_t on) { return rpgo::set_joint_graphs(on != 0) ? 1 : 0; }

extern "C" int64_t rpgo_joint_graph_rounds(void) { return rpgo::joint_graph_rounds(); }

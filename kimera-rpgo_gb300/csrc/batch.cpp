// Batched solve of independent graphs (rpgo_solve_batch, include/rpgo_gb300.h).
//
// Each graph is an ordinary rpgo_solver (RobustSolver look-alike) on its own
// non-blocking stream; `workers` host threads take graphs from a shared
// counter. The GPU runs the workers' kernels concurrently: the per-graph
// kernels of PCM (trajectory scan, odometry and pairwise checks, clique) are
// small, latency-bound launches, and each cooperative direct solve is limited
// to `coop_ctas` CTAs so that several fit on the device at once. Device memory
// is stream-ordered (no device-wide synchronisation on free), so the workers
// do not serialise each other.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/rpgo_gb300.h"
#include "common.cuh"

namespace rpgo {
void set_coop_ctas(rpgo_solver* s, int ctas);
}

namespace {

constexpr int kDefaultWorkers = 16;
// co-resident CTAs of the direct solve per SM (256 threads x 128 registers)
constexpr int kCholCtasPerSm = 2;

void solve_one(const rpgo_params* p, const rpgo_factor_batch& f, const rpgo_value_batch& v, int ctas,
               double* poses, int64_t stride, double* weights, int64_t* num_weights, int32_t* status,
               rpgo_timing* timing) {
  rpgo_solver* s = rpgo_create(p);
  if (!s) {
    *status = RPGO_ERR_CUDA;
    return;
  }
  rpgo::set_coop_ctas(s, ctas);
  int rc = rpgo_update(s, &f, &v, 1);
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
  *status = rc;
  rpgo_destroy(s);
}

}  // namespace

extern "C" int rpgo_solve_batch(const rpgo_params* p, int32_t n, const rpgo_factor_batch* factors,
                                const rpgo_value_batch* values, int32_t workers, int32_t coop_ctas,
                                rpgo_batch_out* out) {
  if (!p || n < 0 || (n > 0 && (!factors || !values || !out || !out->poses || !out->status))) return RPGO_ERR_ARG;
  if (n == 0) return RPGO_OK;
  const int m = p->outlier_removal;
  const int dim = (m == RPGO_OUTLIER_PCM2D || m == RPGO_OUTLIER_PCM_SIMPLE2D) ? 2 : (m == RPGO_OUTLIER_NONE ? p->dim : 3);
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

// Nonlinear least-squares kernels of the robust solve (sm_103a).
//
//  K4 linearise      FP64 residual and exact Jacobians (BetweenFactor /
//                    PriorFactor as GTSAM evaluates them), whitened by
//                    sqrt(w) R; FP64 gradient and Hessian blocks (J_i^T J_i,
//                    J_j^T J_j, J_i^T J_j), plus an FP32 copy of the Hessian
//                    blocks for the PCG preconditioner. Phase A one thread
//                    per factor (residual, Logmap derivative, adjoint), phase
//                    B d lanes per factor (the Jacobian and Hessian products,
//                    one row each).
//  assemble          one thread per variable, fixed factor order (no atomics,
//                    run-to-run deterministic): diagonal blocks, gradient, the
//                    odometry-chain preconditioner blocks and the damping
//                    diagonal clamp(diag H, 1e-6, 1e32) (LM diagonalDamping).
//  K5 linear solve   (H + lambda D) delta = -g. Default: the direct sparse
//                    Cholesky of chol_kernels.cu (FP64, one cooperative
//                    kernel per solve). Here: the alternative whole-GPU
//                    flexible PCG in FP64 (k_pcg_coop) with an FP32 block
//                    cyclic-reduction preconditioner of the odometry chain,
//                    used on request or when the factor would not fit the
//                    memory budget; both also give the linearised cost change
//                    -g.d - d^T H d / 2 (FP64, undamped H).
//  retract / error   X <- X Expmap(delta); per-factor 0.5 w |R e|^2 (FP64).
//  K6 GNC weights    TLS weights of GncOptimizer::calculateWeights (FP64).
#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <exception>
#include <thread>

#include "chol.hpp"
#include "solver_kernels.hpp"
#include "solver_math.cuh"

namespace rpgo {
namespace {

using namespace sm;

// device memory the direct solver's factor may take before the PCG path is used
constexpr double kCholBudgetBytes = 32.0 * (1 << 30);
// Fill-in guard: factorisations above this many flops (about 30 ms of the
// direct kernel) race the two solvers on the first damped system. Measured
// on GB300, 20,000 poses, GNC alone: 8,000 closures, 40 % outliers half
// clustered: direct 170 ms / PCG 374 ms per system (5.3e10 flops); 5,600
// inliers + 2,400 uniform outliers: direct 264 ms / PCG 78 ms (9.2e10).
std::atomic<double> g_guard_flops{1e10};
std::atomic<int> g_guard_prefer{0};

bool use_direct(const SolverDev& s) { return s.chol && !s.pcg_chosen; }
// the PCG path's assembly (FP32 blocks, chain preconditioner) is needed
bool need_pcg(const SolverDev& s) { return !use_direct(s) || s.race; }

// ------------------------------------------------------------------ errors
template <int DIM>
__global__ void k_factor_err(int F, const int32_t* __restrict__ kind, const int32_t* __restrict__ vi,
                             const int32_t* __restrict__ vj, const double* __restrict__ z,
                             const double* __restrict__ R, const double* __restrict__ x,
                             const double* __restrict__ w, double* __restrict__ ferr,
                             const uint8_t* __restrict__ mask = nullptr, uint8_t bit = 0) {
  using L = SLie<DIM>;
  constexpr int d = L::d, st = L::stride;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F || (mask && !(mask[f] & bit))) return;
  typename L::Pose Xi, Z, rel;
  L::load(x + (size_t)vi[f] * st, Xi);
  L::load(z + (size_t)f * st, Z);
  double e[d];
  if (kind[f] == 0) {
    typename L::Pose Xj, h;
    L::load(x + (size_t)vj[f] * st, Xj);
    L::between(Xi, Xj, h);
    L::between(Z, h, rel);
  } else {
    L::between(Xi, Z, rel);
  }
  L::logmap(rel, e);
  const double* Rf = R + (size_t)f * d * d;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < d; ++i) {
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < d; ++k) acc += Rf[d * i + k] * e[k];
    s += acc * acc;
  }
  ferr[f] = 0.5 * (w ? w[f] : 1.0) * s;
}

// Per-factor errors at x and their sum in one launch: each block sums its
// grid-stride share (fixed tree order) into part[block]; the last block to
// finish (ticket counter, reset for the next launch) adds the partials in
// block order into *sum, so the result does not depend on scheduling.
// The error sum runs on blocks of two warps, so that its ~F/32 warps spread
// over the SMs (one per FP64 sub-partition) instead of crowding a few.
constexpr int kErrThreads = 64;

template <int DIM>
__global__ void __launch_bounds__(kErrThreads) k_factor_err_sum(int F, const int32_t* __restrict__ kind,
                                                        const int32_t* __restrict__ vi,
                                                        const int32_t* __restrict__ vj, const double* __restrict__ z,
                                                        const double* __restrict__ R, const double* __restrict__ x,
                                                        const double* __restrict__ w, double* __restrict__ part,
                                                        unsigned int* __restrict__ ticket, double* __restrict__ sum) {
  using L = SLie<DIM>;
  constexpr int d = L::d, st = L::stride;
  __shared__ double sh[kErrThreads];
  __shared__ bool last;
  double acc = 0.0;
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < F; f += gridDim.x * blockDim.x) {
    typename L::Pose Xi, Z, rel;
    L::load(x + (size_t)vi[f] * st, Xi);
    L::load(z + (size_t)f * st, Z);
    double e[d];
    if (kind[f] == 0) {
      typename L::Pose Xj, h;
      L::load(x + (size_t)vj[f] * st, Xj);
      L::between(Xi, Xj, h);
      L::between(Z, h, rel);
    } else {
      L::between(Xi, Z, rel);
    }
    L::logmap(rel, e);
    const double* Rf = R + (size_t)f * d * d;
    double s2 = 0.0;
#pragma unroll
    for (int i = 0; i < d; ++i) {
      double a = 0.0;
#pragma unroll
      for (int k = 0; k < d; ++k) a += Rf[d * i + k] * e[k];
      s2 += a * a;
    }
    acc += 0.5 * (w ? w[f] : 1.0) * s2;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kErrThreads / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sh[0];
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    // the last block adds the block sums: thread t takes t, t + 64, ... in
    // order, then a fixed tree (the same order for the same grid)
    __threadfence();
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kErrThreads) t += ((volatile double*)part)[b];
    sh[threadIdx.x] = t;
    __syncthreads();
    for (int o = kErrThreads / 2; o; o >>= 1) {
      if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      *sum = sh[0];
      *ticket = 0u;
    }
  }
}

__global__ void k_sum_partial(int n, const double* __restrict__ in, double* __restrict__ out) {
  __shared__ double sh[256];
  double v = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v += in[i];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = 128; s; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

double device_sum(const double* in, int n, DeviceBuffer<double>& red, cudaStream_t st) {
  if (n <= 0) return 0.0;
  const int blocks = std::min(256, div_up(n, 256));
  red.resize(blocks + 1);
  k_sum_partial<<<blocks, 256, 0, st>>>(n, in, red.get());
  RPGO_LAUNCHED();
  k_sum_partial<<<1, 256, 0, st>>>(blocks, red.get(), red.get() + blocks);
  RPGO_LAUNCHED();
  double h = 0.0;
  RPGO_CUDA(cudaMemcpyAsync(&h, red.get() + blocks, sizeof(double), cudaMemcpyDeviceToHost, st));
  RPGO_CUDA(cudaStreamSynchronize(st));
  return h;
}

// ------------------------------------------------------------------ K4
// Linearisation of every factor at x (weights w): whitened residual
// r = sqrt(w) R e, Jacobians (between: J_i = -D Ad(h^-1), J_j = D; prior:
// J = I), gradient blocks A^T r and Hessian blocks Hii, Hjj, Hij in FP64 and
// an FP32 copy. A between factor forms only A_j = sqrt(w) R D: since
// A_i = -A_j Ad, its blocks follow as Hjj = A_j^T A_j, Hij = -Ad^T Hjj,
// Hii = -Hij Ad and gi = -Ad^T gj (156 instead of 228 FMAs per lane). Two
// phases, the Jacobian products spread over d lanes per factor. Phase A, one thread per factor: the
// whitened residual r (times sqrt(w)), D = LogmapDerivative(e) and
// Ad(h^-1) into a per-factor record [r (d), D (dd), Ad (dd), sqrt(w)];
// for priors D and Ad are unused. Phase B, d lanes per factor (lane a owns
// row a): Ji = -D Ad, Ai = sqrt(w) R Ji, Aj = sqrt(w) R D through shared
// memory, then gradient entry a and row a of Hii, Hjj, Hij.
template <int DIM>
__global__ void __launch_bounds__(128) k_linearize_a(int F, const int32_t* __restrict__ kind,
                                                     const int32_t* __restrict__ vi, const int32_t* __restrict__ vj,
                                                     const double* __restrict__ z, const double* __restrict__ R,
                                                     const double* __restrict__ x, const double* __restrict__ w,
                                                     double* __restrict__ rec, const uint8_t* __restrict__ mask) {
  using L = SLie<DIM>;
  constexpr int d = L::d, st = L::stride, dd = d * d, RS = d + 2 * dd + 1;
  // Two warps per 32 factors (the FP64 chain of one thread is the cost, and
  // one thread per factor fills only about a quarter of the SM
  // sub-partitions; roles split by warp, not by lane, so that neither
  // role's instructions run with half the lanes idle): the role-0 warp forms
  // the residual, hands its log map to the role-1 warp through shared memory,
  // then forms the adjoint and the whitened residual; the role-1 warp forms
  // the log-map Jacobian.
  __shared__ double sh_e[2][32][d];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pair = warp >> 1, role = warp & 1;
  const int f = (blockIdx.x * 2 + pair) * 32 + lane;
  const bool valid = f < F && (!mask || (mask[f] & 1));
  const bool between = valid && kind[f] == 0;
  double* out = rec + (size_t)(valid ? f : 0) * RS;
  if (role == 0) {
    typename L::Pose h;
    double e[d];
#pragma unroll
    for (int i = 0; i < d; ++i) e[i] = 0.0;
    if (valid) {
      typename L::Pose Xi, Z, rel;
      L::load(x + (size_t)vi[f] * st, Xi);
      L::load(z + (size_t)f * st, Z);
      if (between) {
        typename L::Pose Xj;
        L::load(x + (size_t)vj[f] * st, Xj);
        L::between(Xi, Xj, h);
        L::between(Z, h, rel);
      } else {
        L::between(Xi, Z, rel);
      }
      L::logmap(rel, e);
    }
#pragma unroll
    for (int i = 0; i < d; ++i) sh_e[pair][lane][i] = e[i];
    // (named barrier 1 + pair of the warp pair: role 0 arrives, role 1 waits)
    asm volatile("bar.arrive %0, 64;" ::"r"(1 + pair) : "memory");
    if (!valid) return;
    if (between) {
      typename L::Pose hinv;
      double Ad[dd];
      L::inverse(h, hinv);
      L::adjoint(hinv, Ad);
#pragma unroll
      for (int i = 0; i < dd; ++i) out[d + dd + i] = Ad[i];
    } else {
#pragma unroll
      for (int i = 0; i < d; ++i) e[i] = -e[i];
    }
    const double sw = sqrt(w[f]);
    const double* Rf = R + (size_t)f * dd;
#pragma unroll
    for (int i = 0; i < d; ++i) {
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < d; ++k) acc += Rf[d * i + k] * e[k];
      out[i] = sw * acc;
    }
    out[d + 2 * dd] = sw;
  } else {
    asm volatile("bar.sync %0, 64;" ::"r"(1 + pair) : "memory");
    if (!between) return;
    double e[d], D[dd];
#pragma unroll
    for (int i = 0; i < d; ++i) e[i] = sh_e[pair][lane][i];
    L::dlog(e, D);
#pragma unroll
    for (int i = 0; i < dd; ++i) out[d + i] = D[i];
  }
}

template <int DIM>
__global__ void __launch_bounds__(128) k_linearize_b(int F, const int32_t* __restrict__ kind,
                                                     const double* __restrict__ R, const double* __restrict__ rec,
                                                     float* __restrict__ fH, double* __restrict__ fH64,
                                                     double* __restrict__ fg, const uint8_t* __restrict__ mask) {
  constexpr int d = (DIM == 3) ? 6 : 3, dd = d * d, RS = d + 2 * dd + 1;
  constexpr int per_warp = 32 / d;  // factors per warp
  constexpr int warps = 4;
  __shared__ double sA[warps][per_warp][dd], sH[warps][per_warp][dd], sg[warps][per_warp][d];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = lane / d, a = lane % d;
  const int f = (blockIdx.x * warps + warp) * per_warp + slot;
  const bool active = slot < per_warp && f < F && (!mask || (mask[f] & 1));
  const double* rc = rec + (size_t)(active ? f : 0) * RS;
  const double* Rf = R + (size_t)(active ? f : 0) * dd;
  const bool between = active && kind[f] == 0;
  double* Aj = sA[warp][active ? slot : 0];  // between: Aj = sqrt(w) R D; prior: Ai = sqrt(w) R
  double* Hs = sH[warp][active ? slot : 0];
  double* gs = sg[warp][active ? slot : 0];
  const double sw = active ? rc[d + 2 * dd] : 0.0;
  const double* r = rc;
  float* out = fH ? fH + (size_t)(active ? f : 0) * 3 * dd : nullptr;
  double* out64 = fH64 + (size_t)(active ? f : 0) * 3 * dd;
  double* og = fg + (size_t)(active ? f : 0) * 2 * d;
  // row a of A (Aj for a between factor, Ai for a prior); in 3D the log-map
  // derivative D and the adjoint have a zero upper-right 3x3 block, whose
  // terms are skipped (they add exact zeros)
  constexpr int zb = DIM == 3 ? 3 : 0;
  if (active) {
    const double* D = rc + d;
#pragma unroll
    for (int j = 0; j < d; ++j) {
      double acc = 0.0;
      if (between) {
#pragma unroll
        for (int k = (j >= zb && zb) ? zb : 0; k < d; ++k) acc += Rf[d * a + k] * D[d * k + j];
      } else {
        acc = Rf[d * a + j];
      }
      Aj[d * a + j] = sw * acc;
    }
  }
  __syncwarp();
  // H = A^T A (row a), g = A^T r (entry a): Hjj and gj of a between factor,
  // Hii and gi of a prior
  double h[d];
  double ga = 0.0;
  if (active) {
#pragma unroll
    for (int i = 0; i < d; ++i) ga += Aj[d * i + a] * r[i];
#pragma unroll
    for (int b = 0; b < d; ++b) {
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < d; ++q) acc += Aj[d * q + a] * Aj[d * q + b];
      h[b] = acc;
      Hs[d * a + b] = acc;
    }
    gs[a] = ga;
  }
  __syncwarp();
  if (!active) return;
  auto put = [&](int blk, int b, double v) {
    out64[blk * dd + d * a + b] = v;
    if (out) out[blk * dd + d * a + b] = (float)v;  // the FP32 copy feeds only the PCG path
  };
  if (!between) {
#pragma unroll
    for (int b = 0; b < d; ++b) {
      put(0, b, h[b]);
      put(1, b, 0.0);
      put(2, b, 0.0);
    }
    og[a] = ga;
    og[d + a] = 0.0;
    return;
  }
  // between: J_i = -D Ad, so A_i = -A_j Ad and Hij = A_i^T A_j = -Ad^T Hjj,
  // Hii = A_i^T A_i = -Hij Ad, gi = A_i^T r = -Ad^T gj
  const double* Ad = rc + d + dd;
  double hij[d];
  double gi = 0.0;
#pragma unroll
  for (int k = 0; k < d; ++k) gi += Ad[d * k + a] * gs[k];
#pragma unroll
  for (int b = 0; b < d; ++b) {
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < d; ++k) acc += Ad[d * k + a] * Hs[d * k + b];
    hij[b] = -acc;
  }
#pragma unroll
  for (int b = 0; b < d; ++b) {
    double acc = 0.0;
#pragma unroll
    for (int l = (b >= zb && zb) ? zb : 0; l < d; ++l) acc += hij[l] * Ad[d * l + b];
    put(0, b, -acc);
    put(1, b, h[b]);
    put(2, b, hij[b]);
  }
  og[a] = -gi;
  og[d + a] = ga;
}

template <int D>
__global__ void k_assemble(int N, const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc_fac,
                           const int8_t* __restrict__ inc_role, const int32_t* __restrict__ kind,
                           const int32_t* __restrict__ vi, const int32_t* __restrict__ vj,
                           const uint8_t* __restrict__ tree, const uint8_t* __restrict__ has_tree,
                           const double* __restrict__ fH64, const double* __restrict__ fg,
                           double* __restrict__ Hd64, float* __restrict__ Hd, float* __restrict__ Md,
                           float* __restrict__ Mu, double* __restrict__ g, double* __restrict__ dampD,
                           int diag_damping) {
  constexpr int dd = D * D;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= N) return;
  double H[dd], M[dd], U[dd];
  double gv[D];
#pragma unroll
  for (int i = 0; i < dd; ++i) H[i] = M[i] = U[i] = 0.0;
#pragma unroll
  for (int i = 0; i < D; ++i) gv[i] = 0.0;
  for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
    const int f = inc_fac[k];
    const int role = inc_role[k];
    const double* blk = fH64 + (size_t)f * 3 * dd + (role == 1 ? dd : 0);
    const bool in_m = kind[f] == 1 || tree[f];
#pragma unroll
    for (int i = 0; i < dd; ++i) {
      const double b = blk[i];
      H[i] += b;
      if (in_m) M[i] += b;
    }
    const double* gg = fg + (size_t)f * 2 * D + role * D;
#pragma unroll
    for (int i = 0; i < D; ++i) gv[i] += gg[i];
    if (tree[f]) {
      const int other = role == 0 ? vj[f] : vi[f];
      if (other == v + 1) {
        const double* hij = fH64 + (size_t)f * 3 * dd + 2 * dd;
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
          for (int b = 0; b < D; ++b) U[D * a + b] += (role == 0) ? hij[D * a + b] : hij[D * b + a];
      }
    }
  }
  if (!has_tree[v]) {
#pragma unroll
    for (int i = 0; i < dd; ++i) M[i] = H[i];
  }
#pragma unroll
  for (int i = 0; i < dd; ++i) {
    Hd64[(size_t)v * dd + i] = H[i];
    Hd[(size_t)v * dd + i] = (float)H[i];
    Md[(size_t)v * dd + i] = (float)M[i];
    Mu[(size_t)v * dd + i] = (float)U[i];
  }
#pragma unroll
  for (int i = 0; i < D; ++i) {
    g[(size_t)v * D + i] = gv[i];
    dampD[(size_t)v * D + i] = diag_damping ? fmin(fmax(H[D * i + i], 1e-6), 1e32) : 1.0;
  }
}

// Assembly for the direct solver: one warp per variable, lane e owning the
// block entries e and e + 32 (and gradient entry e < D); the same sums in the
// same factor order as k_assemble (identical FP64 results), without the FP32
// preconditioner blocks, which only the PCG path reads.
template <int D>
__global__ void k_assemble_direct(int N, const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc_fac,
                                  const int8_t* __restrict__ inc_role, const double* __restrict__ fH64,
                                  const double* __restrict__ fg, double* __restrict__ Hd64, double* __restrict__ g,
                                  double* __restrict__ dampD, int diag_damping, const uint8_t* __restrict__ mask) {
  constexpr int dd = D * D;
  const int v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (v >= N || (mask && !(mask[v] & 1))) return;
  const int e0 = lane, e1 = lane + 32;
  double h0 = 0.0, h1 = 0.0, gv = 0.0;
  for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
    const int f = inc_fac[k];
    const int role = inc_role[k];
    const double* blk = fH64 + (size_t)f * 3 * dd + (role == 1 ? dd : 0);
    if (e0 < dd) h0 += blk[e0];
    if (e1 < dd) h1 += blk[e1];
    if (lane < D) gv += fg[(size_t)f * 2 * D + role * D + lane];
  }
  if (e0 < dd) Hd64[(size_t)v * dd + e0] = h0;
  if (e1 < dd) Hd64[(size_t)v * dd + e1] = h1;
  if (lane < D) g[(size_t)v * D + lane] = gv;
  // diagonal entries: e = D i + i
  if (e0 < dd && e0 % (D + 1) == 0)
    dampD[(size_t)v * D + e0 / (D + 1)] = diag_damping ? fmin(fmax(h0, 1e-6), 1e32) : 1.0;
  if (e1 < dd && e1 % (D + 1) == 0)
    dampD[(size_t)v * D + e1 / (D + 1)] = diag_damping ? fmin(fmax(h1, 1e-6), 1e32) : 1.0;
}

// ------------------------------------------------------------------ small dense (FP32)
template <int D>
__device__ bool chol_f(const float* A, float* L) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      float acc = A[D * i + j];
#pragma unroll
      for (int k = 0; k < j; ++k) acc -= L[D * i + k] * L[D * j + k];
      if (i == j) {
        if (!(acc > 0.f)) return false;
        L[D * i + i] = sqrtf(acc);
      } else {
        L[D * i + j] = acc / L[D * j + j];
      }
    }
  return true;
}
// SPD inverse; on a non-positive pivot, retries with a diagonal shift and
// finally falls back to the inverse diagonal.
template <int D>
__device__ void spd_inv_f(const float* A, float* Ai) {
  float L[D * D], B[D * D];
#pragma unroll
  for (int i = 0; i < D * D; ++i) {
    B[i] = A[i];
    L[i] = 0.f;
  }
  bool ok = chol_f<D>(B, L);
  if (!ok) {
    float tr = 0.f;
#pragma unroll
    for (int i = 0; i < D; ++i) tr += fabsf(A[D * i + i]);
    const float eps = 1e-5f * (tr / D) + 1e-30f;
#pragma unroll
    for (int i = 0; i < D; ++i) B[D * i + i] += eps;
    ok = chol_f<D>(B, L);
  }
  if (!ok) {
#pragma unroll
    for (int i = 0; i < D * D; ++i) Ai[i] = 0.f;
#pragma unroll
    for (int i = 0; i < D; ++i) Ai[D * i + i] = 1.f / fmaxf(fabsf(A[D * i + i]), 1e-30f);
    return;
  }
  // Linv (lower)
  float Li[D * D];
#pragma unroll
  for (int i = 0; i < D * D; ++i) Li[i] = 0.f;
#pragma unroll
  for (int j = 0; j < D; ++j) {
    Li[D * j + j] = 1.f / L[D * j + j];
#pragma unroll
    for (int i = j + 1; i < D; ++i) {
      float acc = 0.f;
#pragma unroll
      for (int k = j; k < i; ++k) acc -= L[D * i + k] * Li[D * k + j];
      Li[D * i + j] = acc / L[D * i + i];
    }
  }
  // A^-1 = Li^T Li
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      float acc = 0.f;
#pragma unroll
      for (int k = i; k < D; ++k) acc += Li[D * k + i] * Li[D * k + j];
      Ai[D * i + j] = acc;
      Ai[D * j + i] = acc;
    }
}
template <int D>
__device__ __forceinline__ void mm_f(const float* A, const float* B, float* C, bool at = false, bool bt = false) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < D; ++k) acc += (at ? A[D * k + i] : A[D * i + k]) * (bt ? B[D * j + k] : B[D * k + j]);
      C[D * i + j] = acc;
    }
}

// ------------------------------------------------------------------ block reductions (one CTA)
__device__ __forceinline__ double cta_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[32] = v;
  }
  __syncthreads();
  const double r = sh[32];
  __syncthreads();
  return r;
}

struct CsrView {
  const float* Hd;
  const float* fH;
  const double* Hd64;
  const double* fH64;
  const int32_t* row_ptr;
  const int32_t* col;
  const int32_t* blk;
  const int8_t* btr;
  const double* dampD;
};

template <int DIM>
__global__ void k_retract(int N, const double* __restrict__ x, const double* __restrict__ delta,
                          double* __restrict__ xnew, const uint8_t* __restrict__ mask = nullptr) {
  using L = SLie<DIM>;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= N || (mask && !(mask[v] & 1))) return;
  typename L::Pose X, E, Y;
  L::load(x + (size_t)v * L::stride, X);
  L::exp(delta + (size_t)v * L::d, E);
  L::compose(X, E, Y);
  L::store(Y, xnew + (size_t)v * L::stride);
}

// GncOptimizer::calculateWeights, TLS branch (Yang et al. 2020, eq. 14)
__device__ __forceinline__ double tls_weight(double u, double b, double mu) {
  const double ub = (mu + 1.0) / mu * b;
  const double lb = mu / (mu + 1.0) * b;
  double wk = sqrt(b * mu * (mu + 1.0) / u) - mu;
  if (u >= ub || wk < 0.0) wk = 0.0;
  else if (u <= lb || wk > 1.0) wk = 1.0;
  return wk;
}
__global__ void k_gnc_weights(int F, int n_known, const double* __restrict__ u2, const double* __restrict__ barc,
                              double mu, double* __restrict__ w) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F) return;
  w[f] = f < n_known ? 1.0 : tls_weight(u2[f], barc[f], mu);
}

// ------------------------------------------------------------------ joint batch
// control word of each graph per variable and per factor
__global__ void k_batch_masks(int N, int F, const int32_t* __restrict__ vsys, const int32_t* __restrict__ fsys,
                              const uint8_t* __restrict__ ctl, uint8_t* __restrict__ vmask,
                              uint8_t* __restrict__ fmask) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) vmask[i] = ctl[vsys[i]];
  if (i < F) fmask[i] = ctl[fsys[i]];
}

// dst <- src on the rows (stride doubles) of the variables whose control word has `bit`
__global__ void k_batch_copy(int64_t n, int stride, const uint8_t* __restrict__ vmask, uint8_t bit,
                             const double* __restrict__ src, double* __restrict__ dst) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  if (vmask[e / stride] & bit) dst[e] = src[e];
}

// TLS weights of the factors of graphs with kBatchGnc, each graph with its
// own mu and known inliers (the first nknown factors of the graph)
__global__ void k_batch_gnc(int F, const int32_t* __restrict__ fsys, const int32_t* __restrict__ foff,
                            const int32_t* __restrict__ nknown, const uint8_t* __restrict__ fmask,
                            const double* __restrict__ u2, const double* __restrict__ barc,
                            const double* __restrict__ mu, double* __restrict__ w) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F || !(fmask[f] & kBatchGnc)) return;
  const int g = fsys[f];
  w[f] = f - foff[g] < nknown[g] ? 1.0 : tls_weight(u2[f], barc[f], mu[g]);
}

// per graph: the sum of vals over [off[g], off[g + 1]) for the graphs whose
// control word has `bit`; one warp per graph, lane-strided chains then a
// fixed tree (the order depends on the graph only)
__global__ void k_batch_sums(int G, const int32_t* __restrict__ off, const uint8_t* __restrict__ ctl, uint8_t bit,
                             const double* __restrict__ vals, double* __restrict__ out) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (g >= G || !(ctl[g] & bit)) return;  // (warp-uniform)
  double acc = 0.0;
  for (int i = off[g] + lane; i < off[g + 1]; i += 32) acc += vals[i];
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[g] = acc;
}

}  // namespace

// ------------------------------------------------------------------ host wrappers
void solver_upload(SolverDev& s, int dim, const std::vector<int32_t>& kind, const std::vector<int32_t>& vi,
                   const std::vector<int32_t>& vj, int N, cudaStream_t st, bool direct, CholPlan* given) {
  s.dim = dim;
  s.d = dim == 3 ? 6 : 3;
  s.stride = dim == 3 ? 12 : 4;
  s.N = N;
  s.F = (int)kind.size();
  const int d = s.d, dd = d * d, F = s.F;
  // the direct solve's plan (host work only) is built on its own thread while
  // the lists below are built and uploaded
  CholPlan plan;
  std::exception_ptr plan_err;
  struct Joiner {
    std::thread t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } planner;
  if (direct && N > 0 && !given)
    planner.t = std::thread([&] {
      try {
        plan = make_chol_plan(N, d, kind, vi, vj);
      } catch (...) {
        plan_err = std::current_exception();
      }
    });
  std::vector<uint8_t> tree(F, 0), has_tree(N, 0);
  std::vector<int32_t> deg(N + 1, 0);
  for (int f = 0; f < F; ++f) {
    if (kind[f] == 0 && std::abs(vi[f] - vj[f]) == 1) {
      tree[f] = 1;
      has_tree[vi[f]] = has_tree[vj[f]] = 1;
    }
    deg[vi[f] + 1]++;
    if (kind[f] == 0 && vj[f] != vi[f]) deg[vj[f] + 1]++;
  }
  std::vector<int32_t> inc_ptr(N + 1, 0);
  for (int v = 0; v < N; ++v) inc_ptr[v + 1] = inc_ptr[v] + deg[v + 1];
  std::vector<int32_t> inc_fac(inc_ptr[N]), fill(inc_ptr.begin(), inc_ptr.end() - 1);
  std::vector<int8_t> inc_role(inc_ptr[N]);
  for (int f = 0; f < F; ++f) {
    inc_fac[fill[vi[f]]] = f;
    inc_role[fill[vi[f]]++] = 0;
    if (kind[f] == 0 && vj[f] != vi[f]) {
      inc_fac[fill[vj[f]]] = f;
      inc_role[fill[vj[f]]++] = 1;
    }
  }
  // SpMV rows: off-diagonal blocks of between factors
  std::vector<int32_t> rdeg(N + 1, 0);
  for (int f = 0; f < F; ++f)
    if (kind[f] == 0 && vi[f] != vj[f]) {
      rdeg[vi[f] + 1]++;
      rdeg[vj[f] + 1]++;
    }
  std::vector<int32_t> row_ptr(N + 1, 0);
  for (int v = 0; v < N; ++v) row_ptr[v + 1] = row_ptr[v] + rdeg[v + 1];
  std::vector<int32_t> col(row_ptr[N]), blk(row_ptr[N]), rf(row_ptr.begin(), row_ptr.end() - 1);
  std::vector<int8_t> btr(row_ptr[N]);
  for (int f = 0; f < F; ++f)
    if (kind[f] == 0 && vi[f] != vj[f]) {
      int k = rf[vi[f]]++;
      col[k] = vj[f];
      blk[k] = f;
      btr[k] = 0;
      k = rf[vj[f]]++;
      col[k] = vi[f];
      blk[k] = f;
      btr[k] = 1;
    }
  s.kind.upload(kind, st);
  s.vi.upload(vi, st);
  s.vj.upload(vj, st);
  s.tree.upload(tree, st);
  s.var_has_tree.upload(has_tree, st);
  s.z.resize((size_t)F * s.stride);
  s.sqrt_info.resize((size_t)F * dd);
  s.inc_ptr.upload(inc_ptr, st);
  s.inc_fac.upload(inc_fac, st);
  s.inc_role.upload(inc_role, st);
  s.row_ptr.upload(row_ptr, st);
  s.col.upload(col, st);
  s.blk.upload(blk, st);
  s.btr.upload(btr, st);
  s.x0.resize((size_t)N * s.stride);
  s.x.resize((size_t)N * s.stride);
  s.xnew.resize((size_t)N * s.stride);
  s.weights.resize(F);
  s.fH.resize((size_t)F * 3 * dd);
  s.fH64.resize((size_t)F * 3 * dd);
  s.fg.resize((size_t)F * 2 * d);
  s.ferr.resize(F);
  s.Hd.resize((size_t)N * dd);
  s.Hd64.resize((size_t)N * dd);
  s.Md.resize((size_t)N * dd);
  s.Mu.resize((size_t)N * dd);
  s.g.resize((size_t)N * d);
  s.dampD.resize((size_t)N * d);
  s.delta.resize((size_t)N * d);
  // cyclic reduction levels
  s.lvl_off.clear();
  s.lvl_n.clear();
  int n = N, off = 0;
  while (true) {
    s.lvl_off.push_back(off);
    s.lvl_n.push_back(n);
    off += n;
    if (n <= 1) break;
    n = (n + 1) / 2;
  }
  s.levels = (int)s.lvl_n.size();
  s.d_lvl_off.upload(s.lvl_off, st);
  s.d_lvl_n.upload(s.lvl_n, st);
  const size_t nodes = (size_t)off;
  s.bD.resize(nodes * dd);
  s.bDinv.resize(nodes * dd);
  s.bU.resize(nodes * dd);
  s.bFL.resize(nodes * dd);
  s.bFR.resize(nodes * dd);
  s.bb.resize(nodes * d);
  s.bx.resize(nodes * d);
  for (auto* b : {&s.cr, &s.cz, &s.cp, &s.cq, &s.cx}) b->resize((size_t)N * d);
  for (auto* b : {&s.r64, &s.z64, &s.zo64, &s.p64, &s.q64}) b->resize((size_t)N * d);
  s.out.resize(8);
  s.chol.reset();
  if (direct && N > 0) {
    if (planner.t.joinable()) planner.t.join();
    if (plan_err) std::rethrow_exception(plan_err);
    if (given) plan = std::move(*given);
    const double ntp = (double)plan.n_tiles * plan.tile;
    const double bytes = 8.0 * dd * (plan.n_blocks() + plan.n_sparse) + 8.0 * ntp * ntp +
                         4.0 * (plan.upd_src.size() + plan.tupd_src.size());
    if (bytes <= kCholBudgetBytes) {
      const double flops = plan.flops;
      s.chol = std::make_shared<CholDev>();
      s.chol->upload(std::move(plan), st);
      s.race = (!given && flops > g_guard_flops.load()) ? 1 : 0;
      s.pcg_chosen = false;
    }
  }
}

// enqueue k_factor_err_sum: the sum lands in s.red[blocks]
double* enqueue_error_sum(SolverDev& s, const double* x, const double* weights, cudaStream_t st) {
  const int blocks = std::min(1024, div_up(s.F, kErrThreads));
  if (s.ticket.size() == 0) {
    s.ticket.resize(1);
    s.ticket.zero(st);
  }
  s.red.resize(blocks + 1);
  if (s.dim == 3)
    k_factor_err_sum<3><<<blocks, kErrThreads, 0, st>>>(s.F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                s.sqrt_info.get(), x, weights, s.red.get(), s.ticket.get(),
                                                s.red.get() + blocks);
  else
    k_factor_err_sum<2><<<blocks, kErrThreads, 0, st>>>(s.F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                s.sqrt_info.get(), x, weights, s.red.get(), s.ticket.get(),
                                                s.red.get() + blocks);
  RPGO_LAUNCHED();
  return s.red.get() + blocks;
}

double solver_error(SolverDev& s, const double* x, const double* weights, cudaStream_t st) {
  if (s.F == 0) return 0.0;
  const double* sum = enqueue_error_sum(s, x, weights, st);
  double h = 0.0;
  RPGO_CUDA(cudaMemcpyAsync(&h, sum, sizeof(double), cudaMemcpyDeviceToHost, st));
  RPGO_CUDA(cudaStreamSynchronize(st));
  return h;
}

void solver_factor_errors(SolverDev& s, const double* x, std::vector<double>* out, cudaStream_t st) {
  out->assign(s.F, 0.0);
  if (s.F == 0) return;
  const int tb = 128;
  if (s.dim == 3)
    k_factor_err<3><<<div_up(s.F, tb), tb, 0, st>>>(s.F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                    s.sqrt_info.get(), x, nullptr, s.ferr.get());
  else
    k_factor_err<2><<<div_up(s.F, tb), tb, 0, st>>>(s.F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                    s.sqrt_info.get(), x, nullptr, s.ferr.get());
  RPGO_LAUNCHED();
  s.ferr.download(out->data(), s.F, st);
  RPGO_CUDA(cudaStreamSynchronize(st));
}

void solver_linearize(SolverDev& s, bool diagonal_damping, cudaStream_t st) {
  const int tb = 128;
  if (s.F > 0) {
    const int d = s.d, rs = d + 2 * d * d + 1;
    s.lin_rec.resize((size_t)s.F * rs);
    const int per_block = 4 * (32 / d);  // k_linearize_b: 4 warps of 32/d factors
    if (s.dim == 3) {
      k_linearize_a<3><<<div_up(s.F, 64), 128, 0, st>>>(s.F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                       s.sqrt_info.get(), s.x.get(), s.weights.get(), s.lin_rec.get(), nullptr);
      RPGO_LAUNCHED();
      k_linearize_b<3><<<div_up(s.F, per_block), 128, 0, st>>>(s.F, s.kind.get(), s.sqrt_info.get(), s.lin_rec.get(),
                                                               need_pcg(s) ? s.fH.get() : nullptr, s.fH64.get(),
                                                               s.fg.get(), nullptr);
    } else {
      k_linearize_a<2><<<div_up(s.F, 64), 128, 0, st>>>(s.F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                       s.sqrt_info.get(), s.x.get(), s.weights.get(), s.lin_rec.get(), nullptr);
      RPGO_LAUNCHED();
      k_linearize_b<2><<<div_up(s.F, per_block), 128, 0, st>>>(s.F, s.kind.get(), s.sqrt_info.get(), s.lin_rec.get(),
                                                               need_pcg(s) ? s.fH.get() : nullptr, s.fH64.get(),
                                                               s.fg.get(), nullptr);
    }
    RPGO_LAUNCHED();
  }
  if (use_direct(s)) {
    const int blocks = div_up((int64_t)s.N * 32, tb);
    if (s.dim == 3)
      k_assemble_direct<6><<<blocks, tb, 0, st>>>(s.N, s.inc_ptr.get(), s.inc_fac.get(), s.inc_role.get(),
                                                  s.fH64.get(), s.fg.get(), s.Hd64.get(), s.g.get(), s.dampD.get(),
                                                  diagonal_damping ? 1 : 0, nullptr);
    else
      k_assemble_direct<3><<<blocks, tb, 0, st>>>(s.N, s.inc_ptr.get(), s.inc_fac.get(), s.inc_role.get(),
                                                  s.fH64.get(), s.fg.get(), s.Hd64.get(), s.g.get(), s.dampD.get(),
                                                  diagonal_damping ? 1 : 0, nullptr);
    RPGO_LAUNCHED();
    chol_block_hessian(s, *s.chol, st);
    if (!s.race) return;
    // racing: the PCG path's blocks too (same FP64 diagonal, gradient and
    // damping as k_assemble_direct's)
  }
  if (s.dim == 3)
    k_assemble<6><<<div_up(s.N, tb), tb, 0, st>>>(s.N, s.inc_ptr.get(), s.inc_fac.get(), s.inc_role.get(),
                                                  s.kind.get(), s.vi.get(), s.vj.get(), s.tree.get(),
                                                  s.var_has_tree.get(), s.fH64.get(), s.fg.get(), s.Hd64.get(), s.Hd.get(),
                                                  s.Md.get(), s.Mu.get(), s.g.get(), s.dampD.get(),
                                                  diagonal_damping ? 1 : 0);
  else
    k_assemble<3><<<div_up(s.N, tb), tb, 0, st>>>(s.N, s.inc_ptr.get(), s.inc_fac.get(), s.inc_role.get(),
                                                  s.kind.get(), s.vi.get(), s.vj.get(), s.tree.get(),
                                                  s.var_has_tree.get(), s.fH64.get(), s.fg.get(), s.Hd64.get(), s.Hd.get(),
                                                  s.Md.get(), s.Mu.get(), s.g.get(), s.dampD.get(),
                                                  diagonal_damping ? 1 : 0);
  RPGO_LAUNCHED();
}

// ------------------------------------------------------------------ K5, whole-GPU form
// One cooperative launch (one CTA per SM, grid-wide barriers) runs the
// complete flexible PCG: FP64 vectors and FP64 block SpMV spread over every
// SM (GB300's FP64 rate per SM is a small fraction of its FP32 rate, so FP64
// work must use all SMs), the block cyclic reduction preconditioner in FP32
// with the large levels spread over the grid and the small top levels done by
// CTA 0 alone. All branch decisions come from grid-reduced values every CTA
// reads after the same barrier, so every CTA passes the same barriers.
namespace cg = cooperative_groups;

struct CoopArgs {
  int N, levels, top;
  const int32_t* lvl_off;
  const int32_t* lvl_n;
  CsrView A;
  double lam;
  const double* g;
  const float* Md;
  const float* Mu;
  float *bD, *bDinv, *bU, *bFL, *bFR, *bb, *bx;
  double *r, *z, *zo, *p, *q, *delta;
  float* cr;
  double* part;  // 4 x gridDim.x
  double tol;
  int max_it;
  double* out;
};

__device__ __forceinline__ double grid_sum(double v, double* part, int slot, double* sh, cg::grid_group& grid) {
  v = cta_sum(v, sh);
  if (threadIdx.x == 0) part[slot * gridDim.x + blockIdx.x] = v;
  grid.sync();
  double t = 0.0;
  for (int b = 0; b < (int)gridDim.x; ++b) t += part[slot * gridDim.x + b];  // same order in every CTA
  return t;
}

template <int D>
__device__ void bcr_level_factor_odd(const CoopArgs& a, int l, int t0, int tstride) {
  constexpr int dd = D * D;
  const int base = a.lvl_off[l], n = a.lvl_n[l];
  for (int o = 1 + 2 * t0; o < n; o += 2 * tstride)
    spd_inv_f<D>(a.bD + (size_t)(base + o) * dd, a.bDinv + (size_t)(base + o) * dd);
}
template <int D>
__device__ void bcr_level_factor_even(const CoopArgs& a, int l, int t0, int tstride) {
  constexpr int dd = D * D;
  const int base = a.lvl_off[l], n = a.lvl_n[l], nbase = a.lvl_off[l + 1];
  for (int i = 2 * t0; i < n; i += 2 * tstride) {
    float FL[dd], FR[dd], Dn[dd], T[dd], Un[dd];
    const float* Di = a.bD + (size_t)(base + i) * dd;
#pragma unroll
    for (int k = 0; k < dd; ++k) {
      Dn[k] = Di[k];
      Un[k] = 0.f;
      FL[k] = 0.f;
      FR[k] = 0.f;
    }
    if (i >= 1) {
      const float* Ul = a.bU + (size_t)(base + i - 1) * dd;
      mm_f<D>(Ul, a.bDinv + (size_t)(base + i - 1) * dd, FL, true, false);
      mm_f<D>(FL, Ul, T);
#pragma unroll
      for (int k = 0; k < dd; ++k) Dn[k] -= T[k];
    }
    if (i + 1 < n) {
      const float* Ur = a.bU + (size_t)(base + i) * dd;
      mm_f<D>(Ur, a.bDinv + (size_t)(base + i + 1) * dd, FR);
      mm_f<D>(FR, Ur, T, false, true);
#pragma unroll
      for (int k = 0; k < dd; ++k) Dn[k] -= T[k];
      if (i + 2 < n) {
        mm_f<D>(FR, a.bU + (size_t)(base + i + 1) * dd, T);
#pragma unroll
        for (int k = 0; k < dd; ++k) Un[k] = -T[k];
      }
    }
#pragma unroll
    for (int x = 0; x < D; ++x)
#pragma unroll
      for (int y = 0; y < x; ++y) {
        const float sv = 0.5f * (Dn[D * x + y] + Dn[D * y + x]);
        Dn[D * x + y] = sv;
        Dn[D * y + x] = sv;
      }
#pragma unroll
    for (int k = 0; k < dd; ++k) {
      a.bFL[(size_t)(base + i) * dd + k] = FL[k];
      a.bFR[(size_t)(base + i) * dd + k] = FR[k];
      a.bD[(size_t)(nbase + i / 2) * dd + k] = Dn[k];
      a.bU[(size_t)(nbase + i / 2) * dd + k] = Un[k];
    }
  }
}

template <int D>
__global__ void __launch_bounds__(256) k_bcr_factor_coop(CoopArgs a) {
  cg::grid_group grid = cg::this_grid();
  constexpr int dd = D * D;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  for (int v = gt; v < a.N; v += gs) {
#pragma unroll
    for (int k = 0; k < dd; ++k) {
      a.bD[(size_t)v * dd + k] = a.Md[(size_t)v * dd + k];
      a.bU[(size_t)v * dd + k] = (v + 1 < a.N) ? a.Mu[(size_t)v * dd + k] : 0.f;
    }
#pragma unroll
    for (int x = 0; x < D; ++x) a.bD[(size_t)v * dd + D * x + x] += (float)(a.lam * a.A.dampD[(size_t)v * D + x]);
  }
  grid.sync();
  for (int l = 0; l < a.top; ++l) {
    bcr_level_factor_odd<D>(a, l, gt, gs);
    grid.sync();
    bcr_level_factor_even<D>(a, l, gt, gs);
    grid.sync();
  }
  if (blockIdx.x == 0) {
    for (int l = a.top; l < a.levels; ++l) {
      const int n = a.lvl_n[l];
      if (n == 1) {
        if (threadIdx.x == 0) spd_inv_f<D>(a.bD + (size_t)a.lvl_off[l] * dd, a.bDinv + (size_t)a.lvl_off[l] * dd);
        break;
      }
      bcr_level_factor_odd<D>(a, l, threadIdx.x, blockDim.x);
      __syncthreads();
      bcr_level_factor_even<D>(a, l, threadIdx.x, blockDim.x);
      __syncthreads();
    }
  }
}

template <int D>
__device__ __forceinline__ float* lvl_b(const CoopArgs& a, int l) {
  return l == 0 ? a.cr : a.bb + (size_t)a.lvl_off[l] * D;
}
template <int D>
__device__ void bcr_fwd_level(const CoopArgs& a, int l, int t0, int ts) {
  constexpr int dd = D * D;
  const int base = a.lvl_off[l], n = a.lvl_n[l];
  const float* b = lvl_b<D>(a, l);
  float* bn = lvl_b<D>(a, l + 1);
  for (int i = 2 * t0; i < n; i += 2 * ts) {
    float o[D];
#pragma unroll
    for (int x = 0; x < D; ++x) o[x] = b[(size_t)i * D + x];
    if (i >= 1) {
      const float* F = a.bFL + (size_t)(base + i) * dd;
#pragma unroll
      for (int x = 0; x < D; ++x)
#pragma unroll
        for (int c = 0; c < D; ++c) o[x] -= F[D * x + c] * b[(size_t)(i - 1) * D + c];
    }
    if (i + 1 < n) {
      const float* F = a.bFR + (size_t)(base + i) * dd;
#pragma unroll
      for (int x = 0; x < D; ++x)
#pragma unroll
        for (int c = 0; c < D; ++c) o[x] -= F[D * x + c] * b[(size_t)(i + 1) * D + c];
    }
#pragma unroll
    for (int x = 0; x < D; ++x) bn[(size_t)(i / 2) * D + x] = o[x];
  }
}
// backward level l: x_l from x_{l+1}; at level 0 also writes z (FP64)
template <int D>
__device__ void bcr_bwd_level(const CoopArgs& a, int l, int t0, int ts) {
  constexpr int dd = D * D;
  const int base = a.lvl_off[l], n = a.lvl_n[l], nbase = a.lvl_off[l + 1];
  const float* b = lvl_b<D>(a, l);
  for (int i = t0; i < n; i += ts) {
    float o[D];
    if ((i & 1) == 0) {
#pragma unroll
      for (int x = 0; x < D; ++x) o[x] = a.bx[(size_t)(nbase + i / 2) * D + x];
    } else {
      const float* Di = a.bDinv + (size_t)(base + i) * dd;
#pragma unroll
      for (int x = 0; x < D; ++x) {
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < D; ++c) acc += Di[D * x + c] * b[(size_t)i * D + c];
        o[x] = acc;
      }
      {
        const float* F = a.bFR + (size_t)(base + i - 1) * dd;
        const float* xl = a.bx + (size_t)(nbase + (i - 1) / 2) * D;
#pragma unroll
        for (int x = 0; x < D; ++x)
#pragma unroll
          for (int c = 0; c < D; ++c) o[x] -= F[D * c + x] * xl[c];
      }
      if (i + 1 < n) {
        const float* F = a.bFL + (size_t)(base + i + 1) * dd;
        const float* xr = a.bx + (size_t)(nbase + (i + 1) / 2) * D;
#pragma unroll
        for (int x = 0; x < D; ++x)
#pragma unroll
          for (int c = 0; c < D; ++c) o[x] -= F[D * c + x] * xr[c];
      }
    }
    if (l == 0) {
#pragma unroll
      for (int x = 0; x < D; ++x) a.z[(size_t)i * D + x] = (double)o[x];
    } else {
#pragma unroll
      for (int x = 0; x < D; ++x) a.bx[(size_t)(base + i) * D + x] = o[x];
    }
  }
}
// z = M^-1 r with r already in a.cr (all CTAs must call)
template <int D>
__device__ void precond_grid(const CoopArgs& a, cg::grid_group& grid) {
  constexpr int dd = D * D;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  for (int l = 0; l < a.top; ++l) {
    bcr_fwd_level<D>(a, l, gt, gs);
    grid.sync();
  }
  if (blockIdx.x == 0) {
    int l = a.top;
    for (; l < a.levels && a.lvl_n[l] > 1; ++l) {
      bcr_fwd_level<D>(a, l, threadIdx.x, blockDim.x);
      __syncthreads();
    }
    const int base = a.lvl_off[l];
    const float* bc = lvl_b<D>(a, l);
    if (threadIdx.x < D) {
      const int x = threadIdx.x;
      float acc = 0.f;
      for (int c = 0; c < D; ++c) acc += a.bDinv[(size_t)base * dd + D * x + c] * bc[c];
      if (l == 0) a.z[x] = (double)acc;
      else a.bx[(size_t)base * D + x] = acc;
    }
    __syncthreads();
    for (--l; l >= a.top; --l) {
      bcr_bwd_level<D>(a, l, threadIdx.x, blockDim.x);
      __syncthreads();
    }
  }
  grid.sync();
  for (int l = a.top - 1; l >= 0; --l) {
    bcr_bwd_level<D>(a, l, gt, gs);
    grid.sync();
  }
}

template <int D>
__device__ void spmv_grid(const CsrView& A, int N, double lam, const double* p, double* y) {
  constexpr int dd = D * D;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  for (int v = gt; v < N; v += gs) {
    double acc[D];
    const double* H = A.Hd64 + (size_t)v * dd;
    const double* pv = p + (size_t)v * D;
#pragma unroll
    for (int x = 0; x < D; ++x) {
      double sacc = lam * A.dampD[(size_t)v * D + x] * pv[x];
#pragma unroll
      for (int c = 0; c < D; ++c) sacc += H[D * x + c] * pv[c];
      acc[x] = sacc;
    }
    for (int k = A.row_ptr[v]; k < A.row_ptr[v + 1]; ++k) {
      const double* B = A.fH64 + (size_t)A.blk[k] * 3 * dd + 2 * dd;
      const double* pc = p + (size_t)A.col[k] * D;
      if (A.btr[k]) {
#pragma unroll
        for (int x = 0; x < D; ++x)
#pragma unroll
          for (int c = 0; c < D; ++c) acc[x] += B[D * c + x] * pc[c];
      } else {
#pragma unroll
        for (int x = 0; x < D; ++x)
#pragma unroll
          for (int c = 0; c < D; ++c) acc[x] += B[D * x + c] * pc[c];
      }
    }
#pragma unroll
    for (int x = 0; x < D; ++x) y[(size_t)v * D + x] = acc[x];
  }
}

// out[0] lin_change, [1] ok, [2] iterations, [3] relative residual
template <int D>
__global__ void __launch_bounds__(256) k_pcg_coop(CoopArgs a) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double sh[40];
  const int n = a.N * D;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  double loc = 0.0;
  for (int k = gt; k < n; k += gs) {
    const double rk = -a.g[k];
    a.delta[k] = 0.0;
    a.r[k] = rk;
    a.cr[k] = (float)rk;
    loc += rk * rk;
  }
  const double bnorm = sqrt(grid_sum(loc, a.part, 0, sh, grid));
  int it = 0, ok = 1;
  double rel = 0.0;
  if (bnorm > 0.0) {
    precond_grid<D>(a, grid);
    loc = 0.0;
    for (int k = gt; k < n; k += gs) {
      a.p[k] = a.z[k];
      loc += a.r[k] * a.z[k];
    }
    double rz = grid_sum(loc, a.part, 1, sh, grid);  // also orders the p writes
    for (; it < a.max_it; ++it) {
      spmv_grid<D>(a.A, a.N, a.lam, a.p, a.q);
      grid.sync();
      loc = 0.0;
      for (int k = gt; k < n; k += gs) loc += a.p[k] * a.q[k];
      const double pq = grid_sum(loc, a.part, 2, sh, grid);
      if (!(pq > 0.0) || !(rz > 0.0)) {
        if (it == 0) ok = 0;
        break;
      }
      const double alpha = rz / pq;
      loc = 0.0;
      for (int k = gt; k < n; k += gs) {
        a.delta[k] += alpha * a.p[k];
        const double rk = a.r[k] - alpha * a.q[k];
        a.r[k] = rk;
        a.cr[k] = (float)rk;
        a.zo[k] = a.z[k];
        loc += rk * rk;
      }
      rel = sqrt(grid_sum(loc, a.part, 3, sh, grid)) / bnorm;
      if (rel <= a.tol) {
        ++it;
        break;
      }
      precond_grid<D>(a, grid);
      double rzn = 0.0, rzo = 0.0;
      for (int k = gt; k < n; k += gs) {
        rzn += a.r[k] * a.z[k];
        rzo += a.r[k] * a.zo[k];
      }
      rzn = grid_sum(rzn, a.part, 0, sh, grid);
      rzo = grid_sum(rzo, a.part, 1, sh, grid);
      const double beta = (rzn - rzo) / rz;
      rz = rzn;
      for (int k = gt; k < n; k += gs) a.p[k] = a.z[k] + beta * a.p[k];
      grid.sync();
    }
  }
  // linearised cost change with the undamped H
  spmv_grid<D>(a.A, a.N, 0.0, a.delta, a.q);
  grid.sync();
  double gd = 0.0, dhd = 0.0;
  for (int k = gt; k < n; k += gs) {
    gd += a.g[k] * a.delta[k];
    dhd += a.delta[k] * a.q[k];
  }
  gd = grid_sum(gd, a.part, 2, sh, grid);
  dhd = grid_sum(dhd, a.part, 3, sh, grid);
  if (gt == 0) {
    a.out[0] = -gd - 0.5 * dhd;
    a.out[1] = ok;
    a.out[2] = it;
    a.out[3] = rel;
  }
}

// (H + lambda D) delta = -g with the whole-GPU flexible PCG (k_pcg_coop).
double set_direct_solve_guard(double flops, int prefer) {
  g_guard_prefer.store(prefer);
  return g_guard_flops.exchange(flops);
}

// the whole-GPU PCG solve; *ms (optional) receives its kernel time
SolveOut pcg_solve(SolverDev& s, double lambda, cudaStream_t st, double* ms_out);

// the fill-in guard's race on the first damped system: the PCG path, then
// the direct solve, whose result this solve keeps (the choice affects the
// later solves only); the faster path (or the preferred one) stays
static SolveOut race_solve(SolverDev& s, double lambda, cudaStream_t st) {
  double pcg_ms = 0.0;
  const SolveOut op = pcg_solve(s, lambda, st, &pcg_ms);
  const double before = kernel_times().chol_ms;
  const SolveOut oc = chol_solve(s, *s.chol, lambda, st);
  const double chol_ms = kernel_times().chol_ms - before;
  const int prefer = g_guard_prefer.load();
  s.pcg_chosen = prefer == 2 || (prefer == 0 && op.ok && pcg_ms < chol_ms);
  s.race = 0;
  SolveOut o = oc;
  o.cg_iterations = op.cg_iterations;
  return o;
}

SolveOut solver_solve(SolverDev& s, double lambda, cudaStream_t st) {
  if (use_direct(s)) return s.race ? race_solve(s, lambda, st) : chol_solve(s, *s.chol, lambda, st);
  return pcg_solve(s, lambda, st, nullptr);
}

SolveOut pcg_solve(SolverDev& s, double lambda, cudaStream_t st, double* ms_out) {
  SolveOut o;
  if (s.N == 0) {
    o.ok = 1;
    return o;
  }
  const int sms = device_sm_count();
  const int grid = sms, threads = 256;
  s.part.resize((size_t)4 * grid);
  CsrView A{s.Hd.get(), s.fH.get(), s.Hd64.get(), s.fH64.get(), s.row_ptr.get(), s.col.get(), s.blk.get(),
            s.btr.get(), s.dampD.get()};
  int top = 0;
  while (top < s.levels - 1 && s.lvl_n[top] > 1024) ++top;
  CoopArgs a{s.N, s.levels, top, s.d_lvl_off.get(), s.d_lvl_n.get(), A, lambda, s.g.get(), s.Md.get(), s.Mu.get(),
             s.bD.get(), s.bDinv.get(), s.bU.get(), s.bFL.get(), s.bFR.get(), s.bb.get(), s.bx.get(), s.r64.get(),
             s.z64.get(), s.zo64.get(), s.p64.get(), s.q64.get(), s.delta.get(), s.cr.get(), s.part.get(), 1e-12,
             5000, s.out.get()};
  void* args[] = {&a};
  if (s.dim == 3) {
    RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_bcr_factor_coop<6>, grid, threads, args, 0, st));
  } else {
    RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_bcr_factor_coop<3>, grid, threads, args, 0, st));
  }
  RPGO_LAUNCHED();
  double pcg_ms = 0.0;
  {
    EventTimer timer(st);
    if (s.dim == 3)
      RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_pcg_coop<6>, grid, threads, args, 0, st));
    else
      RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_pcg_coop<3>, grid, threads, args, 0, st));
    RPGO_LAUNCHED();
    pcg_ms = timer.elapsed_ms();
  }
  if (ms_out) *ms_out = pcg_ms;
  double h[4];
  RPGO_CUDA(cudaMemcpyAsync(h, s.out.get(), sizeof(h), cudaMemcpyDeviceToHost, st));
  RPGO_CUDA(cudaStreamSynchronize(st));
  {
    // algorithmic bytes of one CG iteration: FP64 block SpMV (diagonal and
    // off-diagonal blocks, indices, vectors), the FP64 vector updates and
    // dot products, and one FP32 cyclic-reduction apply over all levels
    const double d = s.d, dd = d * d, Nn = s.N, nnz = (double)s.col.size(), n = Nn * d;
    double bcr = 0.0;
    for (int l = 0; l < s.levels; ++l) {
      const double nl = s.lvl_n[l];
      bcr += 0.5 * nl * (2 * dd * 4 + 4 * d * 4) + 0.5 * nl * (2 * d * 4) + 0.5 * nl * (3 * dd * 4 + 5 * d * 4);
    }
    const double spmv = 8 * dd * (Nn + nnz) + 8 * d * (2 * Nn + nnz) + 9 * nnz;
    const double vec = 8 * n * 16 + 4 * n;
    kernel_times().pcg_ms += pcg_ms;
    kernel_times().pcg_launches += 1;
    kernel_times().pcg_bytes += (h[2] + 1.0) * (spmv + vec + bcr);
  }
  o.lin_change = h[0];
  o.ok = (int)h[1];
  o.cg_iterations = (int)h[2];
  o.rel_residual = h[3];
  return o;
}

SolveOut solver_solve_eval(SolverDev& s, double lambda, cudaStream_t st, double* nerr) {
  if (!use_direct(s) || s.race) {
    SolveOut o = solver_solve(s, lambda, st);
    if (o.ok && o.lin_change >= 0.0) {
      solver_retract(s, st);
      *nerr = solver_error(s, s.xnew.get(), s.weights.get(), st);
    }
    return o;
  }
  double* host = s.pin.get(3);
  chol_enqueue(s, *s.chol, lambda, st, host);
  // the candidate step and its cost, whatever the solve's outcome (unused
  // when it failed)
  solver_retract(s, st);
  host[2] = 0.0;
  if (s.F > 0) {
    const double* sum = enqueue_error_sum(s, s.xnew.get(), s.weights.get(), st);
    RPGO_CUDA(cudaMemcpyAsync(host + 2, sum, sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  RPGO_CUDA(cudaStreamSynchronize(st));
  SolveOut o = chol_finish(s, *s.chol, host);
  *nerr = host[2];
  return o;
}

void solver_retract(SolverDev& s, cudaStream_t st) {
  if (s.N == 0) return;
  const int tb = 128;
  if (s.dim == 3) k_retract<3><<<div_up(s.N, tb), tb, 0, st>>>(s.N, s.x.get(), s.delta.get(), s.xnew.get());
  else k_retract<2><<<div_up(s.N, tb), tb, 0, st>>>(s.N, s.x.get(), s.delta.get(), s.xnew.get());
  RPGO_LAUNCHED();
}

void solver_gnc_weights(SolverDev& s, const double* x, int n_known, const double* barc, double mu,
                        cudaStream_t st) {
  if (s.F == 0) return;
  const int tb = 128;
  if (s.dim == 3)
    k_factor_err<3><<<div_up(s.F, tb), tb, 0, st>>>(s.F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                    s.sqrt_info.get(), x, nullptr, s.ferr.get());
  else
    k_factor_err<2><<<div_up(s.F, tb), tb, 0, st>>>(s.F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                    s.sqrt_info.get(), x, nullptr, s.ferr.get());
  RPGO_LAUNCHED();
  k_gnc_weights<<<div_up(s.F, tb), tb, 0, st>>>(s.F, n_known, s.ferr.get(), barc, mu, s.weights.get());
  RPGO_LAUNCHED();
}

template <int DIM>
static void batch_pre_t(SolverDev& s, BatchDev& b, bool diagonal_damping, bool any_active, cudaStream_t st) {
  constexpr int d = DIM == 3 ? 6 : 3;
  const int tb = 128, N = s.N, F = s.F, stride = s.stride;
  k_batch_masks<<<div_up(std::max(N, F), tb), tb, 0, st>>>(N, F, b.vsys.get(), b.fsys.get(), b.ctl.get(),
                                                          b.vmask.get(), b.fmask.get());
  RPGO_LAUNCHED();
  const int64_t nx = (int64_t)N * stride;
  // accept, GNC weights, reset, error at x: in this order
  k_batch_copy<<<div_up(nx, 256), 256, 0, st>>>(nx, stride, b.vmask.get(), kBatchAccept, s.xnew.get(), s.x.get());
  RPGO_LAUNCHED();
  k_factor_err<DIM><<<div_up(F, tb), tb, 0, st>>>(F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                  s.sqrt_info.get(), s.x.get(), nullptr, s.ferr.get(), b.fmask.get(),
                                                  kBatchGnc);
  RPGO_LAUNCHED();
  k_batch_gnc<<<div_up(F, tb), tb, 0, st>>>(F, b.fsys.get(), b.foff.get(), b.nknown.get(), b.fmask.get(),
                                            s.ferr.get(), b.barc.get(), b.mu.get(), s.weights.get());
  RPGO_LAUNCHED();
  k_batch_copy<<<div_up(nx, 256), 256, 0, st>>>(nx, stride, b.vmask.get(), kBatchReset, s.x0.get(), s.x.get());
  RPGO_LAUNCHED();
  k_factor_err<DIM><<<div_up(F, tb), tb, 0, st>>>(F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                  s.sqrt_info.get(), s.x.get(), s.weights.get(), s.ferr.get(),
                                                  b.fmask.get(), kBatchError);
  RPGO_LAUNCHED();
  k_batch_sums<<<div_up((int64_t)b.G * 32, tb), tb, 0, st>>>(b.G, b.foff.get(), b.ctl.get(), kBatchError,
                                                            s.ferr.get(), b.err.get());
  RPGO_LAUNCHED();
  if (!any_active) return;
  // linearise, solve, retract, error at xnew: the active graphs
  const int rs = d + 2 * d * d + 1;
  s.lin_rec.resize((size_t)F * rs);
  k_linearize_a<DIM><<<div_up(F, 64), 128, 0, st>>>(F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                                s.sqrt_info.get(), s.x.get(), s.weights.get(),
                                                                s.lin_rec.get(), b.fmask.get());
  RPGO_LAUNCHED();
  k_linearize_b<DIM><<<div_up(F, 4 * (32 / d)), 128, 0, st>>>(F, s.kind.get(), s.sqrt_info.get(), s.lin_rec.get(),
                                                              nullptr, s.fH64.get(), s.fg.get(), b.fmask.get());
  RPGO_LAUNCHED();
  k_assemble_direct<d><<<div_up((int64_t)N * 32, tb), tb, 0, st>>>(
      N, s.inc_ptr.get(), s.inc_fac.get(), s.inc_role.get(), s.fH64.get(), s.fg.get(), s.Hd64.get(), s.g.get(),
      s.dampD.get(), diagonal_damping ? 1 : 0, b.vmask.get());
  RPGO_LAUNCHED();
  chol_block_hessian(s, *s.chol, st, b.vmask.get());
}

template <int DIM>
static void batch_post_t(SolverDev& s, BatchDev& b, cudaStream_t st) {
  const int tb = 128, N = s.N, F = s.F;
  k_retract<DIM><<<div_up(N, tb), tb, 0, st>>>(N, s.x.get(), s.delta.get(), s.xnew.get(), b.vmask.get());
  RPGO_LAUNCHED();
  k_factor_err<DIM><<<div_up(F, tb), tb, 0, st>>>(F, s.kind.get(), s.vi.get(), s.vj.get(), s.z.get(),
                                                  s.sqrt_info.get(), s.xnew.get(), s.weights.get(), s.ferr.get(),
                                                  b.fmask.get(), kBatchActive);
  RPGO_LAUNCHED();
  k_batch_sums<<<div_up((int64_t)b.G * 32, tb), tb, 0, st>>>(b.G, b.foff.get(), b.ctl.get(), kBatchActive,
                                                            s.ferr.get(), b.err.get() + b.G);
  RPGO_LAUNCHED();
}

void batch_round_pre(SolverDev& s, BatchDev& b, bool diagonal_damping, bool any_active, cudaStream_t st) {
  if (!s.chol) throw std::logic_error("joint batch without a direct-solve plan");
  if (s.dim == 3) batch_pre_t<3>(s, b, diagonal_damping, any_active, st);
  else batch_pre_t<2>(s, b, diagonal_damping, any_active, st);
}

void batch_round_solve(SolverDev& s, BatchDev& b, bool recompact, cudaStream_t st) {
  if (recompact) chol_batch_compact(*s.chol, b, st);
  chol_enqueue_batch(s, *s.chol, b, st);
}

void batch_round_post(SolverDev& s, BatchDev& b, cudaStream_t st) {
  if (s.dim == 3) batch_post_t<3>(s, b, st);
  else batch_post_t<2>(s, b, st);
}

}  // namespace rpgo

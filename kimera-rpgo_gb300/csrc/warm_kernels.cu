// Learned GNC warm start kernels: closure features, the closure network's
// forward pass, and its training step (forward + backward + Adam).
//
// The network is tiny (5,313 trainable parameters) and its batches are a few
// thousand closures, so every kernel here is latency-bound: one thread per
// closure for the forward/backward pass with the whole parameter set in
// shared memory (weights rounded to BF16 once per block, FP32 FMAs), and one
// thread per parameter for the gradient sums over the batch (a fixed
// summation order, so a training step is reproducible bit for bit).
#include <cuda_bf16.h>

#include "solver_kernels.hpp"
#include "solver_math.cuh"
#include "warm.hpp"

namespace rpgo {
namespace {

using namespace sm;

// ------------------------------------------------------------------ features
template <int DIM>
__global__ void k_closure_features(int nlc, int n_known, const int32_t* __restrict__ kind,
                                   const int32_t* __restrict__ vi, const int32_t* __restrict__ vj,
                                   const double* __restrict__ z, const double* __restrict__ R,
                                   const double* __restrict__ x0, const float* __restrict__ aux,
                                   float* __restrict__ out) {
  using L = SLie<DIM>;
  constexpr int d = L::d, st = L::stride;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nlc) return;
  const int f = n_known + q;
  float* o = out + (size_t)q * kFeat;
  if (kind[f] != 0) {
    for (int k = 0; k < kFeat; ++k) o[k] = 0.f;
    return;
  }
  typename L::Pose Xi, Xj, Z, h, rel;
  L::load(x0 + (size_t)vi[f] * st, Xi);
  L::load(x0 + (size_t)vj[f] * st, Xj);
  L::load(z + (size_t)f * st, Z);
  L::between(Xi, Xj, h);
  L::between(Z, h, rel);
  double e[d], ez[d];
  L::logmap(rel, e);
  L::logmap(Z, ez);
  const double* Rf = R + (size_t)f * d * d;
  double c = 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double r = 0.0;
    if (i < d) {
#pragma unroll
      for (int k = 0; k < d; ++k) r += Rf[d * i + k] * e[k];
      c += r * r;
    }
    o[i] = (float)log1p(fabs(r));
  }
  double rot, tr, zrot, ztr;
  if (DIM == 3) {
    rot = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    tr = sqrt(e[3] * e[3] + e[4] * e[4] + e[5] * e[5]);
    zrot = sqrt(ez[0] * ez[0] + ez[1] * ez[1] + ez[2] * ez[2]);
    const double* zt = z + (size_t)f * st + 9;
    ztr = sqrt(zt[0] * zt[0] + zt[1] * zt[1] + zt[2] * zt[2]);
  } else {
    rot = fabs(e[d - 1]);
    tr = sqrt(e[0] * e[0] + e[1] * e[1]);
    zrot = fabs(ez[d - 1]);
    const double* zt = z + (size_t)f * st + 2;
    ztr = sqrt(zt[0] * zt[0] + zt[1] * zt[1]);
  }
  const float* a = aux + (size_t)q * 4;
  const double gap = a[0];
  o[6] = (float)log1p(c);
  o[7] = (float)rot;
  o[8] = (float)log1p(tr);
  o[9] = (float)log1p(gap);
  o[10] = (float)log1p(c / fmax(1.0, gap));
  o[11] = a[1];
  o[12] = a[2];
  o[13] = a[3];
  o[14] = (float)log1p(ztr);
  o[15] = (float)zrot;
}

// one warp per listed row: popcount of the row and of the row AND mask
__global__ void k_row_stats(int n, const uint32_t* __restrict__ adj, int words, const uint32_t* __restrict__ mask,
                            const int32_t* __restrict__ rows, int count, int32_t* __restrict__ deg,
                            int32_t* __restrict__ support) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= count) return;
  const uint32_t* row = adj + (size_t)rows[w] * words;
  const int nw = (n + 31) / 32;
  int a = 0, b = 0;
  for (int k = lane; k < nw; k += 32) {
    const uint32_t x = row[k];
    a += __popc(x);
    b += __popc(x & mask[k]);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    deg[w] = a;
    support[w] = b;
  }
}

// ------------------------------------------------------------------ network
constexpr int kTpb = 128;

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// parameters into shared memory, weights rounded to BF16
__device__ __forceinline__ void load_params(const float* __restrict__ params, float* sp) {
  for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) {
    const float v = params[k];
    const bool weight = (k >= kOffW1 && k < kOffB1) || (k >= kOffW2 && k < kOffB2) || (k >= kOffW3 && k < kOffB3);
    sp[k] = weight ? bf16_round(v) : v;
  }
  __syncthreads();
}

__device__ __forceinline__ void normalise(const float* sp, const float* __restrict__ x, float* xn) {
#pragma unroll
  for (int i = 0; i < kFeat; ++i) xn[i] = (x[i] - sp[kOffMu + i]) * sp[kOffIsd + i];
}

__device__ __forceinline__ void layer1(const float* sp, const float* xn, float* h1) {
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    float acc = sp[kOffB1 + j];
#pragma unroll
    for (int i = 0; i < kFeat; ++i) acc = fmaf(sp[kOffW1 + j * kFeat + i], xn[i], acc);
    h1[j] = fmaxf(acc, 0.f);
  }
}

__device__ __forceinline__ float hidden2(const float* sp, const float* h1, int j) {
  float acc = sp[kOffB2 + j];
#pragma unroll
  for (int i = 0; i < kHid; ++i) acc = fmaf(sp[kOffW2 + j * kHid + i], h1[i], acc);
  return fmaxf(acc, 0.f);
}

__global__ void __launch_bounds__(kTpb) k_mlp_forward(int64_t n, const float* __restrict__ params,
                                                      const float* __restrict__ X, float* __restrict__ prob) {
  __shared__ float sp[kMlpParams];
  load_params(params, sp);
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float xn[kFeat], h1[kHid];
  normalise(sp, X + s * kFeat, xn);
  layer1(sp, xn, h1);
  float logit = sp[kOffB3];
  for (int j = 0; j < kHid; ++j) logit = fmaf(sp[kOffW3 + j], hidden2(sp, h1, j), logit);
  prob[s] = 1.f / (1.f + expf(-logit));
}

// per sample: activations, back-propagated errors of the mean BCE loss
__global__ void __launch_bounds__(kTpb) k_mlp_fwd_bwd(int64_t n, const float* __restrict__ params,
                                                      const float* __restrict__ X, const float* __restrict__ Y,
                                                      float inv_n, float* __restrict__ XN, float* __restrict__ H1,
                                                      float* __restrict__ H2, float* __restrict__ D1,
                                                      float* __restrict__ D2, float* __restrict__ DL,
                                                      float* __restrict__ loss) {
  __shared__ float sp[kMlpParams];
  load_params(params, sp);
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float xn[kFeat], h1[kHid], h2[kHid];
  normalise(sp, X + s * kFeat, xn);
  layer1(sp, xn, h1);
  float logit = sp[kOffB3];
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    h2[j] = hidden2(sp, h1, j);
    logit = fmaf(sp[kOffW3 + j], h2[j], logit);
  }
  const float y = Y[s];
  const float p = 1.f / (1.f + expf(-logit));
  loss[s] = fmaxf(logit, 0.f) - logit * y + log1pf(expf(-fabsf(logit)));
  const float dl = (p - y) * inv_n;
  DL[s] = dl;
#pragma unroll
  for (int i = 0; i < kFeat; ++i) XN[s * kFeat + i] = xn[i];
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    H1[s * kHid + j] = h1[j];
    H2[s * kHid + j] = h2[j];
    h2[j] = h2[j] > 0.f ? dl * sp[kOffW3 + j] : 0.f;  // dh2
    D2[s * kHid + j] = h2[j];
  }
  for (int i = 0; i < kHid; ++i) {
    float acc = 0.f;
#pragma unroll
    for (int j = 0; j < kHid; ++j) acc = fmaf(sp[kOffW2 + j * kHid + i], h2[j], acc);
    D1[s * kHid + i] = H1[s * kHid + i] > 0.f ? acc : 0.f;
  }
}

// one thread per trainable parameter: its gradient summed over the batch in
// sample order
__global__ void k_mlp_grads(int64_t n, const float* __restrict__ XN, const float* __restrict__ H1,
                            const float* __restrict__ H2, const float* __restrict__ D1, const float* __restrict__ D2,
                            const float* __restrict__ DL, float* __restrict__ grad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kMlpTrainable) return;
  const int k = q + kOffW1;
  const float* a;
  const float* b = nullptr;
  int sa, sb = 0;
  if (k < kOffB1) {
    const int j = (k - kOffW1) / kFeat, i = (k - kOffW1) % kFeat;
    a = D1 + j, sa = kHid, b = XN + i, sb = kFeat;
  } else if (k < kOffW2) {
    a = D1 + (k - kOffB1), sa = kHid;
  } else if (k < kOffB2) {
    const int j = (k - kOffW2) / kHid, i = (k - kOffW2) % kHid;
    a = D2 + j, sa = kHid, b = H1 + i, sb = kHid;
  } else if (k < kOffW3) {
    a = D2 + (k - kOffB2), sa = kHid;
  } else if (k < kOffB3) {
    a = DL, sa = 1, b = H2 + (k - kOffW3), sb = kHid;
  } else {
    a = DL, sa = 1;
  }
  float acc = 0.f;
  if (b)
    for (int64_t s = 0; s < n; ++s) acc = fmaf(a[s * sa], b[s * sb], acc);
  else
    for (int64_t s = 0; s < n; ++s) acc += a[s * sa];
  grad[k] = acc;
}

__global__ void k_adam(const float* __restrict__ grad, float* __restrict__ params, float* __restrict__ m,
                       float* __restrict__ v, float lr, float c1, float c2) {
  const int k = kOffW1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kMlpParams) return;
  constexpr float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float g = grad[k];
  const float mk = b1 * m[k] + (1.f - b1) * g;
  const float vk = b2 * v[k] + (1.f - b2) * g * g;
  m[k] = mk;
  v[k] = vk;
  params[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

// fixed-order sum of per-sample losses (one block)
__global__ void k_sum_f(int64_t n, const float* __restrict__ x, double* __restrict__ out) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (int64_t s = threadIdx.x; s < n; s += blockDim.x) acc += x[s];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

}  // namespace

void closure_features(const SolverDev& s, int n_known, const float* aux_dev, float* out_dev, cudaStream_t st) {
  const int nlc = s.F - n_known;
  if (nlc <= 0) return;
  const int tb = 128;
  if (s.dim == 3)
    k_closure_features<3><<<div_up(nlc, tb), tb, 0, st>>>(nlc, n_known, s.kind.get(), s.vi.get(), s.vj.get(),
                                                          s.z.get(), s.sqrt_info.get(), s.x0.get(), aux_dev, out_dev);
  else
    k_closure_features<2><<<div_up(nlc, tb), tb, 0, st>>>(nlc, n_known, s.kind.get(), s.vi.get(), s.vj.get(),
                                                          s.z.get(), s.sqrt_info.get(), s.x0.get(), aux_dev, out_dev);
  RPGO_LAUNCHED();
}

void launch_row_stats(int n, const uint32_t* adj, int words, const uint32_t* mask, const int32_t* rows, int count,
                      int32_t* deg, int32_t* support, cudaStream_t st) {
  if (count <= 0) return;
  const int tb = 256;
  k_row_stats<<<div_up((int64_t)count * 32, tb), tb, 0, st>>>(n, adj, words, mask, rows, count, deg, support);
  RPGO_LAUNCHED();
}

void mlp_forward(const float* params, int64_t n, const float* features, float* prob, cudaStream_t st) {
  if (n <= 0) return;
  k_mlp_forward<<<div_up(n, kTpb), kTpb, 0, st>>>(n, params, features, prob);
  RPGO_LAUNCHED();
}

double mlp_train_step(float* params, float* m, float* v, int64_t step, float lr, int64_t n, const float* features,
                      const float* labels, float* grad, cudaStream_t st) {
  RPGO_CUDA(cudaMemsetAsync(grad, 0, sizeof(float) * kMlpParams, st));
  if (n <= 0) return 0.0;
  DeviceBuffer<float> xn((size_t)n * kFeat), h1((size_t)n * kHid), h2((size_t)n * kHid), d1((size_t)n * kHid),
      d2((size_t)n * kHid), dl((size_t)n), loss((size_t)n);
  DeviceBuffer<double> lsum(1);
  k_mlp_fwd_bwd<<<div_up(n, kTpb), kTpb, 0, st>>>(n, params, features, labels, 1.f / (float)n, xn.get(), h1.get(),
                                                  h2.get(), d1.get(), d2.get(), dl.get(), loss.get());
  RPGO_LAUNCHED();
  k_mlp_grads<<<div_up(kMlpTrainable, 128), 128, 0, st>>>(n, xn.get(), h1.get(), h2.get(), d1.get(), d2.get(),
                                                         dl.get(), grad);
  RPGO_LAUNCHED();
  k_sum_f<<<1, 256, 0, st>>>(n, loss.get(), lsum.get());
  RPGO_LAUNCHED();
  if (lr > 0.f && step >= 1) {
    const float c1 = 1.f - powf(0.9f, (float)step), c2 = 1.f - powf(0.999f, (float)step);
    k_adam<<<div_up(kMlpTrainable, 128), 128, 0, st>>>(grad, params, m, v, lr, c1, c2);
    RPGO_LAUNCHED();
  }
  double total = 0.0;
  RPGO_CUDA(cudaMemcpyAsync(&total, lsum.get(), sizeof(double), cudaMemcpyDeviceToHost, st));
  RPGO_CUDA(cudaStreamSynchronize(st));
  return total / (double)n;
}

}  // namespace rpgo

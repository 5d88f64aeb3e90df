// Learned GNC warm start: per-closure features and the closure network
// (no counterpart in the reference; it feeds the warm-started schedule of
// solver.hpp, gnc_tls_warm).
//
// Network: 16 features -> 64 ReLU -> 64 ReLU -> 1 logit, sigmoid output (the
// probability that plain GNC keeps the closure). Parameters are one flat FP32
// array (the master copy the optimiser updates):
//   [0, 16)      feature mean          [16, 32)     feature 1 / std
//   [32, 1056)   W1 (64 x 16, row = hidden unit)    [1056, 1120) b1
//   [1120, 5216) W2 (64 x 64)          [5216, 5280) b2
//   [5280, 5344) W3 (64)               [5344]       b3
// The kernels multiply with the weights rounded to BF16 (round to nearest
// even) and accumulate in FP32; biases and activations stay FP32.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.cuh"

namespace rpgo {

struct SolverDev;

constexpr int kFeat = 16, kHid = 64;
constexpr int kOffMu = 0, kOffIsd = 16, kOffW1 = 32, kOffB1 = kOffW1 + kHid * kFeat, kOffW2 = kOffB1 + kHid,
              kOffB2 = kOffW2 + kHid * kHid, kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid;
constexpr int kMlpParams = kOffB3 + 1;     // 5345
constexpr int kMlpTrainable = kMlpParams - kOffW1;  // 5313

// Per-closure features of factors [n_known, F) of the solver graph at the
// initial values x0 (rows of 16 floats, factor order). aux holds 4 floats per
// closure computed on the host: odometry gap |i - j| (0 across robots), PCM
// degree ratio, log1p(degree), support by the PCM clique.
void closure_features(const SolverDev& s, int n_known, const float* aux_dev, float* out_dev, cudaStream_t st);

// PCM statistics of `count` adjacency rows: degree and the number of
// neighbours inside `mask` (a bitset over the n closures).
void launch_row_stats(int n, const uint32_t* adj, int words, const uint32_t* mask, const int32_t* rows, int count,
                      int32_t* deg, int32_t* support, cudaStream_t st);

// prob[k] = sigmoid(net(features[k])) for k < n.
void mlp_forward(const float* params, int64_t n, const float* features, float* prob, cudaStream_t st);

// Mean binary cross-entropy of the n samples and its gradient (grad: all
// kMlpParams entries, the normalisation slots zero). lr > 0 then applies one
// Adam step (t = step >= 1) to params[kOffW1:], with moments m, v.
double mlp_train_step(float* params, float* m, float* v, int64_t step, float lr, int64_t n, const float* features,
                      const float* labels, float* grad, cudaStream_t st);

}  // namespace rpgo

// Multi-robot frame alignment kernels (Pcm.h:1011-1131).
#include "align.hpp"
#include "solver_math.cuh"

namespace rpgo {
namespace {

using namespace sm;

// T_w0_wi = T_w0_front o Z o T_wi_back^-1, Z inverted when the closure runs
// from robot i to robot 0 (Pcm.h:1041-1055)
template <int DIM>
__global__ void k_frame_offsets(int count, const int32_t* __restrict__ front, const int32_t* __restrict__ back,
                                const uint8_t* __restrict__ swap, const int64_t* __restrict__ rows,
                                const double* __restrict__ traj, const double* __restrict__ meas,
                                double* __restrict__ out) {
  using L = SLie<DIM>;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  typename L::Pose F, B, Z, Zi, Bi, t, r;
  L::load(traj + (size_t)front[k] * L::stride, F);
  L::load(traj + (size_t)back[k] * L::stride, B);
  L::load(meas + (size_t)rows[k] * L::stride, Z);
  if (swap[k]) {
    L::inverse(Z, Zi);
    Z = Zi;
  }
  L::compose(F, Z, t);
  L::inverse(B, Bi);
  L::compose(t, Bi, r);
  L::store(r, out + (size_t)k * L::stride);
}

// values[rows[k]] = T o traj[slots[k]] (Pcm.h:1080-1088)
template <int DIM>
__global__ void k_transform_rows(int count, const double* __restrict__ T, const int32_t* __restrict__ slots,
                                 const double* __restrict__ traj, const int64_t* __restrict__ rows,
                                 double* __restrict__ values) {
  using L = SLie<DIM>;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  typename L::Pose A, P, r;
  L::load(T, A);
  L::load(traj + (size_t)slots[k] * L::stride, P);
  L::compose(A, P, r);
  L::store(r, values + (size_t)rows[k] * L::stride);
}

}  // namespace

void launch_frame_offsets(int dim, int count, const int32_t* front, const int32_t* back, const uint8_t* swap,
                          const int64_t* rows, const double* traj, const double* meas, double* out, cudaStream_t st) {
  if (count <= 0) return;
  const int tb = 128;
  if (dim == 3) k_frame_offsets<3><<<div_up(count, tb), tb, 0, st>>>(count, front, back, swap, rows, traj, meas, out);
  else k_frame_offsets<2><<<div_up(count, tb), tb, 0, st>>>(count, front, back, swap, rows, traj, meas, out);
  RPGO_LAUNCHED();
}

void launch_transform_rows(int dim, int count, const double* T, const int32_t* slots, const double* traj,
                           const int64_t* rows, double* values, cudaStream_t st) {
  if (count <= 0) return;
  const int tb = 128;
  if (dim == 3) k_transform_rows<3><<<div_up(count, tb), tb, 0, st>>>(count, T, slots, traj, rows, values);
  else k_transform_rows<2><<<div_up(count, tb), tb, 0, st>>>(count, T, slots, traj, rows, values);
  RPGO_LAUNCHED();
}

}  // namespace rpgo

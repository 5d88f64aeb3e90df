// Multi-robot frame alignment (Pcm.h:1011-1131): device helpers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace rpgo {

// out[k] = traj[front[k]] o (swap[k] ? meas[rows[k]]^-1 : meas[rows[k]]) o traj[back[k]]^-1
void launch_frame_offsets(int dim, int count, const int32_t* front, const int32_t* back, const uint8_t* swap,
                          const int64_t* rows, const double* traj, const double* meas, double* out, cudaStream_t st);
// values[rows[k]] = T o traj[slots[k]] (T: one pose on the device)
void launch_transform_rows(int dim, int count, const double* T, const int32_t* slots, const double* traj,
                           const int64_t* rows, double* values, cudaStream_t st);

}  // namespace rpgo

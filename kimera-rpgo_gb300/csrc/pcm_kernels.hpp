// Launch interface of the PCM and clique kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.cuh"

namespace rpgo {

// Device view of the odometry trajectories (one slot per key).
struct TrajView {
  double* pose;     // slots x stride (12 or 4)
  double* cov;      // slots x d*d (PoseWithCovariance)
  int32_t* node;    // slots (PoseWithNode)
  uint8_t* rot;     // slots, rotation_info flag
};

// mode 0: PoseWithCovariance (Pcm), 1: PoseWithNode (PcmSimple)
void launch_traj_scan(int dim, int mode, int64_t count, const int32_t* src, const int32_t* dst,
                      const double* dpose, const double* dcov, TrajView tr, DeviceBuffer<double>& scratch_rec,
                      DeviceBuffer<double>& scratch_cov, DeviceBuffer<uint8_t>& scratch_rot, cudaStream_t st);

void launch_odom_check(int dim, int mode, int64_t count, const int32_t* si, const int32_t* sj, const double* zp,
                       const double* zc, TrajView tr, double th0, double th1, uint8_t* ok, cudaStream_t st);

// adj: n rows of `words` uint32; lower_scratch: (n - row_begin) rows of `words`
// landmark pair checks (Pcm.h:775-844) of `count` observation pairs
// (ij: the two observations' rows; desc: trajectory slots, see the kernel);
// consistent pairs get their two adjacency bits set
void launch_landmark_pairs(int dim, int mode, int count, const int4* desc, const int2* ij, const double* zp,
                           const double* zc, TrajView tr, double th0, double th1, uint32_t* adj, int words,
                           cudaStream_t st);
// rows [0, rows) of a bit-packed adjacency (row stride `words`): clear the
// bits of every column >= from
void launch_clear_columns(uint32_t* adj, int words, int rows, int from, cudaStream_t st);
void launch_pairwise(int dim, int mode, int n, int row_begin, const int32_t* sa, const int32_t* sb,
                     const uint8_t* flip, const double* zp, const double* zc, TrajView tr, double th0, double th1,
                     uint32_t* adj, int words, uint32_t* lower_scratch, cudaStream_t st);

// Greedy max clique (findCliqueHeu.cpp:32-209) on a device bit matrix.
// Returns the clique size (seed if no candidate improved) and fills `clique`
// with the first `size` slots of the winning work buffer.
struct CliqueWorkspace {
  DeviceBuffer<int32_t> deg;
  DeviceBuffer<int32_t> result;   // per window slot: icc or -1
  DeviceBuffer<int32_t> buffers;  // per window slot: work buffer (n + 1)
  DeviceBuffer<uint32_t> sets;    // per window slot: bitset of the current candidate set
  std::vector<int32_t> h_result;
};
int max_clique_heu(int n, const uint32_t* adj, int words, int first, int seed, std::vector<int32_t>* clique,
                   CliqueWorkspace& ws, cudaStream_t st);

}  // namespace rpgo

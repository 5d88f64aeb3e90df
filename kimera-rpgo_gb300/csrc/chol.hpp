// Direct solve of the damped normal equations (H + lambda D) delta = -g:
// sparse block Cholesky over the plan of chol_plan.hpp, in FP64, as one
// cooperative kernel per solve (factorisation, forward and backward
// substitution, model change).
#pragma once
#include <cuda_runtime.h>

#include "chol_plan.hpp"
#include "common.cuh"
#include "solver_kernels.hpp"

namespace rpgo {

struct CholDev {
  CholPlan plan;
  int levels = 0;
  DeviceBuffer<int32_t> perm, col_ptr, blk_row, blk_col, lvl_col_ptr, lvl_cols, lvl_task_ptr, tasks, btask, ftask;
  DeviceBuffer<int32_t> upd_ptr, upd_src, tupd_ptr, tupd_src, a_ptr, a_src, ta_ptr, ta_src;
  DeviceBuffer<int32_t> row_ptr, row_blk, trow_ptr, trow_blk, ttasks, ttask_ptr;
  DeviceBuffer<double> L;     // sparse blocks of L (off-diagonal; the diagonal slots are unused)
  DeviceBuffer<double> Ldiag; // factors of the sparse diagonal blocks (reciprocal pivots on the diagonal)
  DeviceBuffer<double> M;     // dense tail, column-major, padded to whole tiles
  DeviceBuffer<double> Ldd;   // factors of the tail's diagonal tiles (reciprocal pivots on the diagonal)
  DeviceBuffer<double> y;     // right-hand side / solution in elimination order
  DeviceBuffer<double> part;  // per-CTA partial sums
  DeviceBuffer<double> Spart; // level-task partial sums (D x D per task)
  DeviceBuffer<double> Tpart; // tail row task sums (D per task)
  DeviceBuffer<double> out;   // model change, status
  DeviceBuffer<double> Hs;    // H in the block layout of L (per linearisation)
  DeviceBuffer<double> dampS; // damping diagonal of the diagonal blocks, same layout
  DeviceBuffer<int32_t> status;
  cudaEvent_t ev[2] = {nullptr, nullptr};  // around each launch (kernel time)
  ~CholDev();
  void upload(CholPlan&& p, cudaStream_t st);
};

// H and the damping diagonal in the block layout of L, from the linearised
// system (Hd64, fH64, dampD); enqueued after every linearisation.
// mask: a joint batch's variable control words (bit 0: graph in this round)
void chol_block_hessian(SolverDev& s, CholDev& c, cudaStream_t st, const uint8_t* mask = nullptr);
// Solve with the factorisation of (H + lambda D); fills s.delta.
SolveOut chol_solve(SolverDev& s, CholDev& c, double lambda, cudaStream_t st);
// Enqueue the same solve without waiting: the model change and the status
// are copied to host[0] and host[1] (page-locked) by the stream; call
// chol_finish after the stream reached that point.
void chol_enqueue(SolverDev& s, CholDev& c, double lambda, cudaStream_t st, double* host);
SolveOut chol_finish(SolverDev& s, CholDev& c, const double* host);
// Joint batch: enqueue one launch that solves every active system of the
// batch b with its own damping; per-system model change and status land in
// b.out (2 per system), the steps in s.delta.
void chol_enqueue_batch(SolverDev& s, CholDev& c, const BatchDev& b, cudaStream_t st);
// Joint batch: compact the plan's level lists to the graphs whose control
// word (already on the device) has kBatchActive; later chol_enqueue_batch
// launches use the compacted lists.
void chol_batch_compact(CholDev& c, BatchDev& b, cudaStream_t st);
// kernel time of the last enqueued launch (after the stream passed it)
float chol_last_ms(CholDev& c);

}  // namespace rpgo

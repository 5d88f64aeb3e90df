// Launch interface of the nonlinear least-squares kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <vector>

#include "common.cuh"

namespace rpgo {

struct CholDev;
struct CholPlan;

// Joint batch: G independent graphs held as one problem whose variables and
// factors of graph s are contiguous ([voff[s], voff[s + 1]), [foff[s],
// foff[s + 1])); the elimination positions of graph s are its variables'
// range too. Each round works on the graphs selected by their control word:
enum : uint8_t {
  kBatchActive = 1,   // linearise, solve, retract and evaluate the new error
  kBatchAccept = 2,   // first: x <- xnew (the last step was accepted)
  kBatchGnc = 4,      // then: TLS weights from the residuals at x with mu
  kBatchReset = 8,    // then: x <- x0 (an LM run from the initial values)
  kBatchError = 16,   // then: the weighted error at x
};
struct BatchDev {
  int G = 0;
  std::vector<int32_t> h_voff, h_foff;
  DeviceBuffer<int32_t> vsys, fsys;    // variable / factor -> graph
  DeviceBuffer<int32_t> voff, foff;    // G + 1 each
  DeviceBuffer<int32_t> nknown;        // per graph: known inliers (weights fixed at 1)
  DeviceBuffer<uint8_t> ctl;           // per graph control word (kBatch*)
  DeviceBuffer<uint8_t> vmask, fmask;  // the control word per variable / factor
  DeviceBuffer<double> lam, mu;        // per graph damping and GNC parameter
  DeviceBuffer<double> barc;           // per factor TLS threshold
  DeviceBuffer<int32_t> status;        // per graph pivot failure
  DeviceBuffer<double> out;            // per graph: model change, status (direct solve)
  DeviceBuffer<double> term;           // per variable: model change partials
  DeviceBuffer<double> err;            // per graph: error at x (kBatchError), at xnew (kBatchActive)
  // the direct solve's level lists compacted to the graphs in the round
  // (rebuilt when that set changes; chunk tables fixed by the merged plan)
  bool compacted = false;
  DeviceBuffer<int4> task_chunks, col_chunks, tasks_c;
  DeviceBuffer<int32_t> task_level_chunks, col_level_chunks, task_counts, col_counts, task_end, col_end, cols_c;
  int n_task_chunks = 0, n_col_chunks = 0;
};

// Device-resident problem: factors, structure, per-iteration buffers.
struct SolverDev {
  int dim = 3, d = 6, stride = 12, N = 0, F = 0;
  int coop_ctas = 0;  // CTAs of the cooperative direct solve (0: one per SM)
  // fill-in guard: a direct plan whose factorisation exceeds the guard's
  // flops runs its first damped system with both solvers (race = 1) and
  // keeps the faster (pcg_chosen when the PCG path won)
  int race = 0;
  bool pcg_chosen = false;
  // factors
  DeviceBuffer<int32_t> kind, vi, vj;
  DeviceBuffer<uint8_t> tree;            // between factor joining consecutive variables
  DeviceBuffer<double> z, sqrt_info;     // F x stride, F x d*d
  DeviceBuffer<double> weights;          // F
  // incidence CSR (per variable: factor, role 0 = i / prior, 1 = j)
  DeviceBuffer<int32_t> inc_ptr, inc_fac;
  DeviceBuffer<int8_t> inc_role;
  DeviceBuffer<uint8_t> var_has_tree;
  // SpMV CSR of off-diagonal blocks (per row: column, factor, transposed)
  DeviceBuffer<int32_t> row_ptr, col, blk;
  DeviceBuffer<int8_t> btr;
  // linearisation
  DeviceBuffer<float> fH;      // F x 3 x dd (Hii, Hjj, Hij), FP32 copy for CG and preconditioner
  DeviceBuffer<double> fH64;   // the same blocks in FP64 for the refinement residual
  DeviceBuffer<double> fg;     // F x 2 x d
  DeviceBuffer<double> lin_rec;  // F x (d + 2 dd + 1): linearisation phase-A records
  DeviceBuffer<float> Hd, Md, Mu;  // N x dd, N x dd, N x dd (Mu[v] couples v, v+1)
  DeviceBuffer<double> Hd64;       // N x dd
  DeviceBuffer<double> g, dampD;   // N x d
  // values and step
  DeviceBuffer<double> x0, x, xnew;  // N x stride
  DeviceBuffer<double> delta;        // N x d
  DeviceBuffer<double> ferr;         // F (per-factor error)
  DeviceBuffer<double> red;          // reduction scratch
  DeviceBuffer<unsigned int> ticket; // last-block counter of the one-launch error sum
  // preconditioner (block cyclic reduction) and CG scratch
  std::vector<int32_t> lvl_off, lvl_n;
  DeviceBuffer<int32_t> d_lvl_off, d_lvl_n;
  DeviceBuffer<float> bD, bDinv, bU, bFL, bFR, bb, bx;  // per level node
  DeviceBuffer<float> cr, cz, cp, cq, cx;               // N x d, FP32 CG vectors
  DeviceBuffer<double> rowtmp;                          // per-row reduction terms
  DeviceBuffer<double> part;                            // per-CTA partial sums
  DeviceBuffer<double> r64, z64, zo64, p64, q64;        // N x d, CG vectors
  DeviceBuffer<double> out;                              // solve outputs
  int levels = 0;
  // direct solver (sparse Cholesky); null when the PCG path solves
  std::shared_ptr<CholDev> chol;
  PinnedBuffer<double> pin;  // host words of solve_eval's single readback
};

struct SolveOut {
  double lin_change = 0.0;  // -g.delta - 0.5 delta^T H delta
  int ok = 0;
  int cg_iterations = 0;
  double rel_residual = 0.0;
};

// setup: builds the structure from the host factor list and sizes every
// buffer; the caller fills z, sqrt_info and x0 (device gathers)
// direct: plan the sparse Cholesky solve (else, or when its factor would
// exceed the memory budget, the whole-GPU PCG solves the steps)
// plan: a prepared plan for the direct solve (the joint batch's merged plan)
void solver_upload(SolverDev& s, int dim, const std::vector<int32_t>& kind, const std::vector<int32_t>& vi,
                   const std::vector<int32_t>& vj, int N, cudaStream_t st, bool direct,
                   CholPlan* plan = nullptr);
// per-factor error 0.5 w |R e|^2 at values `x` (weights null = 1); returns the sum
double solver_error(SolverDev& s, const double* x, const double* weights, cudaStream_t st);
// per-factor unweighted errors at x into s.ferr (host copy returned)
void solver_factor_errors(SolverDev& s, const double* x, std::vector<double>* out, cudaStream_t st);
// linearise at s.x with s.weights; assembles Hd, g, tree blocks, damping diagonal
void solver_linearize(SolverDev& s, bool diagonal_damping, cudaStream_t st);
// solve (H + lambda D) delta = -g into s.delta
SolveOut solver_solve(SolverDev& s, double lambda, cudaStream_t st);
// fill-in guard of the direct solve (process-wide): plans of more than
// `flops` factorisation flops race both solvers on their first damped
// system; prefer 0 keeps the faster, 1 always the direct solve, 2 always the
// PCG path (for tests). Returns the previous threshold.
double set_direct_solve_guard(double flops, int prefer);
// solve, then xnew = x (+) delta and its weighted error *nerr (valid when
// the solve succeeded with a non-negative model change); with the direct
// solver the three results come back in one synchronisation
SolveOut solver_solve_eval(SolverDev& s, double lambda, cudaStream_t st, double* nerr);
// xnew = x (+) delta
void solver_retract(SolverDev& s, cudaStream_t st);
// enqueue the weighted error of x (one launch); returns the device word that
// will hold it
double* enqueue_error_sum(SolverDev& s, const double* x, const double* weights, cudaStream_t st);
// TLS weights (GncOptimizer::calculateWeights) for factors >= n_known, with
// the per-factor thresholds barc on the device; enqueued only (the stream
// orders them before the next solve)
void solver_gnc_weights(SolverDev& s, const double* x, int n_known, const double* barc, double mu,
                        cudaStream_t st);

// Joint batch rounds (s is the union problem, planned with its own CholPlan
// from merge_chol_plans), for the graphs selected by the control words in
// b.ctl (already on the device). batch_round_pre: the accept / GNC / reset
// updates of x and the weights, the error at x, then (any_active: some graph
// has kBatchActive) the linearisation and block Hessian; batch_round_solve:
// the cooperative direct solve with each graph's damping b.lam (recompact:
// the set of graphs in the round changed, the level lists are compacted
// again first);
// batch_round_post: the retraction and the error at xnew. Results (b.out,
// b.err) stay on the device.
void batch_round_pre(SolverDev& s, BatchDev& b, bool diagonal_damping, bool any_active, cudaStream_t st);
void batch_round_solve(SolverDev& s, BatchDev& b, bool recompact, cudaStream_t st);
void batch_round_post(SolverDev& s, BatchDev& b, cudaStream_t st);

}  // namespace rpgo

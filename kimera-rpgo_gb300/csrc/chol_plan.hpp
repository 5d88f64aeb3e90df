// Symbolic analysis of the block-sparse normal equations for the direct
// (Cholesky) solve of the Gauss-Newton / Levenberg-Marquardt step.
//
// The reference solves the damped normal equations with GTSAM's default
// linear solver, a sparse multifrontal Cholesky (the LevenbergMarquardtParams
// / GaussNewtonParams built in src/RobustSolver.cpp:120-300 keep GTSAM's
// default linearSolverType). Here the same system is factored on the GPU.
// The plan fixes, once per graph structure:
//  * an elimination order (minimum degree on the pose graph, ties by index);
//  * the block structure of L and its elimination tree;
//  * a split into sparse columns, scheduled by elimination-tree level, and a
//    trailing dense block (the columns whose structure is already complete);
//  * for every target block, the list of block products that update it, and
//    the Hessian blocks that initialise it (so that every sum runs in a fixed
//    order: results do not depend on thread scheduling).
#pragma once
#include <cstdint>
#include <vector>

namespace rpgo {

struct CholPlan {
  int N = 0;             // variables (block columns)
  int d = 6;             // block size
  int n_sparse = 0;      // columns [0, n_sparse) are sparse, [n_sparse, N) form the dense tail
  int T = 0;             // tail size in blocks (N - n_sparse)
  int tile = 24;         // tile size (scalars) of the dense tail
  int n_tiles = 0;       // tail tiles per side (padded)
  std::vector<int32_t> perm;  // position -> variable
  std::vector<int32_t> pos;   // variable -> position
  // sparse part of L: per column, its diagonal block first, then the
  // off-diagonal blocks in ascending row order (rows may lie in the tail)
  std::vector<int32_t> col_ptr;  // n_sparse + 1
  std::vector<int32_t> blk_row;  // row position of each block
  std::vector<int32_t> blk_col;  // column position of each block
  // elimination-tree levels of the sparse columns (leaves first)
  std::vector<int32_t> lvl_col_ptr, lvl_cols;  // columns per level
  // Tasks of the sparse levels, 4 ints each (id, first, end, code), code =
  // kind | half << 2 | diagonal block << 3 | slot << 4; each writes partial
  // sums to its slot:
  //  kind 0 / 1: block id's update list [first, end) cut into chunks of at
  //    most `chunk` pairs (kind 1 on the block's first chunk, which also
  //    carries the Hessian block); for 6x6 blocks every chunk is two tasks,
  //    output columns 0-2 (half 0) and 3-5 (half 1), sharing one slot; a
  //    block without update pairs (every block of the first level, the
  //    leaves) has no task (btask count 0) and is read from the Hessian when
  //    its column is finalised;
  //  kind 2: the forward-substitution row sum of column id over its row
  //    list entries [first, end) (chunks of at most `row_chunk`).
  // Tasks of one level are contiguous (lvl_task_ptr), ordered by descending
  // work; the slots of one block (btask: first, count) and of one column's
  // row sum (ftask) are contiguous. Each level's columns (lvl_cols) are
  // ordered by descending block count.
  int chunk = 5, row_chunk = 20, n_slots = 0;
  std::vector<int32_t> lvl_task_ptr, tasks, btask, ftask;
  // tail row tasks: the sparse part of tail block row t, [first, end) of
  // trow_blk, in chunks of at most row_chunk (3 ints each: row, first, end);
  // the tasks of row t are [ttask_ptr[t], ttask_ptr[t + 1])
  std::vector<int32_t> ttasks, ttask_ptr;
  // updates: target -= sum over (a, b) of L[a] * L[b]^T, as flat pairs
  std::vector<int32_t> upd_ptr, upd_src;    // sparse targets (per block)
  std::vector<int32_t> tupd_ptr, tupd_src;  // tail targets (lower blocks bi >= bj, index bi*(bi+1)/2 + bj)
  // Hessian off-diagonal blocks that initialise a target: 2*f + transposed
  std::vector<int32_t> a_ptr, a_src;    // sparse targets
  std::vector<int32_t> ta_ptr, ta_src;  // tail targets
  // forward solve: per sparse row j, its off-diagonal blocks (j, k), k < j;
  // per tail block row t, the sparse blocks in that row; both as (block,
  // column) pairs
  std::vector<int32_t> row_ptr, row_blk;
  std::vector<int32_t> trow_ptr, trow_blk;
  int levels() const { return (int)lvl_col_ptr.size() - 1; }
  int n_blocks() const { return (int)blk_row.size(); }
  int n_tail_blocks() const { return T * (T + 1) / 2; }
  double flops = 0.0;  // algorithmic FP64 flops of one factorisation
  // algorithmic device-memory bytes of one solve: the Hessian blocks read,
  // the factor written once and read by the factorisation's consumers and by
  // the two substitutions, the right-hand side, solution and step vectors
  double bytes = 0.0;
};

// kind/vi/vj: the factor list (kind 0 = between vi-vj, 1 = prior on vi).
// dense_tail false: every column sparse (T = 0), as merge_chol_plans needs.
CholPlan make_chol_plan(int N, int d, const std::vector<int32_t>& kind, const std::vector<int32_t>& vi,
                        const std::vector<int32_t>& vj, bool dense_tail = true);

// One plan for independent systems (a joint batch of graphs), from their
// plans without dense tails: plan g's positions and variables follow those
// of plans 0 .. g-1, as do its blocks, slots and list entries; its factors
// are foff[g] .. foff[g + 1] - 1 of the merged factor list. Level l holds
// every plan's level l, ordered as make_chol_plan orders a level. Each
// system's operations are those of its own plan.
CholPlan merge_chol_plans(const std::vector<CholPlan>& plans, const std::vector<int32_t>& foff);

}  // namespace rpgo

// Sparse block Cholesky solve of (H + lambda D) delta = -g on the GPU (FP64).
//
// One cooperative kernel per solve, 256 threads per CTA, one CTA per SM.
// Phases are separated by grid barriers:
//  1. init: right-hand side in elimination order, padding of the dense tail;
//  2. per elimination-tree level of the sparse columns (leaves first):
//     (A) the level's tasks over all warps: for every block, its Hessian
//         block (read from the block layout Hs that k_block_hessian writes
//         once per linearisation) minus chunks of its L(i,k) L(j,k)^T
//         updates, and chunks of every column's forward-substitution row
//         sum; the leaves have no tasks;
//     (B) every column by one warp (narrow levels: a team of two warps):
//         S_jj from the partial sums, L_jj = chol(S_jj), L_ij = S_ij
//         L_jj^-T, and y_j;
//  3. the dense tail: its blocks from H and the sparse updates (one CTA per
//     block), then a right-looking tiled Cholesky with one barrier per tile
//     column: in phase k the CTAs of tile column k apply the update of column
//     k-1, factor the diagonal tile and solve their tile, while all other CTAs
//     apply the column k-1 update to the trailing tiles; the forward
//     substitution of tile k-1 runs in the same phase. A tail of one tile is
//     factored and solved (both substitutions) by one CTA in one phase;
//  4. backward substitution over the tail tiles, then the sparse levels (top
//     first); scatter to variable order together with the linearised cost
//     change of the undamped system (a fixed-order grid reduction).
// FP64 on this part retires one warp instruction per ~33 ns per SM
// sub-partition whether or not it depends on the previous one (a divide or
// square root costs ~220-300 ns), so the kernel minimises FP64 instructions on
// each phase's busiest warp: lane groups that serve several blocks per warp
// instruction, one FMA chain per output, reductions over the active lane
// groups only, entry-wise partial sums, and one reciprocal square root per
// pivot (the factors keep the reciprocal of each pivot on their diagonal and
// every solve multiplies by it). Work items spread one per SM where a level is
// narrow, and the column work of narrow levels is split over two warps.
// Every sum runs in an order fixed by the plan, so results do not depend on
// scheduling. A non-positive (or NaN) pivot sets the status flag; the factor
// continues with pivot 1 so that every phase still ends, and the host treats
// the solve as failed (as GTSAM's IndeterminantLinearSystemException).
#include <cooperative_groups.h>

#include "chol.hpp"

namespace cg = cooperative_groups;

namespace rpgo {
namespace {

constexpr int kTB = 24;  // dense tail tile (scalars); a multiple of both block sizes
constexpr int kThreads = 256;
// a level's tasks (columns) run one per lane group instead of one per warp
// when there are at least this many per warp of the grid
constexpr int kGroupModeItems = 2;

struct CholArgs {
  int N, ns, T, ntp, n_tiles, levels;
  const int32_t *perm, *col_ptr, *blk_row, *blk_col, *lvl_col_ptr, *lvl_cols, *lvl_task_ptr, *tasks, *btask, *ftask;
  const int32_t *upd_ptr, *upd_src, *tupd_ptr, *tupd_src, *a_ptr, *a_src, *ta_ptr, *ta_src;
  const int32_t *row_ptr, *row_blk, *trow_ptr, *trow_blk, *ttasks, *ttask_ptr;
  const double *Hd64, *fH64, *dampD, *g;
  double lam;
  double *L, *Ldiag, *M, *Ldd, *y, *delta, *part, *out, *Spart, *Tpart;
  const double *Hs, *dampS;  // Hessian and damping diagonal in the factor's block layout
  int32_t* status;
  // Independent systems solved in one launch (a joint batch of graphs; G = 0
  // for one system). System s owns the positions (and variables) [b_off[s],
  // b_off[s + 1]); b_sys maps a position to its system. Systems whose b_act
  // word has bit 0 clear are skipped. Each has its own damping, status and model change.
  int G;
  const int32_t *b_sys, *b_off;
  const uint8_t* b_act;
  const double* b_lam;
  int32_t* b_status;
  double *b_out, *b_term;  // per system (model change, status); per position partials
  // the level lists hold only the solved systems' items (tasks and lvl_cols
  // compacted per level, in plan order, ending at lvl_task_end / lvl_col_end)
  int b_compact;
  const int32_t *lvl_task_end, *lvl_col_end;
};

// end of level l's tasks and columns (the compacted lists of a joint batch
// end early)
__device__ __forceinline__ int task_end(const CholArgs& a, int l) {
  return a.lvl_task_end ? a.lvl_task_end[l] : a.lvl_task_ptr[l + 1];
}
__device__ __forceinline__ int col_end(const CholArgs& a, int l) {
  return a.lvl_col_end ? a.lvl_col_end[l] : a.lvl_col_ptr[l + 1];
}

__device__ __forceinline__ void set_fail(int32_t* status) { atomicExch(status, 1); }

// the system of position j is solved by this launch
__device__ __forceinline__ bool sys_on(const CholArgs& a, int j) {
  return a.G == 0 || a.b_compact || (a.b_act[a.b_sys[j]] & 1);
}
// status word of the system of position j
__device__ __forceinline__ int32_t* sys_status(const CholArgs& a, int j) {
  return a.G == 0 ? a.status : a.b_status + a.b_sys[j];
}

// Hessian entry (r, c) of the block at (row var, col var) from the factor
// off-diagonal blocks in src[beg, end) (2 f + transposed)
template <int D>
__device__ __forceinline__ double gather_offdiag(const double* __restrict__ fH64, const int32_t* __restrict__ src,
                                                 int beg, int end, int r, int c) {
  constexpr int dd = D * D;
  double s = 0.0;
  for (int u = beg; u < end; ++u) {
    const int32_t x = src[u];
    const double* H = fH64 + (size_t)(x >> 1) * 3 * dd + 2 * dd;
    s += (x & 1) ? H[c * D + r] : H[r * D + c];
  }
  return s;
}

template <int D>
__device__ __forceinline__ double gather_diag(const CholArgs& a, int v, int r, int c) {
  constexpr int dd = D * D;
  double s = a.Hd64[(size_t)v * dd + r * D + c];
  if (r == c) s += a.lam * a.dampD[(size_t)v * D + r];
  return s;
}

// entry (r, c) of sparse block p of H + lambda D from the block layout
// (the same values and additions as gather_diag / gather_offdiag)
template <int D>
__device__ __forceinline__ double block_H(const CholArgs& a, int p, bool diag, int r, int c) {
  constexpr int dd = D * D;
  double s = a.Hs[(size_t)p * dd + r * D + c];
  if (diag && r == c) {
    const double lam = a.G == 0 ? a.lam : a.b_lam[a.b_sys[a.blk_col[p]]];
    s += lam * a.dampS[(size_t)p * D + r];
  }
  return s;
}

constexpr unsigned kFull = 0xffffffffu;

// Sparse levels use lane groups: a warp holds 32 / D groups of D lanes and
// lane r of a group owns row r of every D x D block, so one warp-wide FP64
// instruction serves several groups. (The FP64 pipe of this part retires two
// lanes per cycle per SM: a warp instruction costs the same whether or not
// its lanes do useful work.)

// phase A, one warp per task: the groups take the task's entries in turn,
// then the sums of the groups that took entries are added in group order into
// lanes 0 .. D-1. The FP64 pipe retires a warp instruction every ~33 ns
// whether or not it depends on the previous one, so products accumulate in
// one FMA chain per output (no split accumulators) and only groups with
// entries join the sum: the instruction count is the cost.
//  block task (kind 0 / 1): Spart[t] = (kind 1: H block of id, + lambda D on
//    a diagonal block) - sum over its pairs (a, b) of L[a] L[b]^T;
//  row task (kind 2): Spart[t][r] = sum over its row entries (block q,
//    column k) of (L[q] y_k)[r].
// The index chain of task t for a warp: the task record and its lane
// group's first pair (block tasks: the two blocks; row tasks: the block and
// its column). Plan data, so a narrow level's task phase has it loaded ahead
// of the barrier before it.
struct TaskAhead {
  int4 tk;
  int u0, u1;
};
template <int D>
__device__ __forceinline__ void task_ahead(const CholArgs& a, int t, int lane, TaskAhead& x) {
  constexpr int G = 32 / D;
  const int g = lane / D;
  x.tk = reinterpret_cast<const int4*>(a.tasks)[t];
  const int u = x.tk.y + g;
  const int32_t* src = (x.tk.w & 3) < 2 ? a.upd_src : a.row_blk;
  x.u0 = (g < G && u < x.tk.z) ? src[2 * u] : 0;
  x.u1 = (g < G && u < x.tk.z) ? src[2 * u + 1] : 0;
}

template <int D>
__device__ void run_task_core(const CholArgs& a, const TaskAhead& x, int lane) {
  constexpr int G = 32 / D, dd = D * D;
  constexpr int NC = D == 6 ? 3 : D;  // output columns of one block task
  const int g = lane / D, r = lane % D;
  const int4 tk = x.tk;
  const int kind = tk.w & 3, slot = tk.w >> 4;
  if (!sys_on(a, kind < 2 ? a.blk_col[tk.x] : tk.x)) return;  // (warp-uniform)
  if (kind < 2) {
    const int p = tk.x, c0 = ((tk.w >> 2) & 1) * NC;
    double acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = 0.0;
    if (kind == 1 && g == 0) {
      const bool diag = (tk.w >> 3) & 1;
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] = block_H<D>(a, p, diag, r, c0 + c);
    }
    if (g < G) {
      for (int u = tk.y + g; u < tk.z; u += G) {
        const bool first = u == tk.y + g;
        const int pa = first ? x.u0 : a.upd_src[2 * u], pb = first ? x.u1 : a.upd_src[2 * u + 1];
        const double* A = a.L + (size_t)pa * dd + r * D;
        const double* B = a.L + (size_t)pb * dd + c0 * D;
        double ar[D];
#pragma unroll
        for (int k = 0; k < D; ++k) ar[k] = A[k];
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
          for (int k = 0; k < D; ++k) acc[c] = fma(-ar[k], B[c * D + k], acc[c]);
      }
    }
    const int ng = min(G, max(1, tk.z - tk.y));
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double tot = acc[c];
#pragma unroll
      for (int k = 1; k < G; ++k)
        if (k < ng) tot += __shfl_sync(kFull, acc[c], (r + k * D) & 31);
      if (lane < D) a.Spart[(size_t)slot * dd + lane * D + c0 + c] = tot;
    }
  } else {
    double acc = 0.0;
    if (g < G)
      for (int u = tk.y + g; u < tk.z; u += G) {
        const bool first = u == tk.y + g;
        const double* Lq = a.L + (size_t)(first ? x.u0 : a.row_blk[2 * u]) * dd + r * D;
        const double* yk = a.y + (size_t)(first ? x.u1 : a.row_blk[2 * u + 1]) * D;
#pragma unroll
        for (int k = 0; k < D; ++k) acc = fma(Lq[k], yk[k], acc);
      }
    const int ng = min(G, max(1, tk.z - tk.y));
    double tot = acc;
#pragma unroll
    for (int k = 1; k < G; ++k)
      if (k < ng) tot += __shfl_sync(kFull, acc, (r + k * D) & 31);
    if (lane < D) a.Spart[(size_t)slot * dd + lane * D] = tot;
  }
}

template <int D>
__device__ void run_task(const CholArgs& a, int t, int lane) {
  TaskAhead x;
  task_ahead<D>(a, t, lane, x);
  run_task_core<D>(a, x, lane);
}

// off-diagonal block p (row r) of S into s: the sum of its task partials, or
// its Hessian block when it has no update pairs (and no task)
template <int D>
__device__ __forceinline__ void sum_partials_r(const CholArgs& a, int p, int t0, int nt, int r, double (&s)[D]) {
  constexpr int dd = D * D;
  if (nt == 0) {
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = block_H<D>(a, p, false, r, c);
    return;
  }
#pragma unroll
  for (int c = 0; c < D; ++c) s[c] = 0.0;
  for (int t = t0; t < t0 + nt; ++t) {
    const double* P = a.Spart + (size_t)t * dd + r * D;
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] += P[c];
  }
}
template <int D>
__device__ __forceinline__ void sum_partials(const CholArgs& a, int p, int r, double (&s)[D]) {
  sum_partials_r<D>(a, p, a.btask[2 * p], a.btask[2 * p + 1], r, s);
}

// S_jj, the diagonal block of column j (block p), from its task partials,
// summed entry-wise: lane e holds entries e and e + 32, so a partial costs two
// FP64 additions instead of D; every entry is summed from 0 in slot order
// (the same additions as a row-wise sum). A block without update pairs (no
// task) is its Hessian block plus lambda D. Then moved to the lane-group row
// layout (lane r of every group gets row r).
template <int D>
__device__ __forceinline__ void diag_partials_r(const CholArgs& a, int p, int t0, int t1, int lane, int r,
                                                double (&C)[D]) {
  constexpr int dd = D * D;
  const bool has0 = lane < dd, has1 = lane + 32 < dd;
  double e0 = 0.0, e1 = 0.0;
  if (t1 == t0) {
    if (has0) e0 = block_H<D>(a, p, true, lane / D, lane % D);
    if (has1) e1 = block_H<D>(a, p, true, (lane + 32) / D, (lane + 32) % D);
  }
  for (int t = t0; t < t1; t += 4) {
    double x[4], y[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const double* P = a.Spart + (size_t)(t + k) * dd;
      x[k] = (t + k < t1 && has0) ? P[lane] : 0.0;
      y[k] = (t + k < t1 && has1) ? P[32 + lane] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (t + k < t1) {
        e0 += x[k];
        e1 += y[k];
      }
  }
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const int e = r * D + c;
    const double v0 = __shfl_sync(kFull, e0, e & 31), v1 = __shfl_sync(kFull, e1, e & 31);
    C[c] = e < 32 ? v0 : v1;
  }
}
template <int D>
__device__ __forceinline__ void diag_partials(const CholArgs& a, int j, int p, int lane, int r, double (&C)[D]) {
  const int t0 = a.btask[2 * p];
  diag_partials_r<D>(a, p, t0, t0 + a.btask[2 * p + 1], lane, r, C);
}

// In-register Cholesky of S_jj across a lane group (lane r holds row r, the
// group's lanes start at `base`), reciprocal pivots on the diagonal; a failed
// pivot of a group whose lanes have `mine` set sets *status.
template <int D>
__device__ __forceinline__ void factor_diag(const CholArgs& a, int lane, bool mine, int r, int base, double (&C)[D],
                                            int32_t* status) {
  bool ok = true;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    if (r == c) {
      double piv = C[c];
      if (!(piv > 0.0)) {
        ok = false;
        piv = 1.0;
      }
      C[c] = rsqrt(piv);
    }
    const double ilc = __shfl_sync(kFull, C[c], base + c);
    if (r > c) C[c] *= ilc;
#pragma unroll
    for (int q = c + 1; q < D; ++q) {
      const double lqc = __shfl_sync(kFull, C[c], base + q);
      if (r >= q) C[q] = fma(-C[c], lqc, C[q]);
    }
  }
  // the lane whose pivot failed flags its own group's system
  if (!ok && mine) set_fail(status);
}

// L_ij = S_ij L_jj^-T for one row r of an off-diagonal block, in place
// (right-looking), stored to block p when `st`
template <int D>
__device__ __forceinline__ void solve_offdiag(const CholArgs& a, int p, int r, const double (&Lf)[D * D],
                                              double (&sv)[D], bool st = true) {
  constexpr int dd = D * D;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const double x = sv[c] * Lf[c * D + c];
    sv[c] = x;
#pragma unroll
    for (int k = c + 1; k < D; ++k) sv[k] = fma(-x, Lf[k * D + c], sv[k]);
  }
  if (st) {
#pragma unroll
    for (int c = 0; c < D; ++c) a.L[(size_t)p * dd + r * D + c] = sv[c];
  }
}

// y_j - the forward-substitution row sums of column j (row r)
template <int D>
__device__ __forceinline__ double forward_rhs_r(const CholArgs& a, double b, int t0, int nt, int r) {
  constexpr int dd = D * D;
  double acc = 0.0;
  for (int t = t0; t < t0 + nt; ++t) acc += a.Spart[(size_t)t * dd + r * D];
  return b - acc;
}
template <int D>
__device__ __forceinline__ double forward_rhs(const CholArgs& a, int j, int r) {
  return forward_rhs_r<D>(a, a.y[(size_t)j * D + r], a.ftask[2 * j], a.ftask[2 * j + 1], r);
}

// y_j = L_jj^-1 b (lane r of a group holds b_r and row r of L_jj), stored
// by the lanes with `mine` set
template <int D>
__device__ __forceinline__ void forward_solve(const CholArgs& a, int j, bool mine, int r, int base,
                                              const double (&C)[D], double b) {
  double yv = 0.0;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    if (r == c) yv = b * C[c];
    const double yc = __shfl_sync(kFull, yv, base + c);
    if (r > c) b = fma(-C[c], yc, b);
  }
  if (mine) a.y[(size_t)j * D + r] = yv;
}

// phase B, one warp per column j: every lane group factors the diagonal
// block, the groups share the off-diagonal blocks L_ij = S_ij L_jj^-T, and
// group 0 does the column's forward substitution
template <int D>
__device__ void column_warp(const CholArgs& a, int j, int lane) {
  constexpr int G = 32 / D, dd = D * D;
  const int g = lane / D, r = lane % D;
  const bool grp = g < G;
  const int base = (grp ? g : 0) * D;
  if (!sys_on(a, j)) return;  // (warp-uniform)
  const int p0 = a.col_ptr[j], p1 = a.col_ptr[j + 1];
  double C[D];
  diag_partials<D>(a, j, p0, lane, r, C);
  factor_diag<D>(a, lane, g == 0, r, base, C, sys_status(a, j));
  double Lf[dd];
#pragma unroll
  for (int q = 0; q < D; ++q)
#pragma unroll
    for (int c = 0; c <= q; ++c) Lf[q * D + c] = __shfl_sync(kFull, C[c], base + q);
  if (g == 0) {
#pragma unroll
    for (int c = 0; c < D; ++c) a.Ldiag[(size_t)j * dd + r * D + c] = (c <= r) ? C[c] : 0.0;
  }
  if (grp) {
    for (int p = p0 + 1 + g; p < p1; p += G) {
      double sv[D];
      sum_partials<D>(a, p, r, sv);
      solve_offdiag<D>(a, p, r, Lf, sv);
    }
  }
  forward_solve<D>(a, j, g == 0, r, base, C, forward_rhs<D>(a, j, r));
}

__device__ __forceinline__ void team_sync(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }

// phase B for column j by a team of two warps (tw 0 = lead, 1 = helper) that
// meet at named barrier `bar`; sh = D x D + D doubles of shared memory. The
// lead sums and factors the diagonal block, publishes L_jj and does the
// forward substitution; meanwhile the helper sums the forward row sums and the
// partials of the off-diagonal blocks, and after the barrier solves those
// blocks with L_jj. Same operations and order as column_warp.
// The index chain of column j's phase-B team up to its first partial sum:
// block and slot ranges (the lead: the diagonal block's slots; the helper: its
// lane group's first off-diagonal block's slots and the row sums' slots).
// Plan data, so it is followed ahead of the level's task-phase barrier.
struct ColAhead {
  int j, p0, p1, t0, t1, f0, fn;
};
template <int D>
__device__ __forceinline__ void column_ahead(const CholArgs& a, int j, int tw, int lane, ColAhead& c) {
  const int g = lane / D;
  c.j = j;
  c.p0 = a.col_ptr[j];
  c.p1 = a.col_ptr[j + 1];
  if (tw == 0) {
    c.t0 = a.btask[2 * c.p0];
    c.t1 = c.t0 + a.btask[2 * c.p0 + 1];
    c.f0 = c.fn = 0;
  } else {
    const int pf = c.p0 + 1 + g;
    c.t0 = (g < 32 / D && pf < c.p1) ? a.btask[2 * pf] : 0;
    c.t1 = (g < 32 / D && pf < c.p1) ? a.btask[2 * pf + 1] : 0;
    c.f0 = a.ftask[2 * j];
    c.fn = a.ftask[2 * j + 1];
  }
}

template <int D>
__device__ void column_team_core(const CholArgs& a, const ColAhead& ca, int tw, int lane, int bar, double* sh) {
  constexpr int G = 32 / D, dd = D * D;
  const int g = lane / D, r = lane % D;
  const bool grp = g < G;
  const int base = (grp ? g : 0) * D;
  const int j = ca.j, p0 = ca.p0, p1 = ca.p1;
  if (!sys_on(a, j)) return;  // (both warps of the team: no named barrier)
  if (tw == 0) {
    double C[D];
    diag_partials_r<D>(a, p0, ca.t0, ca.t1, lane, r, C);
    factor_diag<D>(a, lane, g == 0, r, base, C, sys_status(a, j));
    if (g == 0) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const double v = (c <= r) ? C[c] : 0.0;
        a.Ldiag[(size_t)j * dd + r * D + c] = v;
        sh[r * D + c] = v;
      }
    }
    team_sync(bar);
    forward_solve<D>(a, j, g == 0, r, base, C, sh[dd + r]);
  } else {
    const double b = forward_rhs_r<D>(a, a.y[(size_t)j * D + r], ca.f0, ca.fn, r);
    if (g == 0) sh[dd + r] = b;
    const int pf = p0 + 1 + g;
    double sv[D];
    if (grp && pf < p1) sum_partials_r<D>(a, pf, ca.t0, ca.t1, r, sv);
    team_sync(bar);
    double Lf[dd];
#pragma unroll
    for (int q = 0; q < D; ++q)
#pragma unroll
      for (int c = 0; c <= q; ++c) Lf[q * D + c] = sh[q * D + c];
    if (grp) {
      for (int p = pf; p < p1; p += G) {
        if (p != pf) sum_partials<D>(a, p, r, sv);
        solve_offdiag<D>(a, p, r, Lf, sv);
      }
    }
  }
}

template <int D>
__device__ void column_team(const CholArgs& a, int j, int tw, int lane, int bar, double* sh) {
  ColAhead ca;
  column_ahead<D>(a, j, tw, lane, ca);
  column_team_core<D>(a, ca, tw, lane, bar, sh);
}

// phase A on wide levels: every lane group runs a task of its own (the
// groups of a warp take consecutive tasks), so one warp instruction serves
// up to G tasks. The operations and their order are run_task's: a block
// task's first pair continues the chain that starts at its Hessian block
// (kind 1) or zero, every further pair starts from zero and is added after
// its chain, in pair order (a task has at most G pairs, as the warp form
// gives each group one); a row task sums its entries in G interleaved
// chains (entry u in chain (u - first) mod G) added in chain order.
template <int D>
__device__ void run_task_group(const CholArgs& a, int t, bool valid, int r) {
  constexpr int G = 32 / D, dd = D * D;
  constexpr int NC = D == 6 ? 3 : D;
  int4 tk = reinterpret_cast<const int4*>(a.tasks)[t];
  const int kind = tk.w & 3, slot = tk.w >> 4;
  // groups without a task of a solved system run empty loops
  valid = valid && sys_on(a, kind < 2 ? a.blk_col[tk.x] : tk.x);
  if (!valid) tk.z = tk.y;
  if (kind < 2) {
    const int p = tk.x, c0 = ((tk.w >> 2) & 1) * NC;
    double tot[NC];
    if (kind == 1) {
      const bool diag = (tk.w >> 3) & 1;
#pragma unroll
      for (int c = 0; c < NC; ++c) tot[c] = block_H<D>(a, p, diag, r, c0 + c);
    } else {
#pragma unroll
      for (int c = 0; c < NC; ++c) tot[c] = 0.0;
    }
    for (int u = tk.y; u < tk.z; ++u) {
      const int pa = a.upd_src[2 * u], pb = a.upd_src[2 * u + 1];
      const double* A = a.L + (size_t)pa * dd + r * D;
      const double* B = a.L + (size_t)pb * dd + c0 * D;
      double ar[D];
#pragma unroll
      for (int k = 0; k < D; ++k) ar[k] = A[k];
      if (u == tk.y) {
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
          for (int k = 0; k < D; ++k) tot[c] = fma(-ar[k], B[c * D + k], tot[c]);
      } else {
        double acc[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          acc[c] = 0.0;
#pragma unroll
          for (int k = 0; k < D; ++k) acc[c] = fma(-ar[k], B[c * D + k], acc[c]);
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) tot[c] += acc[c];
      }
    }
    if (valid) {
#pragma unroll
      for (int c = 0; c < NC; ++c) a.Spart[(size_t)slot * dd + r * D + c0 + c] = tot[c];
    }
  } else {
    double tot = 0.0;
    const int n = tk.z - tk.y, ng = min(G, max(1, n));
    for (int g = 0; g < ng; ++g) {
      double acc = 0.0;
      for (int u = tk.y + g; u < tk.z; u += G) {
        const double* Lq = a.L + (size_t)a.row_blk[2 * u] * dd + r * D;
        const double* yk = a.y + (size_t)a.row_blk[2 * u + 1] * D;
#pragma unroll
        for (int k = 0; k < D; ++k) acc = fma(Lq[k], yk[k], acc);
      }
      tot = g == 0 ? acc : tot + acc;
    }
    if (valid) a.Spart[(size_t)slot * dd + r * D] = tot;
  }
}

// phase B on wide levels: every lane group finalises a column of its own
// (the groups of a warp take consecutive columns of the level): the
// operations and their order are column_warp's. Groups without a column
// (past the level's end, and the spare lanes of a warp) mirror the warp's
// first column and store nothing, so every lane takes part in the shuffles.
template <int D>
__device__ void column_group(const CholArgs& a, int c0, int nc, int w0, int lane) {
  constexpr int G = 32 / D, dd = D * D;
  const int g = lane / D, r = lane % D;
  const int w = w0 + (g < G ? g : 0);
  const int j = a.lvl_cols[c0 + ((g < G && w < nc) ? w : w0)];
  // groups without a column of a solved system run empty loops
  const bool mine = g < G && w < nc && sys_on(a, j);
  const int base = (g < G ? g : 0) * D;
  const int p0 = a.col_ptr[j], p1 = a.col_ptr[j + 1];
  // S_jj row r: every entry summed from 0 over the task slots in order, or
  // the Hessian block plus lambda D when the block has no task
  double C[D];
  {
    const int t0 = a.btask[2 * p0], t1 = t0 + (mine ? a.btask[2 * p0 + 1] : 0);
#pragma unroll
    for (int c = 0; c < D; ++c) C[c] = (t1 == t0) ? block_H<D>(a, p0, true, r, c) : 0.0;
    for (int t = t0; t < t1; ++t) {
      const double* P = a.Spart + (size_t)t * dd + r * D;
#pragma unroll
      for (int c = 0; c < D; ++c) C[c] += P[c];
    }
  }
  factor_diag<D>(a, lane, mine, r, base, C, sys_status(a, j));
  double Lf[dd];
#pragma unroll
  for (int q = 0; q < D; ++q)
#pragma unroll
    for (int c = 0; c <= q; ++c) Lf[q * D + c] = __shfl_sync(kFull, C[c], base + q);
  if (mine) {
#pragma unroll
    for (int c = 0; c < D; ++c) a.Ldiag[(size_t)j * dd + r * D + c] = (c <= r) ? C[c] : 0.0;
    for (int p = p0 + 1; p < p1; ++p) {
      double sv[D];
      sum_partials<D>(a, p, r, sv);
      solve_offdiag<D>(a, p, r, Lf, sv);
    }
  }
  forward_solve<D>(a, j, mine, r, base, C, mine ? forward_rhs<D>(a, j, r) : 0.0);
}

// The index chain of the backward substitution of column j (the column,
// its block range, the row of its lane group's first block): plan data, so a
// warp follows it for its column of the next (narrow) level ahead of the
// barrier, and after the barrier issues every value load of the column at
// once (its blocks, diagonal factor and y_j are final since the forward pass;
// only the solutions x_i come from the level above).
struct BackAhead {
  int j, q, q1, row;
};
template <int D>
__device__ __forceinline__ void backward_ahead(const CholArgs& a, int j, int lane, BackAhead& p) {
  constexpr int G = 32 / D;
  const int g = lane / D;
  p.j = j;
  p.q = a.col_ptr[j] + 1 + g;
  p.q1 = a.col_ptr[j + 1];
  p.row = (g < G && p.q < p.q1) ? a.blk_row[p.q] : 0;
}

// backward substitution of column j by one warp:
// x_j = L_jj^-T (y_j - sum L_ij^T x_i), the groups share the blocks
template <int D>
__device__ void backward_warp_core(const CholArgs& a, const BackAhead& p, int lane) {
  constexpr int G = 32 / D, dd = D * D;
  const int g = lane / D, r = lane % D;
  const int base = (g < G ? g : 0) * D;
  const int j = p.j;
  if (!sys_on(a, j)) return;  // (warp-uniform)
  double acc = 0.0;
  const int q0 = p.q - g, q1 = p.q1;
  if (g < G && p.q < q1) {
    const double* B0 = a.L + (size_t)p.q * dd + r;
    const double* xi = a.y + (size_t)p.row * D;
#pragma unroll
    for (int k = 0; k < D; ++k) acc = fma(B0[k * D], xi[k], acc);
    for (int q = p.q + G; q < q1; q += G) {
      const double* B = a.L + (size_t)q * dd + r;
      const double* xq = a.y + (size_t)a.blk_row[q] * D;
#pragma unroll
      for (int k = 0; k < D; ++k) acc = fma(B[k * D], xq[k], acc);
    }
  }
  const int ng = min(G, q1 - q0);
  double tot = acc;
#pragma unroll
  for (int k = 1; k < G; ++k)
    if (k < ng) tot += __shfl_sync(kFull, acc, (r + k * D) & 31);
  double b = a.y[(size_t)j * D + r] - tot;
  double Lc[D];
#pragma unroll
  for (int c = 0; c < D; ++c) Lc[c] = a.Ldiag[(size_t)j * dd + c * D + r];
  double xv = 0.0;
#pragma unroll
  for (int c = D - 1; c >= 0; --c) {
    if (r == c) xv = b * Lc[c];
    const double xc = __shfl_sync(kFull, xv, base + c);
    if (r < c) b = fma(-Lc[c], xc, b);
  }
  if (g == 0) a.y[(size_t)j * D + r] = xv;
}

template <int D>
__device__ void backward_warp(const CholArgs& a, int j, int lane) {
  BackAhead p;
  backward_ahead<D>(a, j, lane, p);
  backward_warp_core<D>(a, p, lane);
}

// backward substitution for wide levels: every lane group takes a column of
// its own (columns w0 + g of the level); lanes without a column (past the
// level's end, or the spare lanes of a warp) mirror the warp's first column
// and store nothing
template <int D>
__device__ void backward_groups(const CholArgs& a, int c0, int nc, int w0, int lane) {
  constexpr int G = 32 / D, dd = D * D;
  const int g = lane / D, r = lane % D;
  const int w = w0 + (g < G ? g : 0);
  const int j = a.lvl_cols[c0 + ((g < G && w < nc) ? w : w0)];
  // groups without a column of a solved system run an empty loop
  const bool mine = g < G && w < nc && sys_on(a, j);
  const int base = (g < G ? g : 0) * D;
  double acc = 0.0;
  const int q1 = mine ? a.col_ptr[j + 1] : 0;
  for (int q = a.col_ptr[j] + 1; q < q1; ++q) {
    const double* B = a.L + (size_t)q * dd + r;
    const double* xi = a.y + (size_t)a.blk_row[q] * D;
#pragma unroll
    for (int k = 0; k < D; ++k) acc = fma(B[k * D], xi[k], acc);
  }
  double b = a.y[(size_t)j * D + r] - acc;
  double Lc[D];
#pragma unroll
  for (int c = 0; c < D; ++c) Lc[c] = a.Ldiag[(size_t)j * dd + c * D + r];
  double xv = 0.0;
#pragma unroll
  for (int c = D - 1; c >= 0; --c) {
    if (r == c) xv = b * Lc[c];
    const double xc = __shfl_sync(kFull, xv, base + c);
    if (r < c) b = fma(-Lc[c], xc, b);
  }
  if (mine) a.y[(size_t)j * D + r] = xv;
}

__device__ __forceinline__ void tail_coords(int t, int& bi, int& bj) {
  int i = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > t) --i;
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  bi = i;
  bj = t - i * (i + 1) / 2;
}

// tail row task u (one warp, lane groups take the entries in turn):
// Tpart[u][r] = sum over its entries (block q, column k) of (L[q] y_k)[r]
template <int D>
__device__ void tail_row_task(const CholArgs& a, int u, int lane) {
  constexpr int G = 32 / D, dd = D * D;
  const int g = lane / D, r = lane % D;
  const int beg = a.ttasks[3 * u + 1], end = a.ttasks[3 * u + 2];
  double acc = 0.0;
  if (g < G)
    for (int e = beg + g; e < end; e += G) {
      const double* Lq = a.L + (size_t)a.trow_blk[2 * e] * dd + r * D;
      const double* yk = a.y + (size_t)a.trow_blk[2 * e + 1] * D;
#pragma unroll
      for (int k = 0; k < D; ++k) acc = fma(Lq[k], yk[k], acc);
    }
  const int ng = min(G, max(1, end - beg));
  double tot = acc;
#pragma unroll
  for (int k = 1; k < G; ++k)
    if (k < ng) tot += __shfl_sync(kFull, acc, (r + k * D) & 31);
  if (lane < D) a.Tpart[(size_t)u * D + lane] = tot;
}

// tail right-hand side: y_t -= the row task sums of tail block row t
template <int D>
__device__ void tail_rhs(const CholArgs& a, int t, int lane) {
  if (lane >= D) return;
  double acc = 0.0;
  for (int u = a.ttask_ptr[t]; u < a.ttask_ptr[t + 1]; ++u) acc += a.Tpart[(size_t)u * D + lane];
  a.y[(size_t)(a.ns + t) * D + lane] -= acc;
}

constexpr int kWarps = kThreads / 32;

struct TileSmem {
  double A[kTB][kTB + 1];
  double B[kTB][kTB + 1];
  double C[kTB][kTB + 1];
  double E[kTB][kTB + 1];
  double red[kThreads / kTB + 1][kTB];
  double v[kTB];
  double part[kWarps * 36 * 5];  // tail block partial sums: (warp, lane group) x D x D, D = 3 or 6
  double team[2][36 + 6];        // phase B teams: L_jj and the forward right-hand side
  ColAhead ahead[4][32];         // phase B teams (warps 1-4): index chains loaded ahead
  TaskAhead task[kWarps][32];    // narrow task phases: each warp's first task, loaded ahead
};

// S of tail block t into the dense tail, by one CTA: the lane groups of all
// warps take the block's update pairs in turn (group slot k = warp * G +
// group takes pairs k, k + W G, ...), then thread e < D x D adds entry e of
// the Hessian block (+ lambda D on the diagonal) and of the slots' partial
// sums, in slot order.
template <int D>
__device__ void tail_block_cta(const CholArgs& a, int t, TileSmem& s) {
  constexpr int G = 32 / D, dd = D * D;
  static_assert(kWarps * G * dd <= (int)(sizeof(s.part) / sizeof(double)), "tail partial buffer");
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const int g = lane / D, r = lane % D;
  int bi, bj;
  tail_coords(t, bi, bj);
  const int beg = a.tupd_ptr[t], end = a.tupd_ptr[t + 1];
  const int nslots = min(kWarps * G, end - beg);
  const int slot = wi * G + g;
  if (g < G && slot < nslots) {
    double acc[D];
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = 0.0;
    for (int u = beg + slot; u < end; u += kWarps * G) {
      const double* A = a.L + (size_t)a.tupd_src[2 * u] * dd + r * D;
      const double* B = a.L + (size_t)a.tupd_src[2 * u + 1] * dd;
      double ar[D];
#pragma unroll
      for (int k = 0; k < D; ++k) ar[k] = A[k];
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int k = 0; k < D; ++k) acc[c] = fma(-ar[k], B[c * D + k], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < D; ++c) s.part[slot * dd + r * D + c] = acc[c];
  }
  __syncthreads();
  if (threadIdx.x < dd) {
    const int e = threadIdx.x, rr = e / D, cc = e % D;
    double v = bi == bj ? gather_diag<D>(a, a.perm[a.ns + bi], rr, cc)
                        : gather_offdiag<D>(a.fH64, a.ta_src, a.ta_ptr[t], a.ta_ptr[t + 1], rr, cc);
    for (int k = 0; k < nslots; ++k) v += s.part[k * dd + e];
    a.M[(size_t)(bj * D + cc) * a.ntp + bi * D + rr] = v;
  }
  __syncthreads();
}

__device__ __forceinline__ double* tile_ptr(const CholArgs& a, int ti, int tj) {
  return a.M + (size_t)(tj * kTB) * a.ntp + ti * kTB;
}

__device__ void load_tile(const CholArgs& a, int ti, int tj, double (*S)[kTB + 1]) {
  const double* P = tile_ptr(a, ti, tj);
  for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
    const int r = e % kTB, c = e / kTB;
    S[r][c] = P[(size_t)c * a.ntp + r];
  }
}

__device__ __forceinline__ double tile_dot(const double* __restrict__ p, const double* __restrict__ q) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int t = 0; t < kTB; ++t) acc[t & 3] = fma(p[t], q[t], acc[t & 3]);
  return (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

// X[r][c] -= sum_t P[r][t] Q[c][t] (lower part only when lower_only)
__device__ void smem_update(double (*X)[kTB + 1], double (*P)[kTB + 1], double (*Q)[kTB + 1], bool lower_only) {
  for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
    const int r = e % kTB, c = e / kTB;
    if (lower_only && c > r) continue;
    X[r][c] -= tile_dot(P[r], Q[c]);
  }
}

// Cholesky of the lower part of X in place (right-looking); the diagonal
// keeps the reciprocal of each pivot. Columns from `width` on are padding of
// the last tile (identity: pivot 1, reciprocal 1, no updates) and are skipped.
__device__ void smem_chol(double (*X)[kTB + 1], int width, int32_t* status) {
  for (int c = 0; c < width; ++c) {
    if (threadIdx.x == 0) {
      double piv = X[c][c];
      if (!(piv > 0.0)) {
        set_fail(status);
        piv = 1.0;
      }
      X[c][c] = rsqrt(piv);
    }
    __syncthreads();
    const double il = X[c][c];
    for (int r = c + 1 + threadIdx.x; r < kTB; r += blockDim.x) X[r][c] *= il;
    __syncthreads();
    const int m = kTB - c - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int r = c + 1 + e % m, q = c + 1 + e / m;
      if (q <= r) X[r][q] = fma(-X[r][c], X[q][c], X[r][q]);
    }
    __syncthreads();
  }
}

// phase k, tile column item: tile (i, k), i >= k; nt = tail size in scalars
__device__ void tail_column_item(const CholArgs& a, int i, int k, int nt, TileSmem& s) {
  load_tile(a, k, k, s.C);
  if (k > 0) load_tile(a, k, k - 1, s.B);
  if (i > k) {
    load_tile(a, i, k, s.A);
    if (k > 0) load_tile(a, i, k - 1, s.E);
  }
  __syncthreads();
  if (k > 0) {
    smem_update(s.C, s.B, s.B, true);
    if (i > k) smem_update(s.A, s.E, s.B, false);
  }
  __syncthreads();
  smem_chol(s.C, min(kTB, nt - k * kTB), a.status);
  if (i == k) {
    double* O = a.Ldd + (size_t)k * kTB * kTB;
    for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
      const int r = e / kTB, c = e % kTB;
      O[e] = (c <= r) ? s.C[r][c] : 0.0;
    }
  } else {
    // row r of the tile: x = A[r] L^-T, right-looking (independent updates)
    if (threadIdx.x < kTB) {
      const int r = threadIdx.x;
      for (int c = 0; c < kTB; ++c) {
        const double x = s.A[r][c] * s.C[c][c];
        s.A[r][c] = x;
        for (int k = c + 1; k < kTB; ++k) s.A[r][k] = fma(-x, s.C[k][c], s.A[r][k]);
      }
    }
    __syncthreads();
    double* P = tile_ptr(a, i, k);
    for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
      const int r = e % kTB, c = e / kTB;
      P[(size_t)c * a.ntp + r] = s.A[r][c];
    }
  }
  __syncthreads();
}

// phase k >= 1, trailing item: tile (i, j), j >= k + 1, updated by column k - 1
__device__ void tail_trailing_item(const CholArgs& a, int i, int j, int k, TileSmem& s) {
  load_tile(a, i, k - 1, s.A);
  load_tile(a, j, k - 1, s.B);
  __syncthreads();
  double* P = tile_ptr(a, i, j);
  for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
    const int r = e % kTB, c = e / kTB;
    if (i == j && c > r) continue;
    P[(size_t)c * a.ntp + r] -= tile_dot(s.A[r], s.B[c]);
  }
  __syncthreads();
}

// forward substitution of tail tile k (left-looking):
// y_k = Ldd_k^-1 (y_k - sum_{j<k} L(k, j) y_j); yt = tail segment of y
__device__ void tail_forward_item(const CholArgs& a, double* yt, int k, TileSmem& s) {
  constexpr int chunks = kThreads / kTB;
  const int ncol = k * kTB;
  if (threadIdx.x < chunks * kTB) {
    const int r = threadIdx.x % kTB, ch = threadIdx.x / kTB;
    double acc0 = 0.0, acc1 = 0.0;
    const double* P = a.M + k * kTB + r;
    int c = ch;
    for (; c + chunks < ncol; c += 2 * chunks) {
      acc0 = fma(P[(size_t)c * a.ntp], yt[c], acc0);
      acc1 = fma(P[(size_t)(c + chunks) * a.ntp], yt[c + chunks], acc1);
    }
    if (c < ncol) acc0 = fma(P[(size_t)c * a.ntp], yt[c], acc0);
    s.red[ch][r] = acc0 + acc1;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double b = 0.0;
    if (lane < kTB) {
      b = yt[k * kTB + lane];
      for (int ch = 0; ch < chunks; ++ch) b -= s.red[ch][lane];
    }
    const double* Lk = a.Ldd + (size_t)k * kTB * kTB;
    double yv = 0.0;
    for (int c = 0; c < kTB; ++c) {
      if (lane == c) yv = b * Lk[c * kTB + c];
      const double yc = __shfl_sync(0xffffffffu, yv, c);
      if (lane > c && lane < kTB) b = fma(-Lk[lane * kTB + c], yc, b);
    }
    if (lane < kTB) yt[k * kTB + lane] = yv;
  }
  __syncthreads();
}

// backward substitution of tail tile k (left-looking):
// x_k = Ldd_k^-T (y_k - sum_{i>k} L(i, k)^T x_i), in place over y
__device__ void tail_backward_item(const CholArgs& a, double* yt, int k, TileSmem& s) {
  constexpr int chunks = kThreads / kTB;
  const int r0 = (k + 1) * kTB;
  if (threadIdx.x < chunks * kTB) {
    const int c = threadIdx.x % kTB, ch = threadIdx.x / kTB;
    double acc0 = 0.0, acc1 = 0.0;
    const double* P = a.M + (size_t)(k * kTB + c) * a.ntp;
    int r = r0 + ch;
    for (; r + chunks < a.ntp; r += 2 * chunks) {
      acc0 = fma(P[r], yt[r], acc0);
      acc1 = fma(P[r + chunks], yt[r + chunks], acc1);
    }
    if (r < a.ntp) acc0 = fma(P[r], yt[r], acc0);
    s.red[ch][c] = acc0 + acc1;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double b = 0.0;
    if (lane < kTB) {
      b = yt[k * kTB + lane];
      for (int ch = 0; ch < chunks; ++ch) b -= s.red[ch][lane];
    }
    const double* Lk = a.Ldd + (size_t)k * kTB * kTB;
    double xv = 0.0;
    for (int c = kTB - 1; c >= 0; --c) {
      if (lane == c) xv = b * Lk[c * kTB + c];
      const double xc = __shfl_sync(0xffffffffu, xv, c);
      if (lane < c) b = fma(-Lk[c * kTB + lane], xc, b);
    }
    if (lane < kTB) yt[k * kTB + lane] = xv;
  }
  __syncthreads();
}

__device__ __forceinline__ double cta_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < nw; ++i) t += sh[i];
  return t;
}

template <int D>
__global__ void __launch_bounds__(kThreads) k_chol_solve(CholArgs a) {
  cg::grid_group grid = cg::this_grid();
  __shared__ TileSmem sm;
  __shared__ double shr[kThreads / 32];
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  // Warp-sized work items (tasks, columns) go round-robin over the CTAs, so
  // that a level with fewer items than SMs puts one item per SM (no two
  // items share an SM's FP64 pipe), and to warps 1..7 before warp 0: the
  // warp whose thread 0 takes part in the grid barrier runs the phase after
  // it about 2.5 us slower (measured on GB300), so it only takes the items
  // of the widest levels.
  const int gw = (((threadIdx.x >> 5) + kWarps - 1) % kWarps) * (int)gridDim.x + (int)blockIdx.x, nw = gs >> 5;
  const int n = a.N * D, nt = a.T * D;
  double* yt = a.y + (size_t)a.ns * D;

  // 1. init
  if (gt == 0) *a.status = 0;
  for (int k = gt; k < a.G; k += gs) a.b_status[k] = 0;
  for (int k = gt; k < n; k += gs) {
    const int pos = k / D, r = k % D;
    a.y[k] = -a.g[(size_t)a.perm[pos] * D + r];
  }
  for (int k = nt + gt; k < a.ntp; k += gs) yt[k] = 0.0;
  {
    // padded rows / columns of the tail: identity
    const int pad = a.ntp - nt;
    for (int e = gt; e < pad * a.ntp; e += gs) {
      const int c = e / a.ntp, r = e % a.ntp;  // column nt + c, any row; and row nt + c, columns < nt
      a.M[(size_t)(nt + c) * a.ntp + r] = (r == nt + c) ? 1.0 : 0.0;
      if (r < nt) a.M[(size_t)r * a.ntp + nt + c] = 0.0;
    }
  }
  grid.sync();

  // 2. sparse levels: (A) the level's tasks over all warps, (B) its
  // columns, one warp or a two-warp team each; one barrier after each
  // a narrow level's phase B: at most two columns per CTA, each by a team of
  // two warps (warps 1-2 and 3-4, on four different SM sub-partitions)
  const int wi = threadIdx.x >> 5;
  const int team_slot = (wi - 1) >> 1;
  const int team_w = team_slot * (int)gridDim.x + (int)blockIdx.x;
  bool task_ready = false;  // sm.task[wi][lane] holds this warp's first task of level l
  for (int l = 0; l < a.levels; ++l) {
    const int t0 = a.lvl_task_ptr[l], t1 = task_end(a, l);
    const int c0 = a.lvl_col_ptr[l], nc = col_end(a, l) - c0;
    const bool narrow = nc < kGroupModeItems * nw && nc <= 2 * (int)gridDim.x;
    const bool team = narrow && wi >= 1 && wi <= 4 && team_w < nc;
    if (t1 > t0) {  // (the leaves' level has none: no updates, no row sums)
      if (t1 - t0 >= kGroupModeItems * nw) {
        // wide: a task per lane group
        constexpr int G = 32 / D;
        const int g = lane / D;
        for (int w = gw * G; w < t1 - t0; w += nw * G) {
          const int t = w + (g < G ? g : 0);
          const bool valid = g < G && t < t1 - t0;
          run_task_group<D>(a, t0 + (valid ? t : w), valid, lane % D);
        }
      } else {
        for (int t = t0 + gw; t < t1; t += nw) {
          if (t == t0 + gw && task_ready) run_task_core<D>(a, sm.task[wi][lane], lane);
          else run_task<D>(a, t, lane);
        }
      }
      // the team's index chain for phase B, ahead of the barrier (through
      // shared memory: held in registers it would raise the kernel's
      // register count above two CTAs per SM)
      if (team) column_ahead<D>(a, a.lvl_cols[c0 + team_w], (wi - 1) & 1, lane, sm.ahead[wi - 1][lane]);
      grid.sync();
    }
    if (nc >= kGroupModeItems * nw) {
      // wide: a column per lane group
      constexpr int G = 32 / D;
      for (int w = gw * G; w < nc; w += nw * G) column_group<D>(a, c0, nc, w, lane);
    } else if (narrow) {
      if (team) {
        ColAhead ca;
        if (t1 > t0) ca = sm.ahead[wi - 1][lane];
        else column_ahead<D>(a, a.lvl_cols[c0 + team_w], (wi - 1) & 1, lane, ca);
        column_team_core<D>(a, ca, (wi - 1) & 1, lane, 1 + team_slot, sm.team[team_slot]);
      }
    } else {
      for (int w = gw; w < nc; w += nw) column_warp<D>(a, a.lvl_cols[c0 + w], lane);
    }
    // the warp's first task of the next level (narrow task phases), ahead of
    // the barrier, through shared memory
    task_ready = false;
    if (l + 1 < a.levels) {
      const int u0 = a.lvl_task_ptr[l + 1], u1 = task_end(a, l + 1);
      if (u1 > u0 && u1 - u0 < kGroupModeItems * nw && u0 + gw < u1) {
        task_ahead<D>(a, u0 + gw, lane, sm.task[wi][lane]);
        task_ready = true;
      }
    }
    grid.sync();
  }

  // 3. dense tail: its blocks (one CTA each) and the row sums of its
  // right-hand side (one warp each, on the CTAs after the blocks'), then the
  // tiles
  {
    const int nts = a.T * (a.T + 1) / 2, ntr = a.ttask_ptr[a.T];
    for (int b = blockIdx.x; b < nts; b += gridDim.x) tail_block_cta<D>(a, b, sm);
    for (int w = gw; w < nts + ntr; w += nw)
      if (w >= nts) tail_row_task<D>(a, w - nts, lane);
  }
  grid.sync();
  const int nT = a.n_tiles;
  if (nT == 1) {
    // a single tile: one CTA takes the tail's right-hand side, its
    // factorisation and both substitutions, in one phase
    if (blockIdx.x == 0) {
      for (int w = threadIdx.x >> 5; w < a.T; w += kWarps) tail_rhs<D>(a, w, lane);
      __syncthreads();
      tail_column_item(a, 0, 0, nt, sm);
      tail_forward_item(a, yt, 0, sm);
      tail_backward_item(a, yt, 0, sm);
    }
    grid.sync();
  }
  for (int k = 0; nT > 1 && k <= nT; ++k) {
    const int ncol = k < nT ? nT - k : 0;
    const int m = nT - k - 1;  // trailing tile columns k + 1 .. nT - 1
    const int ntrail = (k >= 1 && m > 0) ? m * (m + 1) / 2 : 0;
    const int nfwd = k >= 1 ? 1 : 0;
    const int items = ncol + ntrail + nfwd;
    for (int it = blockIdx.x; it < items; it += gridDim.x) {
      if (it < ncol) {
        tail_column_item(a, k + it, k, nt, sm);
      } else if (it < ncol + ntrail) {
        // trailing tile u -> (i, j), k + 1 <= j <= i <= nT - 1
        const int u = it - ncol;
        int ii, jj;
        tail_coords(u, ii, jj);
        tail_trailing_item(a, k + 1 + ii, k + 1 + jj, k, sm);
      } else {
        tail_forward_item(a, yt, k - 1, sm);
      }
    }
    if (k == 0)
      for (int w = gw; w < a.T; w += nw) tail_rhs<D>(a, w, lane);
    grid.sync();
  }

  // 4. backward substitution: tail tiles (several), then sparse levels (top first)
  for (int k = nT - 1; nT > 1 && k >= 0; --k) {
    if (blockIdx.x == (unsigned)(k % gridDim.x)) tail_backward_item(a, yt, k, sm);
    grid.sync();
  }
  // a narrow level has at most one column per warp (warps 1..7 take them):
  // the warp's column of the next level is loaded ahead of each barrier
  BackAhead back;
  int back_l = -1;  // the level whose column `back` holds
  for (int l = a.levels - 1; l >= 0; --l) {
    const int c0 = a.lvl_col_ptr[l], nc = col_end(a, l) - c0;
    if (nc <= (kWarps - 1) * (int)gridDim.x) {
      if (gw < nc) {
        if (back_l == l) backward_warp_core<D>(a, back, lane);
        else backward_warp<D>(a, a.lvl_cols[c0 + gw], lane);
      }
    } else {
      // more columns than warps 1..7 of the grid: G columns per warp instead
      // of a second round
      constexpr int G = 32 / D;
      for (int w = gw; w * G < nc; w += nw) backward_groups<D>(a, c0, nc, w * G, lane);
    }
    if (l > 0) {
      const int c1 = a.lvl_col_ptr[l - 1], n1 = col_end(a, l - 1) - c1;
      if (n1 <= (kWarps - 1) * (int)gridDim.x && gw < n1) {
        backward_ahead<D>(a, a.lvl_cols[c1 + gw], lane, back);
        back_l = l - 1;
      }
    }
    grid.sync();
  }
  // scatter to variable order, with the linearised cost change of the
  // undamped system: since (H + lambda D) delta = -g, -g.delta - delta^T H
  // delta / 2 = -g.delta / 2 + lambda delta^T D delta / 2
  if (a.G > 0) {
    // several systems: per-position partials, then one warp per system adds
    // its positions in a fixed order (lane-strided chains, then a fixed tree)
    for (int pos = gt; pos < a.N; pos += gs) {
      if (!sys_on(a, pos)) continue;
      double pg = 0.0, pq = 0.0;
#pragma unroll
      for (int r = 0; r < D; ++r) {
        const size_t vi = (size_t)a.perm[pos] * D + r;
        const double x = a.y[(size_t)pos * D + r];
        a.delta[vi] = x;
        pg = fma(a.g[vi], x, pg);
        pq = fma(a.dampD[vi] * x, x, pq);
      }
      a.b_term[2 * pos] = pg;
      a.b_term[2 * pos + 1] = pq;
    }
    grid.sync();
    for (int sy = gw; sy < a.G; sy += nw) {
      if (!(a.b_act[sy] & 1)) continue;
      double sg = 0.0, sq = 0.0;
      for (int pos = a.b_off[sy] + lane; pos < a.b_off[sy + 1]; pos += 32) {
        sg += a.b_term[2 * pos];
        sq += a.b_term[2 * pos + 1];
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        sg += __shfl_xor_sync(kFull, sg, o);
        sq += __shfl_xor_sync(kFull, sq, o);
      }
      if (lane == 0) {
        a.b_out[2 * sy] = -0.5 * sg + 0.5 * a.b_lam[sy] * sq;
        a.b_out[2 * sy + 1] = (double)atomicAdd(a.b_status + sy, 0);
      }
    }
    return;
  }
  double gd = 0.0, dq = 0.0;
  for (int k = gt; k < n; k += gs) {
    const int pos = k / D, r = k % D;
    const size_t vi = (size_t)a.perm[pos] * D + r;
    const double x = a.y[k];
    a.delta[vi] = x;
    gd = fma(a.g[vi], x, gd);
    dq = fma(a.dampD[vi] * x, x, dq);
  }
  gd = cta_sum(gd, shr);
  dq = cta_sum(dq, shr);
  if (threadIdx.x == 0) {
    a.part[2 * blockIdx.x] = gd;
    a.part[2 * blockIdx.x + 1] = dq;
  }
  grid.sync();
  if (blockIdx.x == 0 && threadIdx.x < 32) {
    double sg = 0.0, sq = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) {
      sg += a.part[2 * b];
      sq += a.part[2 * b + 1];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      sg += __shfl_xor_sync(kFull, sg, o);
      sq += __shfl_xor_sync(kFull, sq, o);
    }
    if (threadIdx.x == 0) {
      a.out[0] = -0.5 * sg + 0.5 * a.lam * sq;
      // every block's pivot failures were flagged before the last barrier
      a.out[1] = (double)atomicAdd(a.status, 0);
    }
  }
}

// H (and the damping diagonal, on diagonal blocks) in the factor's block
// layout, once per linearisation: thread per block row; an off-diagonal
// block sums its factors' blocks in the plan's order (each entry the same
// additions as gather_offdiag).
template <int D>
__global__ void k_block_hessian(int nblk, const int32_t* __restrict__ blk_row, const int32_t* __restrict__ blk_col,
                                const int32_t* __restrict__ perm, const int32_t* __restrict__ a_ptr,
                                const int32_t* __restrict__ a_src, const double* __restrict__ Hd64,
                                const double* __restrict__ fH64, const double* __restrict__ dampD,
                                double* __restrict__ Hs, double* __restrict__ dampS,
                                const uint8_t* __restrict__ mask) {
  constexpr int dd = D * D;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)nblk * D) return;
  const int p = (int)(t / D), r = (int)(t % D);
  const int j = blk_col[p];
  if (mask && !(mask[j] & 1)) return;  // (a joint batch's graph not in this round)
  double* out = Hs + (size_t)p * dd + r * D;
  if (blk_row[p] == j) {
    const int v = perm[j];
#pragma unroll
    for (int c = 0; c < D; ++c) out[c] = Hd64[(size_t)v * dd + r * D + c];
    dampS[(size_t)p * D + r] = dampD[(size_t)v * D + r];
  } else {
    double acc[D];
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = 0.0;
    for (int u = a_ptr[p]; u < a_ptr[p + 1]; ++u) {
      const int32_t x = a_src[u];
      const double* H = fH64 + (size_t)(x >> 1) * 3 * dd + 2 * dd;
#pragma unroll
      for (int c = 0; c < D; ++c) acc[c] += (x & 1) ? H[c * D + r] : H[r * D + c];
    }
#pragma unroll
    for (int c = 0; c < D; ++c) out[c] = acc[c];
  }
}

// Joint batch: the items (tasks, columns) of the graphs in the round, per
// level, in plan order. Chunks never straddle a level (chunk table from the
// plan). Pass 1 counts each chunk's active items; pass 2 places each chunk at
// its level's start plus the counts of the level's earlier chunks and writes
// its active items in order (a block-wide scan); pass 3 writes every level's
// end.
constexpr int kCompactThreads = 256;

__device__ __forceinline__ bool task_active(const int4& tk, const int32_t* __restrict__ blk_col,
                                            const int32_t* __restrict__ vsys, const uint8_t* __restrict__ ctl) {
  const int pos = (tk.w & 3) < 2 ? blk_col[tk.x] : tk.x;
  return ctl[vsys[pos]] & 1;
}

// kind 0: tasks (int4 items), 1: columns (int items)
template <int KIND>
__global__ void k_compact_count(const int4* __restrict__ chunks, const int4* __restrict__ tasks,
                                const int32_t* __restrict__ cols, const int32_t* __restrict__ blk_col,
                                const int32_t* __restrict__ vsys, const uint8_t* __restrict__ ctl,
                                int32_t* __restrict__ counts) {
  __shared__ int sh[kCompactThreads / 32];
  const int4 ch = chunks[blockIdx.x];  // (level, begin, end, first chunk of the level)
  int c = 0;
  for (int i = ch.y + threadIdx.x; i < ch.z; i += blockDim.x)
    c += KIND == 0 ? task_active(tasks[i], blk_col, vsys, ctl) : (ctl[vsys[cols[i]]] & 1);
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kCompactThreads / 32; ++w) t += sh[w];
    counts[blockIdx.x] = t;
  }
}

template <int KIND>
__global__ void k_compact_scatter(const int4* __restrict__ chunks, const int32_t* __restrict__ lvl_ptr,
                                  const int4* __restrict__ tasks, const int32_t* __restrict__ cols,
                                  const int32_t* __restrict__ blk_col, const int32_t* __restrict__ vsys,
                                  const uint8_t* __restrict__ ctl, const int32_t* __restrict__ counts,
                                  int4* __restrict__ tasks_c, int32_t* __restrict__ cols_c) {
  __shared__ int sh[kCompactThreads / 32];
  __shared__ int base;
  const int4 ch = chunks[blockIdx.x];
  if (threadIdx.x == 0) {
    int o = lvl_ptr[ch.x];
    for (int k = ch.w; k < (int)blockIdx.x; ++k) o += counts[k];
    base = o;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i0 = ch.y; i0 < ch.z; i0 += blockDim.x) {
    const int i = i0 + threadIdx.x;
    bool on = false;
    if (i < ch.z) on = KIND == 0 ? task_active(tasks[i], blk_col, vsys, ctl) : (ctl[vsys[cols[i]]] & 1);
    const unsigned m = __ballot_sync(0xffffffffu, on);
    if (lane == 0) sh[warp] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < kCompactThreads / 32; ++w) {
      before += w < warp ? sh[w] : 0;
      total += sh[w];
    }
    if (on) {
      const int o = base + before + __popc(m & ((1u << lane) - 1u));
      if (KIND == 0) tasks_c[o] = tasks[i];
      else cols_c[o] = cols[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
}

__global__ void k_compact_ends(int levels, const int32_t* __restrict__ lvl_ptr,
                               const int32_t* __restrict__ level_chunks, const int32_t* __restrict__ counts,
                               int32_t* __restrict__ ends) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= levels) return;
  int e = lvl_ptr[l];
  for (int k = level_chunks[l]; k < level_chunks[l + 1]; ++k) e += counts[k];
  ends[l] = e;
}

}  // namespace

void CholDev::upload(CholPlan&& p, cudaStream_t st) {
  plan = std::move(p);
  levels = plan.levels();
  if (plan.tile != kTB) throw std::logic_error("chol plan tile size differs from the kernel's");
  perm.upload(plan.perm, st);
  col_ptr.upload(plan.col_ptr, st);
  blk_row.upload(plan.blk_row, st);
  blk_col.upload(plan.blk_col, st);
  lvl_col_ptr.upload(plan.lvl_col_ptr, st);
  lvl_cols.upload(plan.lvl_cols, st);
  lvl_task_ptr.upload(plan.lvl_task_ptr, st);
  tasks.upload(plan.tasks, st);
  btask.upload(plan.btask, st);
  ftask.upload(plan.ftask, st);
  Spart.resize(std::max<size_t>(1, (size_t)plan.n_slots * plan.d * plan.d));
  upd_ptr.upload(plan.upd_ptr, st);
  upd_src.upload(plan.upd_src, st);
  tupd_ptr.upload(plan.tupd_ptr, st);
  tupd_src.upload(plan.tupd_src, st);
  a_ptr.upload(plan.a_ptr, st);
  a_src.upload(plan.a_src, st);
  ta_ptr.upload(plan.ta_ptr, st);
  ta_src.upload(plan.ta_src, st);
  row_ptr.upload(plan.row_ptr, st);
  row_blk.upload(plan.row_blk, st);
  trow_ptr.upload(plan.trow_ptr, st);
  trow_blk.upload(plan.trow_blk, st);
  ttasks.upload(plan.ttasks, st);
  ttask_ptr.upload(plan.ttask_ptr, st);
  Tpart.resize(std::max<size_t>(1, plan.ttasks.size() / 3 * (size_t)plan.d));
  const size_t dd = (size_t)plan.d * plan.d, ntp = (size_t)plan.n_tiles * kTB;
  L.resize(std::max<size_t>(1, plan.blk_row.size() * dd));
  Hs.resize(std::max<size_t>(1, plan.blk_row.size() * dd));
  dampS.resize(std::max<size_t>(1, plan.blk_row.size() * plan.d));
  Ldiag.resize(std::max<size_t>(1, (size_t)plan.n_sparse * dd));
  M.resize(std::max<size_t>(1, ntp * ntp));
  Ldd.resize(std::max<size_t>(1, (size_t)plan.n_tiles * kTB * kTB));
  y.resize((size_t)plan.n_sparse * plan.d + ntp + 1);
  out.resize(4);
  status.resize(1);
}

CholDev::~CholDev() {
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
}

void chol_block_hessian(SolverDev& s, CholDev& c, cudaStream_t st, const uint8_t* mask) {
  const int nblk = (int)c.plan.blk_row.size();
  if (nblk == 0) return;
  const int tb = 256;
  const int64_t n = (int64_t)nblk * c.plan.d;
  if (s.dim == 3)
    k_block_hessian<6><<<div_up(n, tb), tb, 0, st>>>(nblk, c.blk_row.get(), c.blk_col.get(), c.perm.get(),
                                                    c.a_ptr.get(), c.a_src.get(), s.Hd64.get(), s.fH64.get(),
                                                    s.dampD.get(), c.Hs.get(), c.dampS.get(), mask);
  else
    k_block_hessian<3><<<div_up(n, tb), tb, 0, st>>>(nblk, c.blk_row.get(), c.blk_col.get(), c.perm.get(),
                                                    c.a_ptr.get(), c.a_src.get(), s.Hd64.get(), s.fH64.get(),
                                                    s.dampD.get(), c.Hs.get(), c.dampS.get(), mask);
  RPGO_LAUNCHED();
}

// CTAs of the cooperative solve: every co-resident CTA (two per SM at 256
// threads x 128 registers: twice the warps per SM to hide the latency of the
// wide levels' loads), or the caller's budget
static int chol_grid(const SolverDev& s) {
  static const int per_sm[2] = {
      [] {
        int n = 0;
        RPGO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_chol_solve<3>, kThreads, 0));
        return std::max(1, n);
      }(),
      [] {
        int n = 0;
        RPGO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_chol_solve<6>, kThreads, 0));
        return std::max(1, n);
      }()};
  const int most = device_sm_count() * per_sm[s.dim == 3 ? 1 : 0];
  return s.coop_ctas > 0 ? std::min(s.coop_ctas, most) : most;
}

// kernel arguments of one solve (one system; the joint batch adds its own)
static CholArgs make_args(SolverDev& s, CholDev& c, double lambda) {
  const CholPlan& p = c.plan;
  CholArgs a{s.N, p.n_sparse, p.T, p.n_tiles * kTB, p.n_tiles, c.levels,
             c.perm.get(), c.col_ptr.get(), c.blk_row.get(), c.blk_col.get(), c.lvl_col_ptr.get(), c.lvl_cols.get(),
             c.lvl_task_ptr.get(), c.tasks.get(), c.btask.get(), c.ftask.get(), c.upd_ptr.get(), c.upd_src.get(), c.tupd_ptr.get(),
             c.tupd_src.get(), c.a_ptr.get(), c.a_src.get(), c.ta_ptr.get(), c.ta_src.get(), c.row_ptr.get(),
             c.row_blk.get(), c.trow_ptr.get(), c.trow_blk.get(), c.ttasks.get(), c.ttask_ptr.get(), s.Hd64.get(), s.fH64.get(), s.dampD.get(),
             s.g.get(), lambda, c.L.get(), c.Ldiag.get(),
             c.M.get(), c.Ldd.get(), c.y.get(), s.delta.get(), c.part.get(), c.out.get(), c.Spart.get(), c.Tpart.get(),
             c.Hs.get(), c.dampS.get(), c.status.get()};
  a.G = 0;
  a.b_sys = a.b_off = nullptr;
  a.b_act = nullptr;
  a.b_lam = nullptr;
  a.b_status = nullptr;
  a.b_out = a.b_term = nullptr;
  a.b_compact = 0;
  a.lvl_task_end = a.lvl_col_end = nullptr;
  return a;
}

void chol_enqueue(SolverDev& s, CholDev& c, double lambda, cudaStream_t st, double* host) {
  if (s.N == 0) {
    host[0] = 0.0;
    host[1] = 0.0;
    return;
  }
  if (!c.ev[0]) {
    RPGO_CUDA(cudaEventCreate(&c.ev[0]));
    RPGO_CUDA(cudaEventCreate(&c.ev[1]));
  }
  const int grid = chol_grid(s);
  c.part.resize((size_t)2 * grid);
  CholArgs a = make_args(s, c, lambda);
  void* args[] = {&a};
  RPGO_CUDA(cudaEventRecord(c.ev[0], st));
  if (s.dim == 3)
    RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_chol_solve<6>, grid, kThreads, args, 0, st));
  else
    RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_chol_solve<3>, grid, kThreads, args, 0, st));
  RPGO_LAUNCHED();
  RPGO_CUDA(cudaEventRecord(c.ev[1], st));
  RPGO_CUDA(cudaMemcpyAsync(host, c.out.get(), 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
}

SolveOut chol_finish(SolverDev& s, CholDev& c, const double* host) {
  SolveOut o;
  if (s.N == 0) {
    o.ok = 1;
    return o;
  }
  float ms = 0.f;
  RPGO_CUDA(cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]));
  const CholPlan& p = c.plan;
  kernel_times().chol_ms += ms;
  kernel_times().chol_launches += 1;
  kernel_times().chol_flops += p.flops;
  kernel_times().chol_bytes += p.bytes;
  kernel_times().chol_levels = c.levels;
  kernel_times().chol_tail = p.T;
  o.lin_change = host[0];
  o.ok = host[1] == 0.0 ? 1 : 0;
  return o;
}

SolveOut chol_solve(SolverDev& s, CholDev& c, double lambda, cudaStream_t st) {
  SolveOut o;
  if (s.N == 0) {
    o.ok = 1;
    return o;
  }
  const int grid = chol_grid(s);
  c.part.resize((size_t)2 * grid);
  const CholPlan& p = c.plan;
  CholArgs a = make_args(s, c, lambda);
  void* args[] = {&a};
  double ms = 0.0;
  {
    EventTimer timer(st);
    if (s.dim == 3)
      RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_chol_solve<6>, grid, kThreads, args, 0, st));
    else
      RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_chol_solve<3>, grid, kThreads, args, 0, st));
    RPGO_LAUNCHED();
    ms = timer.elapsed_ms();
  }
  double h = 0.0;
  int32_t status = 0;
  RPGO_CUDA(cudaMemcpyAsync(&h, c.out.get(), sizeof(double), cudaMemcpyDeviceToHost, st));
  RPGO_CUDA(cudaMemcpyAsync(&status, c.status.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  RPGO_CUDA(cudaStreamSynchronize(st));
  kernel_times().chol_ms += ms;
  kernel_times().chol_launches += 1;
  kernel_times().chol_flops += p.flops;
  kernel_times().chol_bytes += p.bytes;
  kernel_times().chol_levels = c.levels;
  kernel_times().chol_tail = p.T;
  o.lin_change = h;
  o.ok = status == 0 ? 1 : 0;
  o.cg_iterations = 0;
  o.rel_residual = 0.0;
  return o;
}

void chol_enqueue_batch(SolverDev& s, CholDev& c, const BatchDev& b, cudaStream_t st) {
  if (s.N == 0 || b.G == 0) return;
  if (!c.ev[0]) {
    RPGO_CUDA(cudaEventCreate(&c.ev[0]));
    RPGO_CUDA(cudaEventCreate(&c.ev[1]));
  }
  const int grid = chol_grid(s);
  c.part.resize((size_t)2 * grid);
  CholArgs a = make_args(s, c, 0.0);
  a.G = b.G;
  a.b_sys = b.vsys.get();
  a.b_off = b.voff.get();
  a.b_act = b.ctl.get();
  a.b_lam = b.lam.get();
  a.b_status = b.status.get();
  a.b_out = b.out.get();
  a.b_term = b.term.get();
  if (b.compacted) {
    a.tasks = reinterpret_cast<const int32_t*>(b.tasks_c.get());
    a.lvl_cols = b.cols_c.get();
    a.lvl_task_end = b.task_end.get();
    a.lvl_col_end = b.col_end.get();
    a.b_compact = 1;
  }
  void* args[] = {&a};
  RPGO_CUDA(cudaEventRecord(c.ev[0], st));
  if (s.dim == 3)
    RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_chol_solve<6>, grid, kThreads, args, 0, st));
  else
    RPGO_CUDA(cudaLaunchCooperativeKernel((const void*)k_chol_solve<3>, grid, kThreads, args, 0, st));
  RPGO_LAUNCHED();
  RPGO_CUDA(cudaEventRecord(c.ev[1], st));
}

void chol_batch_compact(CholDev& c, BatchDev& b, cudaStream_t st) {
  const CholPlan& p = c.plan;
  const int L = p.levels();
  if (L == 0) return;
  constexpr int kChunk = 4096;
  if (b.n_task_chunks == 0) {
    // chunk tables: (level, begin, end, the level's first chunk), per level
    // its first chunk; every level gets at least one (possibly empty) chunk
    auto tables = [&](const std::vector<int32_t>& ptr, DeviceBuffer<int4>& chunks, DeviceBuffer<int32_t>& level_chunks,
                      int* n) {
      std::vector<int4> ch;
      std::vector<int32_t> lc(L + 1, 0);
      for (int l = 0; l < L; ++l) {
        lc[l] = (int)ch.size();
        const int first = (int)ch.size();
        int i = ptr[l];
        do {
          const int e = std::min(ptr[l + 1], i + kChunk);
          ch.push_back(make_int4(l, i, e, first));
          i = e;
        } while (i < ptr[l + 1]);
      }
      lc[L] = (int)ch.size();
      chunks.upload(ch, st);
      level_chunks.upload(lc, st);
      *n = (int)ch.size();
    };
    tables(p.lvl_task_ptr, b.task_chunks, b.task_level_chunks, &b.n_task_chunks);
    tables(p.lvl_col_ptr, b.col_chunks, b.col_level_chunks, &b.n_col_chunks);
    b.task_counts.resize(b.n_task_chunks);
    b.col_counts.resize(b.n_col_chunks);
    b.tasks_c.resize(std::max<size_t>(1, p.tasks.size() / 4));
    b.cols_c.resize(std::max<size_t>(1, p.lvl_cols.size()));
    b.task_end.resize(L);
    b.col_end.resize(L);
  }
  const int4* tasks = reinterpret_cast<const int4*>(c.tasks.get());
  k_compact_count<0><<<b.n_task_chunks, kCompactThreads, 0, st>>>(b.task_chunks.get(), tasks, nullptr,
                                                                  c.blk_col.get(), b.vsys.get(), b.ctl.get(),
                                                                  b.task_counts.get());
  RPGO_LAUNCHED();
  k_compact_count<1><<<b.n_col_chunks, kCompactThreads, 0, st>>>(b.col_chunks.get(), nullptr, c.lvl_cols.get(),
                                                                 c.blk_col.get(), b.vsys.get(), b.ctl.get(),
                                                                 b.col_counts.get());
  RPGO_LAUNCHED();
  k_compact_scatter<0><<<b.n_task_chunks, kCompactThreads, 0, st>>>(
      b.task_chunks.get(), c.lvl_task_ptr.get(), tasks, nullptr, c.blk_col.get(), b.vsys.get(), b.ctl.get(),
      b.task_counts.get(), b.tasks_c.get(), nullptr);
  RPGO_LAUNCHED();
  k_compact_scatter<1><<<b.n_col_chunks, kCompactThreads, 0, st>>>(
      b.col_chunks.get(), c.lvl_col_ptr.get(), nullptr, c.lvl_cols.get(), c.blk_col.get(), b.vsys.get(),
      b.ctl.get(), b.col_counts.get(), nullptr, b.cols_c.get());
  RPGO_LAUNCHED();
  k_compact_ends<<<div_up(L, 64), 64, 0, st>>>(L, c.lvl_task_ptr.get(), b.task_level_chunks.get(),
                                               b.task_counts.get(), b.task_end.get());
  RPGO_LAUNCHED();
  k_compact_ends<<<div_up(L, 64), 64, 0, st>>>(L, c.lvl_col_ptr.get(), b.col_level_chunks.get(),
                                               b.col_counts.get(), b.col_end.get());
  RPGO_LAUNCHED();
  b.compacted = true;
}

float chol_last_ms(CholDev& c) {
  float ms = 0.f;
  if (c.ev[0]) RPGO_CUDA(cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]));
  return ms;
}

}  // namespace rpgo

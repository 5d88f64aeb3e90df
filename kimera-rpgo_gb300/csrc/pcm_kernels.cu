// PCM outlier-rejection kernels (sm_103a).
//
//  K0 trajectory scan   Pcm::updateOdom (Pcm.h:516-557): the odometry chain
//                       T_k = T_{k-1} o Delta_k with the covariance
//                       Ad(Delta^-1) S Ad(Delta^-1)^T + S_Delta, sequential in
//                       factor order (one warp; lanes split each 6x6 update).
//  K1 odometry check    Pcm::isOdomConsistent / checkOdomConsistent
//                       (Pcm.h:564-629), one thread per loop closure.
//  K2 pairwise check    Pcm::areLoopsConsistent / checkLoopConsistent /
//                       incrementAdjMatrix (Pcm.h:638-768): one thread per
//                       closure pair (i < j), 32 consecutive i per warp, the
//                       verdicts packed into 32-bit adjacency words with one
//                       warp ballot; a second kernel mirrors the lower
//                       triangle into the upper one with warp bit transposes.
// All arithmetic is the exact FP64 sequence of pcm_math.cuh.
#include <type_traits>

#include "pcm_kernels.hpp"
#include "pcm_math.cuh"

namespace rpgo {
namespace {

using namespace pm;

// ------------------------------------------------------------------ uncertain poses
template <int DIM>
struct Lie;
template <>
struct Lie<3> {
  using Pose = P3;
  static constexpr int d = 6, rd = 3, td = 3, stride = 12;
  __device__ static void load(const double* s, Pose& p) { p3_load(s, p); }
  __device__ static void store(const Pose& p, double* s) { p3_store(p, s); }
  __device__ static void compose(const Pose& a, const Pose& b, Pose& c) { p3_compose(a, b, c); }
  __device__ static void inverse(const Pose& a, Pose& c) { p3_inverse(a, c); }
  __device__ static void between(const Pose& a, const Pose& b, Pose& c) { p3_between(a, b, c); }
  __device__ static void congruence(const Pose& T, const double* S, double* C) { p3_congruence(T, S, C); }
  __device__ static void logmap(const Pose& T, double* xi) { p3_logmap(T, xi); }
  __device__ static double rot_trace(const double* c) { return add(add(c[0], c[7]), c[14]); }
};
template <>
struct Lie<2> {
  using Pose = P2;
  static constexpr int d = 3, rd = 1, td = 2, stride = 4;
  __device__ static void load(const double* s, Pose& p) { p2_load(s, p); }
  __device__ static void store(const Pose& p, double* s) { p2_store(p, s); }
  __device__ static void compose(const Pose& a, const Pose& b, Pose& c) { p2_compose(a, b, c); }
  __device__ static void inverse(const Pose& a, Pose& c) { p2_inverse(a, c); }
  __device__ static void between(const Pose& a, const Pose& b, Pose& c) { p2_between(a, b, c); }
  __device__ static void congruence(const Pose& T, const double* S, double* C) { p2_congruence(T, S, C); }
  __device__ static void logmap(const Pose& T, double* xi) { p2_logmap(T, xi); }
  __device__ static double rot_trace(const double* c) { return c[0]; }
};

// PoseWithCovariance (GeometryUtils.h:56-187)
template <int DIM>
struct PWC {
  using L = Lie<DIM>;
  static constexpr int d = L::d;
  typename L::Pose pose;
  double cov[d * d];
  bool rot;

  __device__ void from_factor(const double* zp, const double* zc) {
    L::load(zp, pose);
    rot = !isnan(L::rot_trace(zc));
#pragma unroll
    for (int i = 0; i < d; ++i)
#pragma unroll
      for (int j = 0; j < d; ++j) cov[d * i + j] = (rot || (i >= L::rd && j >= L::rd)) ? zc[d * i + j] : 0.0;
  }
  __device__ void from_traj(const TrajView& t, int s) {
    L::load(t.pose + (size_t)s * L::stride, pose);
#pragma unroll
    for (int i = 0; i < d * d; ++i) cov[i] = t.cov[(size_t)s * d * d + i];
    rot = t.rot[s] != 0;
  }
  // this o other (GeometryUtils.h:119-129)
  __device__ void compose(const PWC& other, PWC& out) const {
    typename L::Pose inv;
    L::compose(pose, other.pose, out.pose);
    L::inverse(other.pose, inv);
    double C[d * d];
    L::congruence(inv, cov, C);
#pragma unroll
    for (int i = 0; i < d; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j) {
        const double v = add(C[d * i + j], other.cov[d * i + j]);
        out.cov[d * i + j] = v;
        out.cov[d * j + i] = v;
      }
    out.rot = rot && other.rot;
  }
  // the same composition with the inverse of other's pose given as its
  // rotation and the K block of its adjoint (per-closure constants, 3D)
  __device__ void compose_pre(const PWC& other, const double* pre, PWC& out) const {
    L::compose(pose, other.pose, out.pose);
    double C[d * d];
    pm::p3_congruence_RK(pre, pre + 9, cov, C);
#pragma unroll
    for (int i = 0; i < d; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j) {
        const double v = add(C[d * i + j], other.cov[d * i + j]);
        out.cov[d * i + j] = v;
        out.cov[d * j + i] = v;
      }
    out.rot = rot && other.rot;
  }
  // GeometryUtils.h:133-139
  __device__ void inverse_inplace() {
    typename L::Pose p;
    L::inverse(pose, p);
    pose = p;
  }
  // this^-1 o other with the LLT fallback (GeometryUtils.h:143-170)
  __device__ void between(const PWC& other, PWC& out) const {
    typename L::Pose res, inv;
    L::between(pose, other.pose, res);
    L::inverse(res, inv);
    double C[d * d];
    L::congruence(inv, cov, C);
#pragma unroll
    for (int i = 0; i < d; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j) {
        const double v = sub(other.cov[d * i + j], C[d * i + j]);
        out.cov[d * i + j] = v;
        out.cov[d * j + i] = v;
      }
    if (!chol_ok<d>(out.cov)) {
      typename L::Pose res2, inv2;
      L::between(other.pose, pose, res2);
      L::inverse(res2, inv2);
      L::congruence(inv2, other.cov, C);
#pragma unroll
      for (int i = 0; i < d; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
          const double v = sub(cov[d * i + j], C[d * i + j]);
          out.cov[d * i + j] = v;
          out.cov[d * j + i] = v;
        }
    }
    out.pose = res;
    out.rot = rot && other.rot;
  }
  __device__ double mahalanobis() const {
    double xi[d];
    L::logmap(pose, xi);
    if (!rot) {
      constexpr int m = L::td, r = L::rd;
      double B[m * m];
#pragma unroll
      for (int i = 0; i < m; ++i)
#pragma unroll
        for (int j = 0; j < m; ++j) B[m * i + j] = cov[d * (r + i) + (r + j)];
      return sqrtd(quad_inv<m>(B, xi + r));
    }
    return sqrtd(quad_inv<d>(cov, xi));
  }
};

// PoseWithNode (GeometryUtils.h:193-289)
template <int DIM>
struct PWN {
  using L = Lie<DIM>;
  static constexpr int d = L::d;
  typename L::Pose pose;
  int node;
  bool rot;
  __device__ void from_factor(const double* zp, const double* zc) {
    L::load(zp, pose);
    rot = !isnan(L::rot_trace(zc));
    node = 1;
  }
  __device__ void from_traj(const TrajView& t, int s) {
    L::load(t.pose + (size_t)s * L::stride, pose);
    node = t.node[s];
    rot = t.rot[s] != 0;
  }
  __device__ void compose(const PWN& o, PWN& out) const {
    L::compose(pose, o.pose, out.pose);
    out.node = node + o.node;
    out.rot = rot && o.rot;
  }
  __device__ void inverse_inplace() {
    typename L::Pose p;
    L::inverse(pose, p);
    pose = p;
  }
  __device__ void between(const PWN& o, PWN& out) const {
    L::between(pose, o.pose, out.pose);
    out.node = abs(o.node - node);
    out.rot = rot && o.rot;
  }
  __device__ static double norm_slice(const double* v, int m) {
    double acc = mul(v[0], v[0]);
    for (int i = 1; i < m; ++i) acc = fmad(v[i], v[i], acc);
    return sqrtd(acc);
  }
  __device__ void norms(double& trans, double& rotn) const {
    double xi[d];
    L::logmap(pose, xi);
    trans = dvd(norm_slice(xi + L::rd, L::td), (double)node);
    rotn = rot ? dvd(norm_slice(xi, L::rd), (double)node) : 0.0;
  }
};

template <class U>
__device__ __forceinline__ bool check_mahal(const U& u, double th0, double) {
  return u.mahalanobis() < th0;
}
template <int DIM>
__device__ __forceinline__ bool check_u(const PWC<DIM>& u, double th0, double) {
  return u.mahalanobis() < th0;
}
template <int DIM>
__device__ __forceinline__ bool check_u(const PWN<DIM>& u, double th0, double th1) {
  double t, r;
  u.norms(t, r);
  return t < th0 && r < th1;
}

// ------------------------------------------------------------------ K0
// Exact per-element pieces of PWC::compose for one lane.
__device__ __forceinline__ double p3_compose_elem(const double* A, const double* B, int e) {
  // A, B: 12-double pose records (R row-major, t)
  if (e < 9) {
    const int i = e / 3, j = e % 3;
    return dot3e(A[3 * i], A[3 * i + 1], A[3 * i + 2], B[j], B[3 + j], B[6 + j]);
  }
  const int i = e - 9;
  double acc = fmad(A[3 * i], B[9], A[9 + i]);
  acc = fmad(A[3 * i + 1], B[10], acc);
  return fmad(A[3 * i + 2], B[11], acc);
}
__device__ __forceinline__ double p2_compose_elem(const double* A, const double* B, int e) {
  // (c, s, x, y)
  switch (e) {
    case 0: return fmad(A[0], B[0], -mul(A[1], B[1]));
    case 1: return fmad(A[1], B[0], mul(A[0], B[1]));
    case 2: return add(A[2], fmad(A[0], B[2], -mul(A[1], B[3])));
    default: return add(A[3], fmad(A[1], B[2], mul(A[0], B[3])));
  }
}

// Per-odometry-factor constants: the measurement as an uncertain pose
// (GeometryUtils.h:91-115) and the pieces of Ad(Delta^-1).
template <int DIM>
__global__ void k_odom_prep(int64_t count, const double* __restrict__ dpose, const double* __restrict__ dcov,
                            double* __restrict__ inv_rec, double* __restrict__ cov_out, uint8_t* __restrict__ rot_out) {
  using L = Lie<DIM>;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  PWC<DIM> z;
  z.from_factor(dpose + k * L::stride, dcov + k * L::d * L::d);
  for (int i = 0; i < L::d * L::d; ++i) cov_out[k * L::d * L::d + i] = z.cov[i];
  rot_out[k] = z.rot ? 1 : 0;
  typename L::Pose inv;
  L::inverse(z.pose, inv);
  if constexpr (DIM == 3) {
    double K[9];
    p3_adjoint_K(inv, K);
    double* r = inv_rec + k * 21;
    for (int i = 0; i < 9; ++i) r[i] = inv.R[i];
    for (int i = 0; i < 9; ++i) r[9 + i] = K[i];
    for (int i = 0; i < 3; ++i) r[18 + i] = inv.t[i];
  } else {
    double A[9];
    p2_adjoint(inv, A);
    double* r = inv_rec + k * 9;
    for (int i = 0; i < 9; ++i) r[i] = A[i];
  }
}

// One warp walks the odometry list in order. The step constants of step k+1
// (odometry pose, Ad(Delta^-1) pieces, covariance, indices) are loaded into
// registers while step k computes and land in shared memory at its end, so
// the walk waits on memory only when a chain restarts from an older pose.
template <int DIM, int MODE>
__global__ void __launch_bounds__(32) k_traj_scan(int64_t count, const int32_t* __restrict__ src,
                                                  const int32_t* __restrict__ dst, const double* __restrict__ dpose,
                                                  const double* __restrict__ inv_rec,
                                                  const double* __restrict__ dcov_p,
                                                  const uint8_t* __restrict__ drot, TrajView tr) {
  using L = Lie<DIM>;
  constexpr int d = L::d, st = L::stride, dd = d * d;
  constexpr int REC = (DIM == 3) ? 21 : 9;
  constexpr int NC = st + ((MODE == 0) ? REC + dd : 0);  // step constants
  constexpr int NQ = (NC + 31) / 32;
  __shared__ double prev_pose[12], prev_cov[36], M[36], newp[12], rec[21], dpz[12], dc[36];
  __shared__ int prev_node;
  __shared__ uint8_t prev_rot;
  const int lane = threadIdx.x;
  double pre[NQ];
  int32_t ps = 0, pt = 0;
  uint8_t prot = 0;
  auto load_step = [&](int64_t k) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int e = lane + 32 * q;
      if (e < st) pre[q] = dpose[k * st + e];
      else if (MODE == 0 && e < st + REC) pre[q] = inv_rec[k * REC + (e - st)];
      else if (MODE == 0 && e < NC) pre[q] = dcov_p[k * dd + (e - st - REC)];
    }
    ps = src[k];
    pt = dst[k];
    prot = drot[k];
  };
  auto store_step = [&]() {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int e = lane + 32 * q;
      if (e < st) dpz[e] = pre[q];
      else if (MODE == 0 && e < st + REC) rec[e - st] = pre[q];
      else if (MODE == 0 && e < NC) dc[e - st - REC] = pre[q];
    }
  };
  // this lane's phase-1 items (e = lane, lane + 32 of [M entries | pose
  // entries]) and phase-2 entry (ii, jj) of the lower triangle, fixed for
  // the whole walk
  constexpr int nm = (MODE == 0) ? dd : 0;
  int it_i[2], it_k[2], it_pl[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int e = lane + 32 * q;
    it_i[q] = -1;
    it_k[q] = 0;
    it_pl[q] = -1;
    if (e < nm) {
      it_i[q] = e / d;
      it_k[q] = e % d;
    } else if (e < nm + st) {
      it_pl[q] = e - nm;
    }
  }
  constexpr int ntri = d * (d + 1) / 2;
  int tri_i = 0, tri_j = 0;
  if (lane < ntri) {
    int idx = lane;
    while (idx > tri_i) {
      idx -= tri_i + 1;
      ++tri_i;
    }
    tri_j = idx;
  }
  int32_t last_dst = -1;
  if (count > 0) {
    load_step(0);
    store_step();
  }
  int32_t s = ps, t = pt;
  uint8_t rot_k = prot;
  for (int64_t k = 0; k < count; ++k) {
    if (k + 1 < count) load_step(k + 1);
    // load previous state (unless it is the pose just written)
    if (s != last_dst) {
      for (int e = lane; e < st; e += 32) prev_pose[e] = tr.pose[(size_t)s * st + e];
      if (MODE == 0)
        for (int e = lane; e < dd; e += 32) prev_cov[e] = tr.cov[(size_t)s * dd + e];
      if (lane == 0) {
        prev_rot = tr.rot[s];
        if (MODE == 1) prev_node = tr.node[s];
      }
    }
    __syncwarp();
    // phase 1: M = Ad(Delta^-1) S_prev (items [0, dd)) and the new pose
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (it_i[q] >= 0) {
        if constexpr (DIM == 3) M[lane + 32 * q] = p3_M_elem(rec, rec + 9, prev_cov, it_i[q], it_k[q]);
        else M[lane + 32 * q] = p2_M_elem(rec, prev_cov, it_i[q], it_k[q]);
      } else if (it_pl[q] >= 0) {
        if constexpr (DIM == 3) newp[it_pl[q]] = p3_compose_elem(prev_pose, dpz, it_pl[q]);
        else newp[it_pl[q]] = p2_compose_elem(prev_pose, dpz, it_pl[q]);
      }
    }
    __syncwarp();
    // phase 2: lower triangle of M Ad^T + S_Delta
    if (MODE == 0) {
      double v = 0.0;
      const int ii = tri_i, jj = tri_j;
      if (lane < ntri) {
        double c;
        if constexpr (DIM == 3) c = p3_C_elem(rec, rec + 9, M + 6 * ii, jj);
        else c = p2_C_elem(rec, M + 3 * ii, jj);
        v = add(c, dc[d * ii + jj]);
      }
      __syncwarp();
      if (lane < ntri) {
        prev_cov[d * ii + jj] = v;
        prev_cov[d * jj + ii] = v;
      }
    }
    for (int e = lane; e < st; e += 32) prev_pose[e] = newp[e];
    if (lane == 0) {
      prev_rot = (prev_rot && rot_k) ? 1 : 0;
      if (MODE == 1) prev_node = prev_node + 1;
    }
    __syncwarp();
    for (int e = lane; e < st; e += 32) tr.pose[(size_t)t * st + e] = prev_pose[e];
    if (MODE == 0)
      for (int e = lane; e < dd; e += 32) tr.cov[(size_t)t * dd + e] = prev_cov[e];
    if (lane == 0) {
      tr.rot[t] = prev_rot;
      if (MODE == 1) tr.node[t] = prev_node;
    }
    last_dst = t;
    __syncwarp();
    if (k + 1 < count) {
      store_step();
      s = ps;
      t = pt;
      rot_k = prot;
    }
    __syncwarp();
  }
}

// The 3D PoseWithCovariance walk on two warps (64 threads), one output
// element per thread. Every element of compose (GeometryUtils.h:119-129) is
// an FMA chain over at most six products, evaluated exactly as p3_M_elem,
// p3_C_elem and p3_compose_elem do (a chain that starts with a product
// starts from fma(a0, b0, -0), which equals mul(a0, b0) bit for bit, so the
// threads run one branch-free chain): warp 0 takes the three-term chains
// (rows 0-2 of M = Ad(Delta^-1) S, the new pose, the C entries of columns
// 0-2), warp 1 the six-term chains (rows 3-5 of M, the C entries of columns
// 3-5), so both warps issue their FP64 chains on their own sub-partitions.
// Step constants are double-buffered in shared memory: the next step's are
// loaded while this one computes. Two block barriers per step.
__global__ void __launch_bounds__(64) k_traj_scan_pwc3(int64_t count, const int32_t* __restrict__ src,
                                                       const int32_t* __restrict__ dst,
                                                       const double* __restrict__ dpose,
                                                       const double* __restrict__ inv_rec,
                                                       const double* __restrict__ dcov_p,
                                                       const uint8_t* __restrict__ drot, TrajView tr) {
  constexpr int st = 12, dd = 36, REC = 21, NC = st + REC + dd;  // 69 step constants
  __shared__ double prev_pose[12], prev_cov[36], M[36];
  __shared__ double cst[2][72];  // [0,12) Delta pose, [12,33) Ad(Delta^-1) pieces (R, K, t), [33,69) Sigma_Delta
  __shared__ uint8_t prev_rot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // ---- this thread's chains (fixed for the whole walk)
  // phase 1 kind: 0 none, 1 M row < 3, 2 pose R entry, 3 pose t entry, 4 M row >= 3
  int p1 = 0, mi = 0, mk = 0, pe = 0;
  if (warp == 0) {
    if (lane < 18) {
      p1 = 1;
      mi = lane / 6;
      mk = lane % 6;
    } else if (lane < 27) {
      p1 = 2;
      pe = lane - 18;
    } else if (lane < 30) {
      p1 = 3;
      pe = 9 + (lane - 27);
    }
  } else if (lane < 18) {
    p1 = 4;
    mi = 3 + lane / 6;
    mk = lane % 6;
  }
  // phase 2: lower-triangle entry (ci, cj) of M Ad^T
  int p2 = 0, ci = 0, cj = 0;
  if (warp == 0 && lane < 15) {  // columns 0-2: rows cj..5 of each column
    int idx = lane;
    cj = 0;
    while (idx >= 6 - cj) {
      idx -= 6 - cj;
      ++cj;
    }
    ci = cj + idx;
    p2 = 1;
  } else if (warp == 1 && lane < 6) {  // columns 3-5, rows >= column
    const int tab_i[6] = {3, 4, 5, 4, 5, 5}, tab_j[6] = {3, 3, 3, 4, 4, 5};
    ci = tab_i[lane];
    cj = tab_j[lane];
    p2 = 2;
  }
  double pre[2];
  int32_t ps = 0, pt = 0;
  uint8_t prot = 0;
  auto load_step = [&](int64_t k) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int e = tid + 64 * q;
      if (e < st) pre[q] = dpose[k * st + e];
      else if (e < st + REC) pre[q] = inv_rec[k * REC + (e - st)];
      else if (e < NC) pre[q] = dcov_p[k * dd + (e - st - REC)];
    }
    ps = src[k];
    pt = dst[k];
    prot = drot[k];
  };
  auto store_step = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int e = tid + 64 * q;
      if (e < NC) cst[buf][e] = pre[q];
    }
  };
  int32_t last_dst = -1;
  if (count > 0) {
    load_step(0);
    store_step(0);
  }
  __syncthreads();
  int32_t s = ps, t = pt;
  uint8_t rot_k = prot;
  for (int64_t k = 0; k < count; ++k) {
    const int b = (int)(k & 1);
    const double* dpz = cst[b];
    const double* R = cst[b] + 12;
    const double* K = cst[b] + 21;
    const double* dc = cst[b] + 33;
    if (k + 1 < count) load_step(k + 1);
    if (s != last_dst) {  // the chain continues from an older pose: read it back
      for (int e = tid; e < st; e += 64) prev_pose[e] = tr.pose[(size_t)s * st + e];
      for (int e = tid; e < dd; e += 64) prev_cov[e] = tr.cov[(size_t)s * dd + e];
      if (tid == 0) prev_rot = tr.rot[s];
      __syncthreads();
    }
    // ---- phase 1
    double newp = 0.0;
    if (p1 != 0) {
      double a[6], x[6], c0 = -0.0;
      int nt = 3;
      if (p1 == 1) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          a[q] = R[3 * mi + q];
          x[q] = prev_cov[6 * q + mk];
        }
      } else if (p1 == 4) {
        const int r = mi - 3;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          a[q] = K[3 * r + q];
          x[q] = prev_cov[6 * q + mk];
          a[3 + q] = R[3 * r + q];
          x[3 + q] = prev_cov[18 + 6 * q + mk];
        }
        nt = 6;
      } else if (p1 == 2) {
        const int i = pe / 3, j = pe % 3;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          a[q] = prev_pose[3 * i + q];
          x[q] = dpz[3 * q + j];
        }
      } else {
        const int i = pe - 9;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          a[q] = prev_pose[3 * i + q];
          x[q] = dpz[9 + q];
        }
        c0 = prev_pose[9 + i];
      }
      double acc = fmad(a[0], x[0], c0);
      acc = fmad(a[1], x[1], acc);
      acc = fmad(a[2], x[2], acc);
      if (nt == 6) {
        acc = fmad(a[3], x[3], acc);
        acc = fmad(a[4], x[4], acc);
        acc = fmad(a[5], x[5], acc);
      }
      if (p1 == 1 || p1 == 4) M[6 * mi + mk] = acc;
      else newp = acc;
    }
    __syncthreads();
    // ---- phase 2: C = M Ad^T + Sigma_Delta (lower triangle, mirrored), the new pose
    if (p2 != 0) {
      const double* m = M + 6 * ci;
      double acc;
      if (p2 == 1) {
        acc = fmad(m[0], R[3 * cj], -0.0);
        acc = fmad(m[1], R[3 * cj + 1], acc);
        acc = fmad(m[2], R[3 * cj + 2], acc);
      } else {
        const double* kk = K + 3 * (cj - 3);
        const double* rr = R + 3 * (cj - 3);
        acc = fmad(m[0], kk[0], -0.0);
        acc = fmad(m[1], kk[1], acc);
        acc = fmad(m[2], kk[2], acc);
        acc = fmad(m[3], rr[0], acc);
        acc = fmad(m[4], rr[1], acc);
        acc = fmad(m[5], rr[2], acc);
      }
      const double v = add(acc, dc[6 * ci + cj]);
      prev_cov[6 * ci + cj] = v;
      prev_cov[6 * cj + ci] = v;
      tr.cov[(size_t)t * dd + 6 * ci + cj] = v;
      if (ci != cj) tr.cov[(size_t)t * dd + 6 * cj + ci] = v;
    }
    if (p1 == 2 || p1 == 3) {
      prev_pose[pe] = newp;
      tr.pose[(size_t)t * st + pe] = newp;
    }
    if (tid == 0) {
      prev_rot = (prev_rot && rot_k) ? 1 : 0;
      tr.rot[t] = prev_rot;
    }
    last_dst = t;
    if (k + 1 < count) {
      store_step(b ^ 1);
      s = ps;
      t = pt;
      rot_k = prot;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ K1
template <int DIM, class U>
__global__ void k_odom_check(int64_t count, const int32_t* __restrict__ si, const int32_t* __restrict__ sj,
                             const double* __restrict__ zp, const double* __restrict__ zc, TrajView tr, double th0,
                             double th1, uint8_t* __restrict__ ok) {
  using L = Lie<DIM>;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  U a, b, pij, z, res;
  a.from_traj(tr, si[k]);
  b.from_traj(tr, sj[k]);
  a.between(b, pij);
  z.from_factor(zp + k * L::stride, zc + k * L::d * L::d);
  z.inverse_inplace();
  pij.compose(z, res);
  ok[k] = check_u<DIM>(res, th0, th1) ? 1 : 0;
}

// ------------------------------------------------------------------ K2
// Per-closure constants of the 3D PoseWithCovariance test: the rotation of
// the inverse of each measured pose and the K block of that inverse's adjoint
// (what each composition with the closure computes first), 18 doubles per
// closure. The pairwise test uses them instead of recomputing them per pair:
// the same operations, so the same bits.
constexpr int kClosurePre = 18;
__global__ void k_closure_pre3(int n, const double* __restrict__ zp, double* __restrict__ pre) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  pm::P3 Z, inv;
  pm::p3_load(zp + (size_t)k * 12, Z);
  pm::p3_inverse(Z, inv);
  double* o = pre + (size_t)k * kClosurePre;
#pragma unroll
  for (int e = 0; e < 9; ++e) o[e] = inv.R[e];
  pm::p3_adjoint_K(inv, o + 9);
}

template <int DIM, class U>
__device__ __forceinline__ bool pair_consistent(int i, int j, const int32_t* __restrict__ sa,
                                                const int32_t* __restrict__ sb, const uint8_t* __restrict__ flip,
                                                const double* __restrict__ zp, const double* __restrict__ zc,
                                                const TrajView& tr, double th0, double th1,
                                                const double* __restrict__ pre) {
  using L = Lie<DIM>;
  int a = sa[i], b = sb[i], c = sa[j], dd = sb[j];
  if (flip[i] != flip[j]) {
    const int t = c;
    c = dd;
    dd = t;
  }
  U A, B, Ta, Tc, Zj, Zi, P, Q, loop;
  Ta.from_traj(tr, a);
  Tc.from_traj(tr, c);
  Ta.between(Tc, A);
  Ta.from_traj(tr, b);
  Tc.from_traj(tr, dd);
  Ta.between(Tc, B);
  Zj.from_factor(zp + (size_t)j * L::stride, zc + (size_t)j * L::d * L::d);
  Zi.from_factor(zp + (size_t)i * L::stride, zc + (size_t)i * L::d * L::d);
  if constexpr (std::is_same<U, PWC<3>>::value) {
    A.compose_pre(Zj, pre + (size_t)j * kClosurePre, P);
    P.inverse_inplace();
    P.compose_pre(Zi, pre + (size_t)i * kClosurePre, Q);
  } else {
    A.compose(Zj, P);
    P.inverse_inplace();
    P.compose(Zi, Q);
  }
  Q.compose(B, loop);
  return check_u<DIM>(loop, th0, th1);
}

// Landmark pair (Pcm.h:775-844): observations i, j (pose -> landmark) of one
// landmark. i_odom_j = getBetween(pose_i, pose_j) of pose_i's trajectory
// (GraphUtils.h:37-58): slots (s.x, s.y) for one robot; for two robots
// (s.x, s.y, s.z, s.w) = (root a0, pose_i, root b0, pose_j) as looked up in
// pose_i's trajectory. loop = (i_odom_j o Z_j)^-1 o Z_i.
template <int DIM, class U>
__global__ void k_landmark_pairs(int count, const int4* __restrict__ desc, const int2* __restrict__ ij,
                                 const double* __restrict__ zp, const double* __restrict__ zc, TrajView tr,
                                 double th0, double th1, uint32_t* __restrict__ adj, int words) {
  using L = Lie<DIM>;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int4 s = desc[k];
  const int i = ij[k].x, j = ij[k].y;
  U iodomj, X, Y;
  if (s.z < 0) {
    X.from_traj(tr, s.x);
    Y.from_traj(tr, s.y);
    X.between(Y, iodomj);
  } else {
    U pa, pb, pab, t;
    X.from_traj(tr, s.x);
    Y.from_traj(tr, s.y);
    X.between(Y, pa);
    U B0, Kb;
    B0.from_traj(tr, s.z);
    Kb.from_traj(tr, s.w);
    B0.between(Kb, pb);
    X.between(B0, pab);
    pa.inverse_inplace();
    pa.compose(pab, t);
    t.compose(pb, iodomj);
  }
  U zj, zi, path, loop;
  zj.from_factor(zp + (size_t)j * L::stride, zc + (size_t)j * L::d * L::d);
  iodomj.compose(zj, path);
  path.inverse_inplace();
  zi.from_factor(zp + (size_t)i * L::stride, zc + (size_t)i * L::d * L::d);
  path.compose(zi, loop);
  if (check_u<DIM>(loop, th0, th1)) {
    atomicOr(adj + (size_t)i * words + (j >> 5), 1u << (j & 31));
    atomicOr(adj + (size_t)j * words + (i >> 5), 1u << (i & 31));
  }
}

// block (32, ROWS): lane -> column i = 32*bx + lane, row j = row_begin + ROWS*by + ty.
// lower[(j - row_begin) * words + bx] receives bits i < j.
template <int DIM, class U, int ROWS>
__global__ void __launch_bounds__(32 * ROWS) k_pairwise(int n, int row_begin, const int32_t* __restrict__ sa,
                                                        const int32_t* __restrict__ sb,
                                                        const uint8_t* __restrict__ flip,
                                                        const double* __restrict__ zp,
                                                        const double* __restrict__ zc, TrajView tr, double th0,
                                                        double th1, uint32_t* __restrict__ lower, int words,
                                                        const double* __restrict__ pre) {
  const int lane = threadIdx.x;
  const int j = row_begin + ROWS * blockIdx.y + threadIdx.y;
  const int i0 = 32 * blockIdx.x;
  if (j >= n || i0 >= j) return;  // whole warp: tile above the diagonal or past the end
  const int i = i0 + lane;
  bool ok = false;
  if (i < j) ok = pair_consistent<DIM, U>(i, j, sa, sb, flip, zp, zc, tr, th0, th1, pre);
  const unsigned bits = __ballot_sync(0xffffffffu, ok);
  if (lane == 0) lower[(size_t)(j - row_begin) * words + blockIdx.x] = bits;
}

// Mirror: adj[r][c] for c < r from lower rows (r >= row_begin) or the old
// matrix (r < row_begin); for c > r from lower[c][r] (c >= row_begin) or the
// old matrix. One warp per 32x32 block, lane = row within the block.
__global__ void k_symmetrize(int n, int row_begin, const uint32_t* __restrict__ lower, uint32_t* __restrict__ adj,
                             int words) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nb = (n + 31) / 32;
  if (warp >= nb * nb) return;
  const int bi = warp / nb, bj = warp % nb;
  const int r = 32 * bi + lane;
  // transpose source: word (rows c = 32*bj + lane) column block bi of lower
  const int c_src = 32 * bj + lane;
  uint32_t src = 0;
  if (c_src < n && c_src >= row_begin) src = lower[(size_t)(c_src - row_begin) * words + bi];
  uint32_t tr_word = 0;
#pragma unroll 4
  for (int b = 0; b < 32; ++b) {
    const uint32_t col = __ballot_sync(0xffffffffu, (src >> b) & 1u);
    if (b == lane) tr_word = col;  // bits over c of row 32*bi + b
  }
  if (r >= n) return;
  const uint32_t old = (r < row_begin) ? adj[(size_t)r * words + bj] : 0u;
  uint32_t out = 0;
  // column mask helpers within block bj
  const int c0 = 32 * bj;
  uint32_t lt = 0, gt = 0, valid = 0;
  for (int b = 0; b < 32; ++b) {
    const int c = c0 + b;
    if (c >= n) break;
    valid |= 1u << b;
    if (c < r) lt |= 1u << b;
    if (c > r) gt |= 1u << b;
  }
  // lower part
  if (r >= row_begin) out |= lower[(size_t)(r - row_begin) * words + bj] & lt;
  else out |= old & lt;
  // upper part: new columns from the transpose, old columns from the old matrix
  uint32_t newcols = 0;
  for (int b = 0; b < 32; ++b)
    if (c0 + b >= row_begin && c0 + b < n) newcols |= 1u << b;
  out |= tr_word & gt & newcols;
  out |= old & gt & ~newcols;
  adj[(size_t)r * words + bj] = out & valid;
}

}  // namespace

// ------------------------------------------------------------------ launchers
void launch_traj_scan(int dim, int mode, int64_t count, const int32_t* src, const int32_t* dst,
                      const double* dpose, const double* dcov, TrajView tr, DeviceBuffer<double>& scratch_rec,
                      DeviceBuffer<double>& scratch_cov, DeviceBuffer<uint8_t>& scratch_rot, cudaStream_t st) {
  if (count <= 0) return;
  const int d = dim == 3 ? 6 : 3;
  scratch_rec.resize((size_t)count * (dim == 3 ? 21 : 9));
  scratch_cov.resize((size_t)count * d * d);
  scratch_rot.resize((size_t)count);
  const int tb = 128;
  if (dim == 3) k_odom_prep<3><<<div_up(count, tb), tb, 0, st>>>(count, dpose, dcov, scratch_rec.get(),
                                                                   scratch_cov.get(), scratch_rot.get());
  else k_odom_prep<2><<<div_up(count, tb), tb, 0, st>>>(count, dpose, dcov, scratch_rec.get(), scratch_cov.get(),
                                                        scratch_rot.get());
  RPGO_LAUNCHED();
  if (dim == 3) {
    if (mode == 0) k_traj_scan_pwc3<<<1, 64, 0, st>>>(count, src, dst, dpose, scratch_rec.get(), scratch_cov.get(),
                                                     scratch_rot.get(), tr);
    else k_traj_scan<3, 1><<<1, 32, 0, st>>>(count, src, dst, dpose, scratch_rec.get(), scratch_cov.get(),
                                             scratch_rot.get(), tr);
  } else {
    if (mode == 0) k_traj_scan<2, 0><<<1, 32, 0, st>>>(count, src, dst, dpose, scratch_rec.get(), scratch_cov.get(),
                                                       scratch_rot.get(), tr);
    else k_traj_scan<2, 1><<<1, 32, 0, st>>>(count, src, dst, dpose, scratch_rec.get(), scratch_cov.get(),
                                             scratch_rot.get(), tr);
  }
  RPGO_LAUNCHED();
}

void launch_odom_check(int dim, int mode, int64_t count, const int32_t* si, const int32_t* sj, const double* zp,
                       const double* zc, TrajView tr, double th0, double th1, uint8_t* ok, cudaStream_t st) {
  if (count <= 0) return;
  const int tb = 64;
  const int g = div_up(count, tb);
  if (dim == 3) {
    if (mode == 0) k_odom_check<3, PWC<3>><<<g, tb, 0, st>>>(count, si, sj, zp, zc, tr, th0, th1, ok);
    else k_odom_check<3, PWN<3>><<<g, tb, 0, st>>>(count, si, sj, zp, zc, tr, th0, th1, ok);
  } else {
    if (mode == 0) k_odom_check<2, PWC<2>><<<g, tb, 0, st>>>(count, si, sj, zp, zc, tr, th0, th1, ok);
    else k_odom_check<2, PWN<2>><<<g, tb, 0, st>>>(count, si, sj, zp, zc, tr, th0, th1, ok);
  }
  RPGO_LAUNCHED();
}

void launch_pairwise(int dim, int mode, int n, int row_begin, const int32_t* sa, const int32_t* sb,
                     const uint8_t* flip, const double* zp, const double* zc, TrajView tr, double th0, double th1,
                     uint32_t* adj, int words, uint32_t* lower_scratch, cudaStream_t st) {
  if (n <= 0 || row_begin >= n) return;
  constexpr int ROWS = 4;
  const int rows = n - row_begin;
  dim3 block(32, ROWS), grid(div_up(n, 32), div_up(rows, ROWS));
  if (n > 1) {
    DeviceBuffer<double> pre;
    if (dim == 3 && mode == 0) {
      pre.resize((size_t)n * kClosurePre);
      k_closure_pre3<<<div_up(n, 128), 128, 0, st>>>(n, zp, pre.get());
      RPGO_LAUNCHED();
    }
    EventTimer timer(st);
    if (dim == 3) {
      if (mode == 0)
        k_pairwise<3, PWC<3>, ROWS><<<grid, block, 0, st>>>(n, row_begin, sa, sb, flip, zp, zc, tr, th0, th1,
                                                            lower_scratch, words, pre.get());
      else
        k_pairwise<3, PWN<3>, ROWS><<<grid, block, 0, st>>>(n, row_begin, sa, sb, flip, zp, zc, tr, th0, th1,
                                                            lower_scratch, words, nullptr);
    } else {
      if (mode == 0)
        k_pairwise<2, PWC<2>, ROWS><<<grid, block, 0, st>>>(n, row_begin, sa, sb, flip, zp, zc, tr, th0, th1,
                                                            lower_scratch, words, nullptr);
      else
        k_pairwise<2, PWN<2>, ROWS><<<grid, block, 0, st>>>(n, row_begin, sa, sb, flip, zp, zc, tr, th0, th1,
                                                            lower_scratch, words, nullptr);
    }
    RPGO_LAUNCHED();
    kernel_times().pair_ms += timer.elapsed_ms();
    kernel_times().pair_launches += 1;
  }
  // rows whose tiles were all skipped (j < 32*bx) keep stale words; the
  // ballot writes only tiles with i0 < j, so clear the rest first: the
  // mirror kernel reads only words bx <= j/32, all of which were written
  // except word j/32 when 32*(j/32) >= j, i.e. j a multiple of 32 -> handled
  // by masking with c < r in the mirror.
  const int nb = div_up(n, 32);
  const int warps = nb * nb;
  k_symmetrize<<<div_up((int64_t)warps * 32, 256), 256, 0, st>>>(n, row_begin, lower_scratch, adj, words);
  RPGO_LAUNCHED();
}

void launch_landmark_pairs(int dim, int mode, int count, const int4* desc, const int2* ij, const double* zp,
                           const double* zc, TrajView tr, double th0, double th1, uint32_t* adj, int words,
                           cudaStream_t st) {
  if (count <= 0) return;
  const int tb = 128, nb = div_up(count, tb);
  if (dim == 3) {
    if (mode == 0) k_landmark_pairs<3, PWC<3>><<<nb, tb, 0, st>>>(count, desc, ij, zp, zc, tr, th0, th1, adj, words);
    else k_landmark_pairs<3, PWN<3>><<<nb, tb, 0, st>>>(count, desc, ij, zp, zc, tr, th0, th1, adj, words);
  } else {
    if (mode == 0) k_landmark_pairs<2, PWC<2>><<<nb, tb, 0, st>>>(count, desc, ij, zp, zc, tr, th0, th1, adj, words);
    else k_landmark_pairs<2, PWN<2>><<<nb, tb, 0, st>>>(count, desc, ij, zp, zc, tr, th0, th1, adj, words);
  }
  RPGO_LAUNCHED();
}

namespace {
// rows [0, rows): clear every bit of columns >= from
__global__ void k_clear_columns(uint32_t* __restrict__ adj, int words, int rows, int from) {
  const int w0 = from >> 5;
  const int per_row = words - w0;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (per_row <= 0 || t >= (int64_t)rows * per_row) return;
  const int r = (int)(t / per_row), w = w0 + (int)(t % per_row);
  uint32_t* word = adj + (size_t)r * words + w;
  *word = (w == w0) ? (*word & ((1u << (from & 31)) - 1u)) : 0u;
}
}  // namespace

void launch_clear_columns(uint32_t* adj, int words, int rows, int from, cudaStream_t st) {
  const int per_row = words - (from >> 5);
  if (rows <= 0 || per_row <= 0) return;
  const int64_t n = (int64_t)rows * per_row;
  k_clear_columns<<<div_up(n, 256), 256, 0, st>>>(adj, words, rows, from);
  RPGO_LAUNCHED();
}

std::atomic<int64_t>& launch_counter() {
  static std::atomic<int64_t> c{0};
  return c;
}
std::atomic<int64_t>& alloc_counter() {
  static std::atomic<int64_t> c{0};
  return c;
}
int64_t& thread_launch_counter() {
  thread_local int64_t c = 0;
  return c;
}
KernelTimes& kernel_times() {
  thread_local KernelTimes t;
  return t;
}
cudaStream_t& alloc_stream() {
  thread_local cudaStream_t st = nullptr;
  return st;
}

}  // namespace rpgo

// Exact FP64 uncertain-pose algebra for the PCM kernels (device).
//
// Implements, for Pose3 and Pose2, the operations Kimera-RPGO's PCM runs on
// loop closures:
//   include/KimeraRPGO/utils/GeometryUtils.h:91-186  PoseWithCovariance
//   include/KimeraRPGO/utils/GeometryUtils.h:193-289 PoseWithNode
// with GTSAM's conventions (tangent [omega; v] / [v_x, v_y, omega]; compose
// Jacobian Ad(other^-1); between Jacobian -Ad(result^-1)).
//
// Every result is a fixed sequence of correctly rounded IEEE double
// operations: products, sums and quotients go through __dmul_rn / __dadd_rn /
// __dsub_rn / __ddiv_rn / __dsqrt_rn / __fma_rn, which the compiler never
// fuses or reorders. The functions below spell the sequence out operation by
// operation, so a host implementation that follows it with
// -ffp-contract=off produces the same bits.
#pragma once
#include <cstdint>

namespace rpgo {
namespace pm {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double fmad(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double sqrtd(double a) { return __dsqrt_rn(a); }

__device__ __forceinline__ double dot3e(double a0, double a1, double a2, double b0, double b1, double b2) {
  double acc = mul(a0, b0);
  acc = fmad(a1, b1, acc);
  return fmad(a2, b2, acc);
}

// atan2 from the Taylor series of atan on |w| <= tan(pi/8) (coefficients
// (-1)^k / (2k+1), Horner in w^2), reduced with atan(z) = pi/4 + atan((z-1)/(z+1)).
__device__ __forceinline__ double r_atan2(double y, double x) {
  const double kPi = 3.141592653589793, kPi_2 = 1.5707963267948966, kPi_4 = 0.7853981633974483;
  const double ax = fabs(x), ay = fabs(y);
  if (ay == 0.0 && ax == 0.0) return (x < 0.0) ? (y < 0.0 ? -kPi : kPi) : y;
  const bool swap = ay > ax;
  const double z = swap ? dvd(ax, ay) : dvd(ay, ax);
  const bool big = z > 0.41421356237309503;
  const double w = big ? dvd(sub(z, 1.0), add(z, 1.0)) : z;
  const double w2 = mul(w, w);
  double acc = -0.02127659574468085;
  acc = fmad(acc, w2, 0.022222222222222223);
  acc = fmad(acc, w2, -0.023255813953488372);
  acc = fmad(acc, w2, 0.024390243902439025);
  acc = fmad(acc, w2, -0.02564102564102564);
  acc = fmad(acc, w2, 0.02702702702702703);
  acc = fmad(acc, w2, -0.02857142857142857);
  acc = fmad(acc, w2, 0.030303030303030304);
  acc = fmad(acc, w2, -0.03225806451612903);
  acc = fmad(acc, w2, 0.034482758620689655);
  acc = fmad(acc, w2, -0.037037037037037035);
  acc = fmad(acc, w2, 0.04);
  acc = fmad(acc, w2, -0.043478260869565216);
  acc = fmad(acc, w2, 0.047619047619047616);
  acc = fmad(acc, w2, -0.05263157894736842);
  acc = fmad(acc, w2, 0.058823529411764705);
  acc = fmad(acc, w2, -0.06666666666666667);
  acc = fmad(acc, w2, 0.07692307692307693);
  acc = fmad(acc, w2, -0.09090909090909091);
  acc = fmad(acc, w2, 0.1111111111111111);
  acc = fmad(acc, w2, -0.14285714285714285);
  acc = fmad(acc, w2, 0.2);
  acc = fmad(acc, w2, -0.3333333333333333);
  acc = fmad(acc, w2, 1.0);
  double a = mul(w, acc);
  if (big) a = add(kPi_4, a);
  if (swap) a = sub(kPi_2, a);
  if (x < 0.0) a = sub(kPi, a);
  if (y < 0.0) a = -a;
  return a;
}

// ------------------------------------------------------------------ Pose3
struct P3 {
  double R[9];
  double t[3];
};
__device__ __forceinline__ void p3_identity(P3& p) {
#pragma unroll
  for (int i = 0; i < 9; ++i) p.R[i] = (i % 4 == 0) ? 1.0 : 0.0;
  p.t[0] = p.t[1] = p.t[2] = 0.0;
}
__device__ __forceinline__ void p3_load(const double* s, P3& p) {
#pragma unroll
  for (int i = 0; i < 9; ++i) p.R[i] = s[i];
#pragma unroll
  for (int i = 0; i < 3; ++i) p.t[i] = s[9 + i];
}
__device__ __forceinline__ void p3_store(const P3& p, double* s) {
#pragma unroll
  for (int i = 0; i < 9; ++i) s[i] = p.R[i];
#pragma unroll
  for (int i = 0; i < 3; ++i) s[9 + i] = p.t[i];
}
__device__ __forceinline__ void p3_compose(const P3& A, const P3& B, P3& C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C.R[3 * i + j] = dot3e(A.R[3 * i], A.R[3 * i + 1], A.R[3 * i + 2], B.R[j], B.R[3 + j], B.R[6 + j]);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double acc = fmad(A.R[3 * i], B.t[0], A.t[i]);
    acc = fmad(A.R[3 * i + 1], B.t[1], acc);
    C.t[i] = fmad(A.R[3 * i + 2], B.t[2], acc);
  }
}
__device__ __forceinline__ void p3_inverse(const P3& A, P3& C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C.R[3 * i + j] = A.R[3 * j + i];
#pragma unroll
  for (int i = 0; i < 3; ++i) C.t[i] = -dot3e(A.R[i], A.R[3 + i], A.R[6 + i], A.t[0], A.t[1], A.t[2]);
}
__device__ __forceinline__ void p3_between(const P3& A, const P3& B, P3& C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C.R[3 * i + j] = dot3e(A.R[i], A.R[3 + i], A.R[6 + i], B.R[j], B.R[3 + j], B.R[6 + j]);
  const double d0 = sub(B.t[0], A.t[0]), d1 = sub(B.t[1], A.t[1]), d2 = sub(B.t[2], A.t[2]);
#pragma unroll
  for (int i = 0; i < 3; ++i) C.t[i] = dot3e(A.R[i], A.R[3 + i], A.R[6 + i], d0, d1, d2);
}
__device__ __forceinline__ void p3_adjoint_K(const P3& T, double K[9]) {
  const double t0 = T.t[0], t1 = T.t[1], t2 = T.t[2];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    K[j] = fmad(t1, T.R[6 + j], -mul(t2, T.R[3 + j]));
    K[3 + j] = fmad(t2, T.R[j], -mul(t0, T.R[6 + j]));
    K[6 + j] = fmad(t0, T.R[3 + j], -mul(t1, T.R[j]));
  }
}
// Element (i, k) of M = Ad(T) S, Ad(T) = [[R, 0], [K, R]]
__device__ __forceinline__ double p3_M_elem(const double* R, const double* K, const double* S, int i, int k) {
  const double s0 = S[k], s1 = S[6 + k], s2 = S[12 + k];
  if (i < 3) return dot3e(R[3 * i], R[3 * i + 1], R[3 * i + 2], s0, s1, s2);
  const int r = i - 3;
  double acc = mul(K[3 * r], s0);
  acc = fmad(K[3 * r + 1], s1, acc);
  acc = fmad(K[3 * r + 2], s2, acc);
  acc = fmad(R[3 * r], S[18 + k], acc);
  acc = fmad(R[3 * r + 1], S[24 + k], acc);
  return fmad(R[3 * r + 2], S[30 + k], acc);
}
// Element (i, j), j <= i, of C = M Ad(T)^T (m = row i of M)
__device__ __forceinline__ double p3_C_elem(const double* R, const double* K, const double* m, int j) {
  if (j < 3) return dot3e(m[0], m[1], m[2], R[3 * j], R[3 * j + 1], R[3 * j + 2]);
  const double* kk = K + 3 * (j - 3);
  const double* rr = R + 3 * (j - 3);
  double acc = mul(m[0], kk[0]);
  acc = fmad(m[1], kk[1], acc);
  acc = fmad(m[2], kk[2], acc);
  acc = fmad(m[3], rr[0], acc);
  acc = fmad(m[4], rr[1], acc);
  return fmad(m[5], rr[2], acc);
}
// C = Ad(T) S Ad(T)^T, lower triangle computed, mirrored (S full, row-major)
__device__ __forceinline__ void p3_congruence_RK(const double* R, const double* K, const double* S, double* C) {
  double M[36];
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int i = 0; i < 6; ++i) M[6 * i + k] = p3_M_elem(R, K, S, i, k);
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      const double v = p3_C_elem(R, K, M + 6 * i, j);
      C[6 * i + j] = v;
      C[6 * j + i] = v;
    }
}
__device__ __forceinline__ void p3_congruence(const P3& T, const double* S, double* C) {
  double K[9];
  p3_adjoint_K(T, K);
  p3_congruence_RK(T.R, K, S, C);
}
__device__ __forceinline__ void so3_log(const double* R, double w[3], double& th, double& s_half, double& c_half) {
  const double tr = add(add(R[0], R[4]), R[8]);
  const double vx = sub(R[7], R[5]), vy = sub(R[2], R[6]), vz = sub(R[3], R[1]);
  double sn2 = mul(vx, vx);
  sn2 = fmad(vy, vy, sn2);
  sn2 = fmad(vz, vz, sn2);
  const double sn = sqrtd(sn2);
  const double cs = sub(tr, 1.0);
  th = r_atan2(sn, cs);
  if (cs > -1.6) {
    double k;
    if (th < 0.01) {
      const double t2 = mul(th, th);
      k = fmad(fmad(0.009722222222222222, t2, 0.08333333333333333), t2, 0.5);
    } else {
      k = dvd(th, sn);
    }
    w[0] = mul(k, vx);
    w[1] = mul(k, vy);
    w[2] = mul(k, vz);
  } else {
    const double c = mul(cs, 0.5);
    const double omc = sub(1.0, c);
    int i = 0;
    if (R[4] > R[0]) i = 1;
    if (R[8] > R[4 * i]) i = 2;
    const double ni = sqrtd(dvd(sub(R[4 * i], c), omc));
    const double den = mul(mul(2.0, omc), ni);
    double n[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) n[j] = (j == i) ? ni : dvd(add(R[3 * i + j], R[3 * j + i]), den);
    const double sgn = dot3e(n[0], n[1], n[2], vx, vy, vz);
    const double f = (sgn < 0.0) ? -th : th;
    w[0] = mul(f, n[0]);
    w[1] = mul(f, n[1]);
    w[2] = mul(f, n[2]);
  }
  s_half = mul(sn, 0.5);
  c_half = mul(cs, 0.5);
}
__device__ __forceinline__ void p3_logmap(const P3& T, double xi[6]) {
  double w[3], th, s, c;
  so3_log(T.R, w, th, s, c);
  const double* t = T.t;
  const double W0 = fmad(w[1], t[2], -mul(w[2], t[1]));
  const double W1 = fmad(w[2], t[0], -mul(w[0], t[2]));
  const double W2 = fmad(w[0], t[1], -mul(w[1], t[0]));
  const double V0 = fmad(w[1], W2, -mul(w[2], W1));
  const double V1 = fmad(w[2], W0, -mul(w[0], W2));
  const double V2 = fmad(w[0], W1, -mul(w[1], W0));
  const double t2 = mul(th, th);
  double beta;
  if (th < 0.01) {
    beta = fmad(fmad(3.306878306878307e-05, t2, 0.001388888888888889), t2, 0.08333333333333333);
  } else {
    const double omc = sub(1.0, c);
    const double den = fmad(s, s, mul(omc, omc));
    const double X = dvd(mul(th, s), den);
    beta = dvd(sub(1.0, X), t2);
  }
  xi[0] = w[0];
  xi[1] = w[1];
  xi[2] = w[2];
  xi[3] = fmad(beta, V0, fmad(-0.5, W0, t[0]));
  xi[4] = fmad(beta, V1, fmad(-0.5, W1, t[1]));
  xi[5] = fmad(beta, V2, fmad(-0.5, W2, t[2]));
}

// ------------------------------------------------------------------ Pose2
struct P2 {
  double c, s, x, y;
};
__device__ __forceinline__ void p2_identity(P2& p) { p.c = 1.0; p.s = 0.0; p.x = 0.0; p.y = 0.0; }
__device__ __forceinline__ void p2_load(const double* s, P2& p) { p.c = s[0]; p.s = s[1]; p.x = s[2]; p.y = s[3]; }
__device__ __forceinline__ void p2_store(const P2& p, double* s) { s[0] = p.c; s[1] = p.s; s[2] = p.x; s[3] = p.y; }
__device__ __forceinline__ void p2_compose(const P2& A, const P2& B, P2& C) {
  C.c = fmad(A.c, B.c, -mul(A.s, B.s));
  C.s = fmad(A.s, B.c, mul(A.c, B.s));
  C.x = add(A.x, fmad(A.c, B.x, -mul(A.s, B.y)));
  C.y = add(A.y, fmad(A.s, B.x, mul(A.c, B.y)));
}
__device__ __forceinline__ void p2_inverse(const P2& A, P2& C) {
  C.c = A.c;
  C.s = -A.s;
  C.x = -fmad(A.c, A.x, mul(A.s, A.y));
  C.y = -fmad(A.c, A.y, -mul(A.s, A.x));
}
__device__ __forceinline__ void p2_between(const P2& A, const P2& B, P2& C) {
  C.c = fmad(A.c, B.c, mul(A.s, B.s));
  C.s = fmad(A.c, B.s, -mul(A.s, B.c));
  const double dx = sub(B.x, A.x), dy = sub(B.y, A.y);
  C.x = fmad(A.c, dx, mul(A.s, dy));
  C.y = fmad(A.c, dy, -mul(A.s, dx));
}
__device__ __forceinline__ void p2_adjoint(const P2& T, double A[9]) {
  A[0] = T.c; A[1] = -T.s; A[2] = T.y;
  A[3] = T.s; A[4] = T.c;  A[5] = -T.x;
  A[6] = 0.0; A[7] = 0.0;  A[8] = 1.0;
}
__device__ __forceinline__ double p2_M_elem(const double* A, const double* S, int i, int k) {
  return dot3e(A[3 * i], A[3 * i + 1], A[3 * i + 2], S[k], S[3 + k], S[6 + k]);
}
__device__ __forceinline__ double p2_C_elem(const double* A, const double* m, int j) {
  return dot3e(m[0], m[1], m[2], A[3 * j], A[3 * j + 1], A[3 * j + 2]);
}
__device__ __forceinline__ void p2_congruence(const P2& T, const double* S, double* C) {
  double A[9], M[9];
  p2_adjoint(T, A);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) M[3 * i + k] = p2_M_elem(A, S, i, k);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      const double v = p2_C_elem(A, M + 3 * i, j);
      C[3 * i + j] = v;
      C[3 * j + i] = v;
    }
}
__device__ __forceinline__ void p2_logmap(const P2& T, double xi[3]) {
  const double th = r_atan2(T.s, T.c);
  if (fabs(th) < 1e-10) {
    xi[0] = T.x;
    xi[1] = T.y;
    xi[2] = th;
    return;
  }
  const double omc = sub(1.0, T.c);
  const double det = fmad(T.s, T.s, mul(omc, omc));
  const double k = dvd(th, det);
  xi[0] = mul(k, fmad(T.s, T.x, mul(omc, T.y)));
  xi[1] = mul(k, fmad(T.s, T.y, -mul(omc, T.x)));
  xi[2] = th;
}

// ------------------------------------------------------------------ SPD helpers
// Positive-definiteness test of a symmetric matrix as Eigen's LLT decides it
// (fails when a pivot is <= 0; a NaN pivot passes), evaluated as an LDL^T
// factorisation with reciprocal pivots: the pivots D_j are LLT's L_jj^2, so
// the decision is the same up to rounding, with one division per pivot and
// no square roots (LLT: one division per entry and a square root per pivot).
// Row i: e_j = A_ij - sum_k e_k L_jk (k < j) is L_ij D_j, L_ij = e_j / D_j;
// D_i = A_ii - sum_k e_k L_ik.
template <int N>
__device__ __forceinline__ bool ldlt_factor(const double* A, double* L, double* iD, bool nan_passes) {
#pragma unroll
  for (int i = 0; i < N; ++i) {
    double e[N];
#pragma unroll
    for (int j = 0; j < i; ++j) {
      double acc = A[N * i + j];
#pragma unroll
      for (int k = 0; k < j; ++k) acc = fmad(-e[k], L[N * j + k], acc);
      e[j] = acc;
      L[N * i + j] = mul(acc, iD[j]);
    }
    double acc = A[N * i + i];
#pragma unroll
    for (int k = 0; k < i; ++k) acc = fmad(-e[k], L[N * i + k], acc);
    if (nan_passes ? (acc <= 0.0) : !(acc > 0.0)) return false;
    iD[i] = dvd(1.0, acc);
  }
  return true;
}
template <int N>
__device__ __forceinline__ bool chol_ok(const double* A) {
  double L[N * N], iD[N];
  return ldlt_factor<N>(A, L, iD, true);
}
// x^T A^-1 x: from the LDL^T factors (z = L^-1 x, sum of z_i^2 / D_i); when a
// pivot is <= 0 or NaN, Gaussian elimination with partial pivoting.
template <int N>
__device__ __forceinline__ double quad_inv(const double* A, const double* x) {
  {
    double L[N * N], iD[N];
    if (ldlt_factor<N>(A, L, iD, false)) {
      double z[N];
      double d2 = 0.0;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        double acc = x[i];
#pragma unroll
        for (int k = 0; k < i; ++k) acc = fmad(-L[N * i + k], z[k], acc);
        z[i] = acc;
        const double t = mul(acc, iD[i]);
        d2 = (i == 0) ? mul(t, acc) : fmad(t, acc, d2);
      }
      return d2;
    }
  }
  double M[N * N], b[N], z[N];
  for (int i = 0; i < N * N; ++i) M[i] = A[i];
  for (int i = 0; i < N; ++i) b[i] = x[i];
  for (int col = 0; col < N; ++col) {
    int p = col;
    double best = fabs(M[N * col + col]);
    for (int r = col + 1; r < N; ++r) {
      const double v = fabs(M[N * r + col]);
      if (v > best) { best = v; p = r; }
    }
    if (p != col) {
      for (int c = 0; c < N; ++c) { double tmp = M[N * col + c]; M[N * col + c] = M[N * p + c]; M[N * p + c] = tmp; }
      double tmp = b[col]; b[col] = b[p]; b[p] = tmp;
    }
    const double piv = M[N * col + col];
    for (int r = col + 1; r < N; ++r) {
      const double f = dvd(M[N * r + col], piv);
      for (int c = col + 1; c < N; ++c) M[N * r + c] = fmad(-f, M[N * col + c], M[N * r + c]);
      b[r] = fmad(-f, b[col], b[r]);
    }
  }
  for (int i = N - 1; i >= 0; --i) {
    double acc = b[i];
    for (int k = i + 1; k < N; ++k) acc = fmad(-M[N * i + k], z[k], acc);
    z[i] = dvd(acc, M[N * i + i]);
  }
  double d2 = mul(x[0], z[0]);
  for (int i = 1; i < N; ++i) d2 = fmad(x[i], z[i], d2);
  return d2;
}

}  // namespace pm
}  // namespace rpgo

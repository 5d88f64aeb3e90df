// CPU FP64 oracle — TEST INFRASTRUCTURE ONLY.
//
// This header restates, in plain C++ double arithmetic, the uncertain-pose
// algebra that Kimera-RPGO's PCM outlier rejection runs on every loop
// closure and every pair of loop closures:
//   include/KimeraRPGO/utils/GeometryUtils.h:56-187  PoseWithCovariance
//   include/KimeraRPGO/utils/GeometryUtils.h:193-289 PoseWithNode
// plus the GTSAM Pose2/Pose3 group operations those call (compose, between,
// inverse, AdjointMap, Logmap), restated from the Lie-group mathematics
// (GTSAM is not vendored by the reference).
//
// Every value is produced by a fixed sequence of IEEE-754 double operations
// (+, -, *, /, sqrt, fma), each correctly rounded, so the CUDA kernels that
// follow the same sequence produce bit-identical results. The build must use
// -ffp-contract=off so that no a*b+c is fused behind our back; the fused
// multiply-adds below are explicit std::fma calls.
//
// Conventions (GTSAM): Pose3 tangent order [omega; v], Pose2 tangent order
// [v_x, v_y, omega]; compose Jacobian wrt the first argument is
// Ad(other^-1), wrt the second is I; between Jacobian wrt the first argument
// is -Ad(result^-1).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle {

// ---------------------------------------------------------------- scalars
static inline double fmad(double a, double b, double c) { return std::fma(a, b, c); }

static inline double dot3(const double* a, const double* b) {
  double acc = a[0] * b[0];
  acc = fmad(a[1], b[1], acc);
  return fmad(a[2], b[2], acc);
}
// a and b given element-wise
static inline double dot3e(double a0, double a1, double a2, double b0, double b1, double b2) {
  double acc = a0 * b0;
  acc = fmad(a1, b1, acc);
  return fmad(a2, b2, acc);
}
static inline double dot6e(const double* a3, const double* b3, const double* c3, const double* d3) {
  // (a3 ++ b3) . (c3 ++ d3), accumulated left to right
  double acc = a3[0] * c3[0];
  acc = fmad(a3[1], c3[1], acc);
  acc = fmad(a3[2], c3[2], acc);
  acc = fmad(b3[0], d3[0], acc);
  acc = fmad(b3[1], d3[1], acc);
  return fmad(b3[2], d3[2], acc);
}

// Own atan2: argument reduction to |w| <= tan(pi/8) and the Taylor series of
// atan (coefficients (-1)^k/(2k+1)), evaluated by Horner in w^2. Only IEEE
// basic operations are used so that host and device agree bit for bit.
static const double kAtanCoef[24] = {
    1.0, -0.3333333333333333, 0.2, -0.14285714285714285, 0.1111111111111111,
    -0.09090909090909091, 0.07692307692307693, -0.06666666666666667,
    0.058823529411764705, -0.05263157894736842, 0.047619047619047616,
    -0.043478260869565216, 0.04, -0.037037037037037035, 0.034482758620689655,
    -0.03225806451612903, 0.030303030303030304, -0.02857142857142857,
    0.02702702702702703, -0.02564102564102564, 0.024390243902439025,
    -0.023255813953488372, 0.022222222222222223, -0.02127659574468085};
static const double kPi = 3.141592653589793;
static const double kPi_2 = 1.5707963267948966;
static const double kPi_4 = 0.7853981633974483;
static const double kTanPi_8 = 0.41421356237309503;

static inline double r_atan2(double y, double x) {
  const double ax = std::fabs(x), ay = std::fabs(y);
  if (ay == 0.0 && ax == 0.0) return (x < 0.0) ? (y < 0.0 ? -kPi : kPi) : y;
  const bool swap = ay > ax;
  const double z = swap ? (ax / ay) : (ay / ax);
  const bool big = z > kTanPi_8;
  const double w = big ? ((z - 1.0) / (z + 1.0)) : z;
  const double w2 = w * w;
  double acc = kAtanCoef[23];
  for (int k = 22; k >= 0; --k) acc = fmad(acc, w2, kAtanCoef[k]);
  double a = w * acc;
  if (big) a = kPi_4 + a;
  if (swap) a = kPi_2 - a;
  if (x < 0.0) a = kPi - a;
  if (y < 0.0) a = -a;
  return a;
}

// ---------------------------------------------------------------- Pose3
struct P3 {
  double R[9];  // row-major rotation
  double t[3];
};
static inline P3 p3_identity() {
  P3 p;
  std::memset(&p, 0, sizeof(p));
  p.R[0] = p.R[4] = p.R[8] = 1.0;
  return p;
}
static inline P3 p3_compose(const P3& A, const P3& B) {
  P3 C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C.R[3 * i + j] = dot3e(A.R[3 * i], A.R[3 * i + 1], A.R[3 * i + 2], B.R[j], B.R[3 + j], B.R[6 + j]);
  for (int i = 0; i < 3; ++i) {
    double acc = fmad(A.R[3 * i], B.t[0], A.t[i]);
    acc = fmad(A.R[3 * i + 1], B.t[1], acc);
    C.t[i] = fmad(A.R[3 * i + 2], B.t[2], acc);
  }
  return C;
}
static inline P3 p3_inverse(const P3& A) {
  P3 C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C.R[3 * i + j] = A.R[3 * j + i];
  for (int i = 0; i < 3; ++i) C.t[i] = -dot3e(A.R[i], A.R[3 + i], A.R[6 + i], A.t[0], A.t[1], A.t[2]);
  return C;
}
// A^-1 * B  ==  (A.R^T B.R, A.R^T (B.t - A.t))
static inline P3 p3_between(const P3& A, const P3& B) {
  P3 C;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C.R[3 * i + j] = dot3e(A.R[i], A.R[3 + i], A.R[6 + i], B.R[j], B.R[3 + j], B.R[6 + j]);
  const double d0 = B.t[0] - A.t[0], d1 = B.t[1] - A.t[1], d2 = B.t[2] - A.t[2];
  for (int i = 0; i < 3; ++i) C.t[i] = dot3e(A.R[i], A.R[3 + i], A.R[6 + i], d0, d1, d2);
  return C;
}
// K = [t]x R (bottom-left block of the Pose3 adjoint in [omega; v] order)
static inline void p3_adjoint_K(const P3& T, double K[9]) {
  const double* R = T.R;
  const double t0 = T.t[0], t1 = T.t[1], t2 = T.t[2];
  for (int j = 0; j < 3; ++j) {
    K[j] = fmad(t1, R[6 + j], -(t2 * R[3 + j]));
    K[3 + j] = fmad(t2, R[j], -(t0 * R[6 + j]));
    K[6 + j] = fmad(t0, R[3 + j], -(t1 * R[j]));
  }
}
// C = Ad(T) S Ad(T)^T for a 6x6 covariance S (row-major, full). The lower
// triangle is computed and mirrored. Ad(T) = [[R, 0], [K, R]].
static inline void p3_congruence(const P3& T, const double S[36], double C[36]) {
  double K[9];
  p3_adjoint_K(T, K);
  const double* R = T.R;
  double M[36];  // M = Ad S
  for (int k = 0; k < 6; ++k) {
    const double s0 = S[k], s1 = S[6 + k], s2 = S[12 + k], s3 = S[18 + k], s4 = S[24 + k], s5 = S[30 + k];
    for (int i = 0; i < 3; ++i) {
      M[6 * i + k] = dot3e(R[3 * i], R[3 * i + 1], R[3 * i + 2], s0, s1, s2);
      double acc = K[3 * i] * s0;
      acc = fmad(K[3 * i + 1], s1, acc);
      acc = fmad(K[3 * i + 2], s2, acc);
      acc = fmad(R[3 * i], s3, acc);
      acc = fmad(R[3 * i + 1], s4, acc);
      M[6 * (i + 3) + k] = fmad(R[3 * i + 2], s5, acc);
    }
  }
  for (int i = 0; i < 6; ++i) {
    const double* m = M + 6 * i;
    for (int j = 0; j <= i; ++j) {
      double v;
      if (j < 3) v = dot3(m, R + 3 * j);
      else v = dot6e(m, m + 3, K + 3 * (j - 3), R + 3 * (j - 3));
      C[6 * i + j] = v;
      C[6 * j + i] = v;
    }
  }
}

// SO(3) logarithm. theta from atan2(|v|, tr-1); axis from the skew part away
// from pi and from the symmetric part near pi.
static inline void so3_log(const double* R, double w[3], double* theta_out, double* sin_out, double* cos_out) {
  const double tr = (R[0] + R[4]) + R[8];
  const double vx = R[7] - R[5], vy = R[2] - R[6], vz = R[3] - R[1];
  double sn2 = vx * vx;
  sn2 = fmad(vy, vy, sn2);
  sn2 = fmad(vz, vz, sn2);
  const double sn = std::sqrt(sn2);  // 2 sin(theta)
  const double cs = tr - 1.0;        // 2 cos(theta)
  const double th = r_atan2(sn, cs);
  if (cs > -1.6) {
    double k;
    if (th < 0.01) {
      const double t2 = th * th;
      k = fmad(fmad(0.009722222222222222, t2, 0.08333333333333333), t2, 0.5);
    } else {
      k = th / sn;
    }
    w[0] = k * vx;
    w[1] = k * vy;
    w[2] = k * vz;
  } else {
    const double c = cs * 0.5;
    const double omc = 1.0 - c;
    int i = 0;
    if (R[4] > R[0]) i = 1;
    if (R[8] > R[4 * i]) i = 2;
    const double ni = std::sqrt((R[4 * i] - c) / omc);
    const double den = (2.0 * omc) * ni;
    double n[3];
    for (int j = 0; j < 3; ++j) n[j] = (j == i) ? ni : ((R[3 * i + j] + R[3 * j + i]) / den);
    const double sgn = dot3e(n[0], n[1], n[2], vx, vy, vz);
    const double f = (sgn < 0.0) ? -th : th;
    w[0] = f * n[0];
    w[1] = f * n[1];
    w[2] = f * n[2];
  }
  if (theta_out) *theta_out = th;
  if (sin_out) *sin_out = sn * 0.5;
  if (cos_out) *cos_out = cs * 0.5;
}

// SE(3) logarithm, [omega; v]: v = t - 1/2 w x t + beta w x (w x t),
// beta = (1 - theta sin / (sin^2 + (1-cos)^2)) / theta^2 (Taylor for small theta)
static inline void p3_logmap(const P3& T, double xi[6]) {
  double w[3], th, s, c;
  so3_log(T.R, w, &th, &s, &c);
  const double* t = T.t;
  const double W0 = fmad(w[1], t[2], -(w[2] * t[1]));
  const double W1 = fmad(w[2], t[0], -(w[0] * t[2]));
  const double W2 = fmad(w[0], t[1], -(w[1] * t[0]));
  const double V0 = fmad(w[1], W2, -(w[2] * W1));
  const double V1 = fmad(w[2], W0, -(w[0] * W2));
  const double V2 = fmad(w[0], W1, -(w[1] * W0));
  const double t2 = th * th;
  double beta;
  if (th < 0.01) {
    beta = fmad(fmad(3.306878306878307e-05, t2, 0.001388888888888889), t2, 0.08333333333333333);
  } else {
    const double omc = 1.0 - c;
    const double den = fmad(s, s, omc * omc);
    const double X = (th * s) / den;
    beta = (1.0 - X) / t2;
  }
  xi[0] = w[0];
  xi[1] = w[1];
  xi[2] = w[2];
  xi[3] = fmad(beta, V0, fmad(-0.5, W0, t[0]));
  xi[4] = fmad(beta, V1, fmad(-0.5, W1, t[1]));
  xi[5] = fmad(beta, V2, fmad(-0.5, W2, t[2]));
}

// ---------------------------------------------------------------- Pose2
struct P2 {
  double c, s, x, y;
};
static inline P2 p2_identity() { return P2{1.0, 0.0, 0.0, 0.0}; }
static inline P2 p2_compose(const P2& A, const P2& B) {
  P2 C;
  C.c = fmad(A.c, B.c, -(A.s * B.s));
  C.s = fmad(A.s, B.c, A.c * B.s);
  C.x = A.x + fmad(A.c, B.x, -(A.s * B.y));
  C.y = A.y + fmad(A.s, B.x, A.c * B.y);
  return C;
}
static inline P2 p2_inverse(const P2& A) {
  P2 C;
  C.c = A.c;
  C.s = -A.s;
  C.x = -fmad(A.c, A.x, A.s * A.y);
  C.y = -fmad(A.c, A.y, -(A.s * A.x));
  return C;
}
static inline P2 p2_between(const P2& A, const P2& B) {
  P2 C;
  C.c = fmad(A.c, B.c, A.s * B.s);
  C.s = fmad(A.c, B.s, -(A.s * B.c));
  const double dx = B.x - A.x, dy = B.y - A.y;
  C.x = fmad(A.c, dx, A.s * dy);
  C.y = fmad(A.c, dy, -(A.s * dx));
  return C;
}
// Ad(T) = [[c, -s, y], [s, c, -x], [0, 0, 1]] in [v_x, v_y, omega] order
static inline void p2_adjoint(const P2& T, double A[9]) {
  A[0] = T.c; A[1] = -T.s; A[2] = T.y;
  A[3] = T.s; A[4] = T.c;  A[5] = -T.x;
  A[6] = 0.0; A[7] = 0.0;  A[8] = 1.0;
}
static inline void p2_congruence(const P2& T, const double S[9], double C[9]) {
  double A[9], M[9];
  p2_adjoint(T, A);
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) M[3 * i + k] = dot3e(A[3 * i], A[3 * i + 1], A[3 * i + 2], S[k], S[3 + k], S[6 + k]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j <= i; ++j) {
      const double v = dot3(M + 3 * i, A + 3 * j);
      C[3 * i + j] = v;
      C[3 * j + i] = v;
    }
}
static inline void p2_logmap(const P2& T, double xi[3]) {
  const double th = r_atan2(T.s, T.c);
  if (std::fabs(th) < 1e-10) {
    xi[0] = T.x;
    xi[1] = T.y;
    xi[2] = th;
    return;
  }
  const double omc = 1.0 - T.c;
  const double det = fmad(T.s, T.s, omc * omc);
  const double k = th / det;
  xi[0] = k * fmad(T.s, T.x, omc * T.y);
  xi[1] = k * fmad(T.s, T.y, -(omc * T.x));
  xi[2] = th;
}

// ---------------------------------------------------------------- dense SPD helpers
// Positive-definiteness test of a symmetric matrix as Eigen's LLT decides it
// (fails when a pivot is <= 0; a NaN pivot passes), evaluated as an LDL^T
// factorisation with reciprocal pivots (the pivots D_j are LLT's L_jj^2):
// row i: e_j = A_ij - sum_k e_k L_jk (k < j), L_ij = e_j * (1 / D_j);
// D_i = A_ii - sum_k e_k L_ik. The GPU kernels evaluate the same sequence.
static inline bool ldlt_factor(const double* A, int n, double* L, double* iD, bool nan_passes) {
  for (int i = 0; i < n; ++i) {
    double e[6];
    for (int j = 0; j < i; ++j) {
      double acc = A[n * i + j];
      for (int k = 0; k < j; ++k) acc = fmad(-e[k], L[n * j + k], acc);
      e[j] = acc;
      L[n * i + j] = acc * iD[j];
    }
    double acc = A[n * i + i];
    for (int k = 0; k < i; ++k) acc = fmad(-e[k], L[n * i + k], acc);
    if (nan_passes ? (acc <= 0.0) : !(acc > 0.0)) return false;
    iD[i] = 1.0 / acc;
  }
  return true;
}
static inline bool llt_ok(const double* A, int n) {
  double L[36], iD[6];
  return ldlt_factor(A, n, L, iD, true);
}
// x^T A^-1 x for symmetric A: from the LDL^T factors (z = L^-1 x, sum of
// z_i^2 / D_i); if a pivot is <= 0 or NaN, Gaussian elimination with partial
// pivoting.
static inline double quad_inv(const double* A, int n, const double* x) {
  {
    double L[36], iD[6];
    if (ldlt_factor(A, n, L, iD, false)) {
      double z[6];
      double d2 = 0.0;
      for (int i = 0; i < n; ++i) {
        double acc = x[i];
        for (int k = 0; k < i; ++k) acc = fmad(-L[n * i + k], z[k], acc);
        z[i] = acc;
        const double t = acc * iD[i];
        d2 = (i == 0) ? t * acc : fmad(t, acc, d2);
      }
      return d2;
    }
  }
  double M[36], b[6], z[6];
  for (int i = 0; i < n * n; ++i) M[i] = A[i];
  for (int i = 0; i < n; ++i) b[i] = x[i];
  for (int col = 0; col < n; ++col) {
    int p = col;
    double best = std::fabs(M[n * col + col]);
    for (int r = col + 1; r < n; ++r) {
      const double v = std::fabs(M[n * r + col]);
      if (v > best) { best = v; p = r; }
    }
    if (p != col) {
      for (int c = 0; c < n; ++c) { double tmp = M[n * col + c]; M[n * col + c] = M[n * p + c]; M[n * p + c] = tmp; }
      double tmp = b[col]; b[col] = b[p]; b[p] = tmp;
    }
    const double piv = M[n * col + col];
    for (int r = col + 1; r < n; ++r) {
      const double f = M[n * r + col] / piv;
      for (int c = col + 1; c < n; ++c) M[n * r + c] = fmad(-f, M[n * col + c], M[n * r + c]);
      b[r] = fmad(-f, b[col], b[r]);
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double acc = b[i];
    for (int k = i + 1; k < n; ++k) acc = fmad(-M[n * i + k], z[k], acc);
    z[i] = acc / M[n * i + i];
  }
  double d2 = x[0] * z[0];
  for (int i = 1; i < n; ++i) d2 = fmad(x[i], z[i], d2);
  return d2;
}

}  // namespace oracle

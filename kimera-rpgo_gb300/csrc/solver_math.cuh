// Device Lie-group algebra of the nonlinear least-squares solve (FP64).
//
// What GTSAM provides to RobustSolver::optimize (src/RobustSolver.cpp:115-306)
// through BetweenFactor<Pose3|Pose2> / PriorFactor and the EXPMAP chart:
//   e_between = Logmap(Z^-1 (Xi^-1 Xj)),  J_i = -D Ad((Xi^-1 Xj)^-1), J_j = D,
//   D = LogmapDerivative(e) (inverse right Jacobian, exact),
//   e_prior   = -Logmap(X^-1 P), J = I,
//   retraction X <- X Expmap(delta).
// SE(3) right-Jacobian block Q from Barfoot & Furgale (IEEE TRO 2014, eq. 102)
// with odd orders negated for the right Jacobian; SE(2) right Jacobian from
// its closed form (Sola et al., "A micro Lie theory", 2018).
#pragma once
#include "pcm_math.cuh"

namespace rpgo {
namespace sm {

using pm::P2;
using pm::P3;

__device__ __forceinline__ void mat3mul(const double* A, const double* B, double* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}
__device__ __forceinline__ void skew(const double* w, double* W) {
  W[0] = 0; W[1] = -w[2]; W[2] = w[1];
  W[3] = w[2]; W[4] = 0; W[5] = -w[0];
  W[6] = -w[1]; W[7] = w[0]; W[8] = 0;
}

__device__ __forceinline__ void se3_exp(const double* xi, P3& T) {
  const double* w = xi;
  const double* v = xi + 3;
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double th = sqrt(th2);
  double A, B, C;
  if (th < 1e-4) {
    A = 1.0 - th2 / 6.0;
    B = 0.5 - th2 / 24.0;
    C = 1.0 / 6.0 - th2 / 120.0;
  } else {
    double s, c;
    sincos(th, &s, &c);
    A = s / th;
    B = (1.0 - c) / th2;
    C = (th - s) / (th2 * th);
  }
  double W[9], W2[9];
  skew(w, W);
  mat3mul(W, W, W2);
#pragma unroll
  for (int i = 0; i < 9; ++i) T.R[i] = A * W[i] + B * W2[i] + ((i % 4 == 0) ? 1.0 : 0.0);
  double V[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) V[i] = B * W[i] + C * W2[i] + ((i % 4 == 0) ? 1.0 : 0.0);
#pragma unroll
  for (int i = 0; i < 3; ++i) T.t[i] = V[3 * i] * v[0] + V[3 * i + 1] * v[1] + V[3 * i + 2] * v[2];
}

// 6x6 adjoint [[R, 0], [[t]x R, R]]
__device__ __forceinline__ void se3_adjoint(const P3& T, double* Ad) {
  double K[9];
  pm::p3_adjoint_K(T, K);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      Ad[6 * i + j] = T.R[3 * i + j];
      Ad[6 * i + j + 3] = 0.0;
      Ad[6 * (i + 3) + j] = K[3 * i + j];
      Ad[6 * (i + 3) + j + 3] = T.R[3 * i + j];
    }
}

// inverse right Jacobian of SE(3) at xi = [w; rho]
__device__ __forceinline__ void se3_logmap_derivative(const double* xi, double* J) {
  const double* w = xi;
  const double* r = xi + 3;
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double th = sqrt(th2);
  double a, b, c, beta;
  if (th < 0.05) {
    a = 1.0 / 6.0 - th2 / 120.0 + th2 * th2 / 5040.0;
    b = -1.0 / 24.0 + th2 / 720.0 - th2 * th2 / 40320.0;
    c = 1.0 / 120.0 - th2 / 2520.0 + th2 * th2 / 120960.0;
    beta = 1.0 / 12.0 + th2 / 720.0 + th2 * th2 / 30240.0;
  } else {
    double s, co;
    sincos(th, &s, &co);
    a = (th - s) / (th2 * th);
    b = (1.0 - th2 / 2.0 - co) / (th2 * th2);
    c = (2.0 * th - 3.0 * s + th * co) / (2.0 * th2 * th2 * th);
    beta = (1.0 - th * s / (2.0 * (1.0 - co))) / th2;
  }
  // Q of the SE(3) Jacobian, with the products of the skew matrices W = [w]x
  // and V = [r]x in closed form ([a]x[b]x = b a^T - (a.b) I, [a]x[b]x[a]x =
  // -(a.b)[a]x): WV + VW - WVW = r w^T + w r^T - 2 (w.r) I + (w.r) W;
  // WWV + VWW - 3 WVW = w (w x r)^T - (w x r) w^T - 2 th2 V + 3 (w.r) W;
  // WVWW + WWVW = -2 (w.r) WW, with WW = w w^T - th2 I
  double W[9], V[9], WW[9], T1[9];
  skew(w, W);
  skew(r, V);
  const double wr = w[0] * r[0] + w[1] * r[1] + w[2] * r[2];
  const double wxr[3] = {w[1] * r[2] - w[2] * r[1], w[2] * r[0] - w[0] * r[2], w[0] * r[1] - w[1] * r[0]};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) WW[3 * i + j] = w[i] * w[j] - (i == j ? th2 : 0.0);
  double Q[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int k = 3 * i + j;
      const double ta = r[i] * w[j] + w[i] * r[j] - (i == j ? 2.0 * wr : 0.0) + wr * W[k];
      const double tb = w[i] * wxr[j] - wxr[i] * w[j] - 2.0 * th2 * V[k] + 3.0 * wr * W[k];
      Q[k] = -0.5 * V[k] + a * ta + b * tb - 2.0 * c * wr * WW[k];
    }
  double Ji[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) Ji[i] = 0.5 * W[i] + beta * WW[i] + ((i % 4 == 0) ? 1.0 : 0.0);
  double T2[9];
  mat3mul(Ji, Q, T1);
  mat3mul(T1, Ji, T2);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      J[6 * i + j] = Ji[3 * i + j];
      J[6 * i + j + 3] = 0.0;
      J[6 * (i + 3) + j] = -T2[3 * i + j];
      J[6 * (i + 3) + j + 3] = Ji[3 * i + j];
    }
}

__device__ __forceinline__ void se2_exp(const double* xi, P2& T) {
  const double w = xi[2];
  double s, c;
  sincos(w, &s, &c);
  double A, B;
  if (fabs(w) < 1e-6) {
    A = 1.0 - w * w / 6.0;
    B = 0.5 * w;
  } else {
    A = s / w;
    B = (1.0 - c) / w;
  }
  T.c = c;
  T.s = s;
  T.x = A * xi[0] - B * xi[1];
  T.y = B * xi[0] + A * xi[1];
}
__device__ __forceinline__ void se2_adjoint(const P2& T, double* Ad) { pm::p2_adjoint(T, Ad); }
__device__ __forceinline__ void se2_logmap_derivative(const double* xi, double* J) {
  const double v1 = xi[0], v2 = xi[1], w = xi[2];
  double Ai[4], bv[2];
  if (fabs(w) < 1e-6) {
    const double det = 1.0 + w * w / 4.0;
    Ai[0] = 1.0 / det; Ai[1] = -0.5 * w / det; Ai[2] = 0.5 * w / det; Ai[3] = 1.0 / det;
    bv[0] = -0.5 * v2 + v1 * w / 6.0;
    bv[1] = 0.5 * v1 + v2 * w / 6.0;
  } else {
    double s, c;
    sincos(w, &s, &c);
    const double omc = 1.0 - c;
    const double k = w / (s * s + omc * omc);
    Ai[0] = k * s; Ai[1] = -k * omc; Ai[2] = k * omc; Ai[3] = k * s;
    bv[0] = (w * v1 - v2 + v2 * c - v1 * s) / (w * w);
    bv[1] = (v1 + w * v2 - v1 * c - v2 * s) / (w * w);
  }
  J[0] = Ai[0]; J[1] = Ai[1]; J[2] = -(Ai[0] * bv[0] + Ai[1] * bv[1]);
  J[3] = Ai[2]; J[4] = Ai[3]; J[5] = -(Ai[2] * bv[0] + Ai[3] * bv[1]);
  J[6] = 0.0; J[7] = 0.0; J[8] = 1.0;
}

template <int DIM>
struct SLie;
template <>
struct SLie<3> {
  using Pose = P3;
  static constexpr int d = 6, stride = 12;
  __device__ static void load(const double* s, Pose& p) { pm::p3_load(s, p); }
  __device__ static void store(const Pose& p, double* s) { pm::p3_store(p, s); }
  __device__ static void compose(const Pose& a, const Pose& b, Pose& c) { pm::p3_compose(a, b, c); }
  __device__ static void inverse(const Pose& a, Pose& c) { pm::p3_inverse(a, c); }
  __device__ static void between(const Pose& a, const Pose& b, Pose& c) { pm::p3_between(a, b, c); }
  __device__ static void logmap(const Pose& T, double* xi) { pm::p3_logmap(T, xi); }
  __device__ static void exp(const double* xi, Pose& T) { se3_exp(xi, T); }
  __device__ static void adjoint(const Pose& T, double* Ad) { se3_adjoint(T, Ad); }
  __device__ static void dlog(const double* xi, double* J) { se3_logmap_derivative(xi, J); }
};
template <>
struct SLie<2> {
  using Pose = P2;
  static constexpr int d = 3, stride = 4;
  __device__ static void load(const double* s, Pose& p) { pm::p2_load(s, p); }
  __device__ static void store(const Pose& p, double* s) { pm::p2_store(p, s); }
  __device__ static void compose(const Pose& a, const Pose& b, Pose& c) { pm::p2_compose(a, b, c); }
  __device__ static void inverse(const Pose& a, Pose& c) { pm::p2_inverse(a, c); }
  __device__ static void between(const Pose& a, const Pose& b, Pose& c) { pm::p2_between(a, b, c); }
  __device__ static void logmap(const Pose& T, double* xi) { pm::p2_logmap(T, xi); }
  __device__ static void exp(const double* xi, Pose& T) { se2_exp(xi, T); }
  __device__ static void adjoint(const Pose& T, double* Ad) { se2_adjoint(T, Ad); }
  __device__ static void dlog(const double* xi, double* J) { se2_logmap_derivative(xi, J); }
};

}  // namespace sm
}  // namespace rpgo

// CPU FP64 oracle — TEST INFRASTRUCTURE ONLY.
//
// Restatement of the nonlinear least-squares half of Kimera-RPGO's robust
// back-end: RobustSolver::optimize (src/RobustSolver.cpp:115-306) and
// GenericSolver (src/GenericSolver.cpp:37-65). The arithmetic lives in GTSAM
// (commit 686e16aaae26c9a4f23d4af7f2d4a504125ec9c3, README.md:37, built with
// GTSAM_POSE3_EXPMAP / GTSAM_ROT3_EXPMAP, README.md:52), which the reference
// does not vendor; it is restated here from its documented behaviour:
//  * BetweenFactor<T>: e = Logmap(Z^-1 * (Xi^-1 Xj)) with the exact Logmap
//    derivative (SLOW_BUT_CORRECT_BETWEENFACTOR), J_i = -D Ad((Xi^-1 Xj)^-1),
//    J_j = D, whitened by the upper-triangular square-root information R.
//  * PriorFactor<T>: e = -Logmap(X^-1 P), Jacobian I.
//  * Retraction X <- X * Expmap(delta); factor error 0.5 * w * |R e|^2.
//  * LevenbergMarquardtParams defaults: lambdaInitial 1e-5, lambdaFactor 10,
//    lambdaUpperBound 1e5, lambdaLowerBound 0, minModelFidelity 1e-3,
//    minDiagonal 1e-6, maxDiagonal 1e32, fixed lambda factor; damping
//    lambda*clamp(diag(H)) (diagonalDamping) or lambda*I.
//  * NonlinearOptimizerParams defaults: maxIterations 100, relativeErrorTol
//    1e-5, absoluteErrorTol 1e-5, errorTol 0.
//  * GncOptimizer with the TLS loss (Yang et al., RA-L 2020): every outer
//    iteration re-solves the weighted problem from the initial values;
//    mu_0 = min_k barcSq/(2 r_k - barcSq) over factors with 2 r_k > barcSq
//    (clamped below at 1e-6; no such factor => stop); TLS weights from the
//    bounds mu/(mu+1) barcSq and (mu+1)/mu barcSq; mu *= muStep; stop on
//    relative cost change, binary weights (weightsTol) or maxIterations;
//    threshold at probability alpha is 0.5 * chi2inv(alpha, dim).
// The sparse linear solve is a block Cholesky in minimum-degree order.
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>
#include <map>
#include <set>
#include <stdexcept>
#include <unordered_set>
#include <vector>

#include "oracle_pcm.hpp"

namespace oracle {

// ---------------------------------------------------------------- small dense helpers
static inline void matmul(const double* A, const double* B, double* C, int n, int k, int m) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) {
      double acc = 0.0;
      for (int l = 0; l < k; ++l) acc += A[i * k + l] * B[l * m + j];
      C[i * m + j] = acc;
    }
}
static inline void skew(const double* w, double* W) {
  W[0] = 0; W[1] = -w[2]; W[2] = w[1];
  W[3] = w[2]; W[4] = 0; W[5] = -w[0];
  W[6] = -w[1]; W[7] = w[0]; W[8] = 0;
}

// ---------------------------------------------------------------- SE(3) for the solver
static inline P3 se3_exp(const double* xi) {
  const double* w = xi;
  const double* v = xi + 3;
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double th = std::sqrt(th2);
  double A, B, C;
  if (th < 1e-4) {
    A = 1.0 - th2 / 6.0;
    B = 0.5 - th2 / 24.0;
    C = 1.0 / 6.0 - th2 / 120.0;
  } else {
    A = std::sin(th) / th;
    B = (1.0 - std::cos(th)) / th2;
    C = (th - std::sin(th)) / (th2 * th);
  }
  double W[9], W2[9];
  skew(w, W);
  matmul(W, W, W2, 3, 3, 3);
  P3 T;
  for (int i = 0; i < 9; ++i) T.R[i] = A * W[i] + B * W2[i] + ((i % 4 == 0) ? 1.0 : 0.0);
  double V[9];
  for (int i = 0; i < 9; ++i) V[i] = B * W[i] + C * W2[i] + ((i % 4 == 0) ? 1.0 : 0.0);
  for (int i = 0; i < 3; ++i) T.t[i] = V[3 * i] * v[0] + V[3 * i + 1] * v[1] + V[3 * i + 2] * v[2];
  return T;
}
// Full 6x6 adjoint of T in [omega; v] order
static inline void se3_adjoint(const P3& T, double Ad[36]) {
  double K[9];
  p3_adjoint_K(T, K);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      Ad[6 * i + j] = T.R[3 * i + j];
      Ad[6 * i + j + 3] = 0.0;
      Ad[6 * (i + 3) + j] = K[3 * i + j];
      Ad[6 * (i + 3) + j + 3] = T.R[3 * i + j];
    }
}
// Inverse of the right Jacobian of SE(3) at xi = [w; rho] (GTSAM
// Pose3::LogmapDerivative): [[Jw^-1, 0], [-Jw^-1 Q Jw^-1, Jw^-1]], Q from
// Barfoot & Furgale (TRO 2014, eq. 102) with odd orders negated.
static inline void se3_logmap_derivative(const double* xi, double J[36]) {
  const double* w = xi;
  const double* r = xi + 3;
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double th = std::sqrt(th2);
  double a, b, c, beta;
  if (th < 0.05) {
    a = 1.0 / 6.0 - th2 / 120.0 + th2 * th2 / 5040.0;
    b = -1.0 / 24.0 + th2 / 720.0 - th2 * th2 / 40320.0;
    c = 1.0 / 120.0 - th2 / 2520.0 + th2 * th2 / 120960.0;
    beta = 1.0 / 12.0 + th2 / 720.0 + th2 * th2 / 30240.0;
  } else {
    const double s = std::sin(th), co = std::cos(th);
    a = (th - s) / (th2 * th);
    b = (1.0 - th2 / 2.0 - co) / (th2 * th2);
    c = (2.0 * th - 3.0 * s + th * co) / (2.0 * th2 * th2 * th);
    beta = (1.0 - th * s / (2.0 * (1.0 - co))) / th2;
  }
  double W[9], V[9], WV[9], VW[9], WVW[9], WW[9], WWV[9], VWW[9], WVWW[9], WWVW[9];
  skew(w, W);
  skew(r, V);
  matmul(W, V, WV, 3, 3, 3);
  matmul(V, W, VW, 3, 3, 3);
  matmul(WV, W, WVW, 3, 3, 3);
  matmul(W, W, WW, 3, 3, 3);
  matmul(WW, V, WWV, 3, 3, 3);
  matmul(VW, W, VWW, 3, 3, 3);
  matmul(WVW, W, WVWW, 3, 3, 3);
  matmul(W, WVW, WWVW, 3, 3, 3);
  double Q[9], Ji[9];
  for (int i = 0; i < 9; ++i) {
    Q[i] = -0.5 * V[i] + a * (WV[i] + VW[i] - WVW[i]) + b * (WWV[i] + VWW[i] - 3.0 * WVW[i]) +
           c * (WVWW[i] + WWVW[i]);
    Ji[i] = 0.5 * W[i] + beta * WW[i] + ((i % 4 == 0) ? 1.0 : 0.0);
  }
  double T1[9], T2[9];
  matmul(Ji, Q, T1, 3, 3, 3);
  matmul(T1, Ji, T2, 3, 3, 3);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      J[6 * i + j] = Ji[3 * i + j];
      J[6 * i + j + 3] = 0.0;
      J[6 * (i + 3) + j] = -T2[3 * i + j];
      J[6 * (i + 3) + j + 3] = Ji[3 * i + j];
    }
}

// ---------------------------------------------------------------- SE(2) for the solver
static inline P2 se2_exp(const double* xi) {
  const double w = xi[2];
  const double c = std::cos(w), s = std::sin(w);
  double A, B;  // sin w / w, (1 - cos w) / w
  if (std::fabs(w) < 1e-6) {
    A = 1.0 - w * w / 6.0;
    B = 0.5 * w;
  } else {
    A = s / w;
    B = (1.0 - c) / w;
  }
  return P2{c, s, A * xi[0] - B * xi[1], B * xi[0] + A * xi[1]};
}
static inline void se2_adjoint(const P2& T, double Ad[9]) { p2_adjoint(T, Ad); }
// Inverse right Jacobian of SE(2) at xi = [v1, v2, w]
static inline void se2_logmap_derivative(const double* xi, double J[9]) {
  const double v1 = xi[0], v2 = xi[1], w = xi[2];
  double Ai[4], bvec[2];
  if (std::fabs(w) < 1e-6) {
    // J_r ~ [[1, w/2, -v2/2], [-w/2, 1, v1/2], [0,0,1]]
    const double det = 1.0 + w * w / 4.0;
    Ai[0] = 1.0 / det; Ai[1] = -0.5 * w / det; Ai[2] = 0.5 * w / det; Ai[3] = 1.0 / det;
    bvec[0] = -0.5 * v2 + v1 * w / 6.0;
    bvec[1] = 0.5 * v1 + v2 * w / 6.0;
  } else {
    const double s = std::sin(w), c = std::cos(w);
    const double omc = 1.0 - c;
    const double k = w / (s * s + omc * omc);
    Ai[0] = k * s; Ai[1] = -k * omc; Ai[2] = k * omc; Ai[3] = k * s;
    bvec[0] = (w * v1 - v2 + v2 * c - v1 * s) / (w * w);
    bvec[1] = (v1 + w * v2 - v1 * c - v2 * s) / (w * w);
  }
  J[0] = Ai[0]; J[1] = Ai[1]; J[2] = -(Ai[0] * bvec[0] + Ai[1] * bvec[1]);
  J[3] = Ai[2]; J[4] = Ai[3]; J[5] = -(Ai[2] * bvec[0] + Ai[3] * bvec[1]);
  J[6] = 0.0; J[7] = 0.0; J[8] = 1.0;
}

// ---------------------------------------------------------------- solver traits
struct Sol3 {
  using L = Lie3;
  using Pose = P3;
  static constexpr int d = 6;
  static Pose exp(const double* xi) { return se3_exp(xi); }
  static void adjoint(const Pose& T, double* Ad) { se3_adjoint(T, Ad); }
  static void logmap_derivative(const double* xi, double* J) { se3_logmap_derivative(xi, J); }
};
struct Sol2 {
  using L = Lie2;
  using Pose = P2;
  static constexpr int d = 3;
  static Pose exp(const double* xi) { return se2_exp(xi); }
  static void adjoint(const Pose& T, double* Ad) { se2_adjoint(T, Ad); }
  static void logmap_derivative(const double* xi, double* J) { se2_logmap_derivative(xi, J); }
};

// whitened residual and Jacobians of one factor, scaled by sqrt(w)
template <class S>
static inline void linearize_factor(const Factor<typename S::L>& f, const typename S::Pose& Xi,
                                    const typename S::Pose& Xj, double w, double* r, double* Ji, double* Jj) {
  using L = typename S::L;
  constexpr int d = S::d;
  double e[d], Ei[d * d], Ej[d * d];
  if (f.kind == 0) {
    const auto hx = L::between(Xi, Xj);
    const auto rel = L::between(f.measured, hx);
    L::logmap(rel, e);
    double D[d * d], Ad[d * d];
    S::logmap_derivative(e, D);
    S::adjoint(L::inverse(hx), Ad);
    matmul(D, Ad, Ei, d, d, d);
    for (int i = 0; i < d * d; ++i) {
      Ei[i] = -Ei[i];
      Ej[i] = D[i];
    }
  } else {
    L::logmap(L::between(Xi, f.measured), e);
    for (int i = 0; i < d; ++i) e[i] = -e[i];
    for (int i = 0; i < d * d; ++i) Ei[i] = (i % (d + 1) == 0) ? 1.0 : 0.0;
  }
  const double sw = std::sqrt(w);
  for (int i = 0; i < d; ++i) {
    double acc = 0.0;
    for (int k = 0; k < d; ++k) acc += f.sqrt_info[d * i + k] * e[k];
    r[i] = sw * acc;
  }
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      double ai = 0.0, aj = 0.0;
      for (int k = 0; k < d; ++k) {
        ai += f.sqrt_info[d * i + k] * Ei[d * k + j];
        if (f.kind == 0) aj += f.sqrt_info[d * i + k] * Ej[d * k + j];
      }
      Ji[d * i + j] = sw * ai;
      if (Jj) Jj[d * i + j] = sw * aj;
    }
}

template <class S>
static inline double factor_error(const Factor<typename S::L>& f, const std::map<uint64_t, typename S::Pose>& vals,
                                  double w) {
  using L = typename S::L;
  constexpr int d = S::d;
  double e[d];
  if (f.kind == 0) {
    const auto hx = L::between(vals.at(f.k1), vals.at(f.k2));
    L::logmap(L::between(f.measured, hx), e);
  } else {
    L::logmap(L::between(vals.at(f.k1), f.measured), e);
  }
  double s = 0.0;
  for (int i = 0; i < d; ++i) {
    double acc = 0.0;
    for (int k = 0; k < d; ++k) acc += f.sqrt_info[d * i + k] * e[k];
    s += acc * acc;
  }
  return 0.5 * w * s;
}

// ---------------------------------------------------------------- block sparse Cholesky
struct BlockChol {
  int N = 0, b = 0;
  std::vector<int> order, pos;             // elimination order, inverse
  std::vector<std::vector<int>> cols;      // per position k: later positions adjacent at elimination
  std::vector<std::vector<double>> L;      // per position k: [L_kk, L_{cols[k][0]},k, ...]
  std::vector<std::vector<int>> upd_slot;  // per k: for pairs (a>=c) of cols[k], slot in column cols[k][c]
  // Left-looking form of the same updates: per column j, per block slot, the
  // sources (k, a, q) in ascending k (the order in which the right-looking
  // loop over k applies them), and the columns grouped by dependency level.
  struct Upd {
    int k, a, q;
  };
  std::vector<std::vector<std::vector<Upd>>> upd_in;  // [j][slot] -> sources
  std::vector<int> lvl_ptr, lvl_cols;

  void symbolic(int n, int bs, const std::vector<std::pair<int, int>>& edges) {
    N = n;
    b = bs;
    std::vector<std::set<int>> adj(n);
    for (auto& e : edges)
      if (e.first != e.second) {
        adj[e.first].insert(e.second);
        adj[e.second].insert(e.first);
      }
    order.clear();
    pos.assign(n, -1);
    std::vector<std::vector<int>> nb_at(n);
    // minimum degree, ties to the smallest index: the first element of the
    // set ordered by (degree, index) is the vertex a scan v = 0..n-1 with a
    // strict "<" on the degree would pick
    std::set<std::pair<size_t, int>> queue;
    for (int v = 0; v < n; ++v) queue.insert({adj[v].size(), v});
    for (int step = 0; step < n; ++step) {
      const int v = queue.begin()->second;
      queue.erase(queue.begin());
      pos[v] = step;
      order.push_back(v);
      std::vector<int> nb(adj[v].begin(), adj[v].end());
      nb_at[v] = nb;
      for (int u : nb) queue.erase({adj[u].size(), u});
      for (int u : nb) adj[u].erase(v);
      for (size_t i = 0; i < nb.size(); ++i)
        for (size_t j = i + 1; j < nb.size(); ++j) {
          adj[nb[i]].insert(nb[j]);
          adj[nb[j]].insert(nb[i]);
        }
      for (int u : nb) queue.insert({adj[u].size(), u});
      adj[v].clear();
    }
    cols.assign(n, {});
    for (int v = 0; v < n; ++v) {
      std::vector<int> c;
      for (int u : nb_at[v]) c.push_back(pos[u]);
      std::sort(c.begin(), c.end());
      cols[pos[v]] = c;
    }
    upd_slot.assign(n, {});
    for (int k = 0; k < n; ++k) {
      const auto& c = cols[k];
      for (size_t a = 0; a < c.size(); ++a)
        for (size_t q = 0; q <= a; ++q) {
          // target block (row c[a], col c[q]) lives in column c[q]
          if (a == q) {
            upd_slot[k].push_back(0);
          } else {
            const auto& cc = cols[c[q]];
            const size_t s = std::lower_bound(cc.begin(), cc.end(), c[a]) - cc.begin();
            upd_slot[k].push_back((int)s + 1);
          }
        }
    }
    upd_in.assign(n, {});
    for (int j = 0; j < n; ++j) upd_in[j].assign(cols[j].size() + 1, {});
    std::vector<int> level(n, 0);
    for (int k = 0; k < n; ++k) {
      const auto& c = cols[k];
      size_t idx = 0;
      for (size_t a = 0; a < c.size(); ++a)
        for (size_t q = 0; q <= a; ++q) upd_in[c[q]][upd_slot[k][idx++]].push_back({k, (int)a, (int)q});
      for (int u : c) level[u] = std::max(level[u], level[k] + 1);
    }
    const int nl = n ? *std::max_element(level.begin(), level.end()) + 1 : 0;
    lvl_ptr.assign(nl + 1, 0);
    for (int j = 0; j < n; ++j) lvl_ptr[level[j] + 1]++;
    for (int l = 0; l < nl; ++l) lvl_ptr[l + 1] += lvl_ptr[l];
    lvl_cols.assign(n, 0);
    std::vector<int> fill(lvl_ptr.begin(), lvl_ptr.end() - 1);
    for (int j = 0; j < n; ++j) lvl_cols[fill[level[j]]++] = j;
  }
  // load H (diag blocks per variable, off-diagonal blocks per edge (i,j) meaning H_ij)
  void load(const std::vector<double>& Hd, const std::vector<std::pair<int, int>>& edges,
            const std::vector<double>& He) {
    const int bb = b * b;
    L.resize(N);  // keeps each column's storage from the previous load
    for (int k = 0; k < N; ++k) L[k].assign((size_t)bb * (cols[k].size() + 1), 0.0);
    for (int v = 0; v < N; ++v)
      for (int i = 0; i < bb; ++i) L[pos[v]][i] += Hd[(size_t)v * bb + i];
    for (size_t e = 0; e < edges.size(); ++e) {
      int i = edges[e].first, j = edges[e].second;
      if (i == j) continue;
      const double* B = &He[e * bb];
      int pi = pos[i], pj = pos[j];
      // store the lower block (row = later position) in the earlier column
      bool tr = false;
      if (pi < pj) {
        std::swap(pi, pj);
        tr = true;  // block (pos i < pos j): we need H_ji = H_ij^T at row pj... swap
      }
      // now block row pi (later), column pj (earlier) = H_{row var, col var}
      const auto& cc = cols[pj];
      const size_t s = std::lower_bound(cc.begin(), cc.end(), pi) - cc.begin();
      double* dst = &L[pj][(s + 1) * bb];
      // H_{i,j} given; if no swap, row var = i (later), col var = j: block = H_ij
      // if swapped, row var = j, col var = i: block = H_ji = H_ij^T
      for (int r = 0; r < b; ++r)
        for (int c = 0; c < b; ++c) dst[r * b + c] += tr ? B[c * b + r] : B[r * b + c];
    }
  }
  // Column j of the factor, left-looking: every block of column j first
  // takes its updates -= L(row, k) L(j, k)^T from the earlier columns k in
  // ascending k (each product summed t = 0..b-1 from 0, then subtracted),
  // which are the operations and the order of the right-looking loop (column
  // k applying its updates to all later columns after being factored); then
  // the diagonal block's Cholesky and the off-diagonal solves. Columns of one
  // dependency level do not touch each other, so they run on the OpenMP
  // threads; the factor does not depend on the thread count.
  bool factor_column(int j) {
    const int bb = b * b;
    auto& Lj = L[j];
    for (size_t s = 0; s < upd_in[j].size(); ++s) {
      double* T = &Lj[s * bb];
      for (const Upd& u : upd_in[j][s]) {
        const double* La = &L[u.k][(size_t)(u.a + 1) * bb];
        const double* Lq = &L[u.k][(size_t)(u.q + 1) * bb];
        for (int r = 0; r < b; ++r)
          for (int c = 0; c < b; ++c) {
            double acc = 0.0;
            for (int t = 0; t < b; ++t) acc += La[r * b + t] * Lq[c * b + t];
            T[r * b + c] -= acc;
          }
      }
    }
    double* D = &Lj[0];
    double Lk[36];
    // dense Cholesky of the diagonal block (lower)
    for (int i = 0; i < b; ++i)
      for (int jj = 0; jj <= i; ++jj) {
        double acc = D[i * b + jj];
        for (int q = 0; q < jj; ++q) acc -= Lk[i * b + q] * Lk[jj * b + q];
        if (i == jj) {
          if (!(acc > 0.0)) return false;
          Lk[i * b + i] = std::sqrt(acc);
        } else {
          Lk[i * b + jj] = acc / Lk[jj * b + jj];
        }
      }
    for (int i = 0; i < b; ++i)
      for (int jj = 0; jj < b; ++jj) D[i * b + jj] = (jj <= i) ? Lk[i * b + jj] : 0.0;
    // L_uj = A_uj Lj^-T  (row-wise forward substitution)
    for (size_t a = 0; a < cols[j].size(); ++a) {
      double* B = &Lj[(a + 1) * bb];
      for (int r = 0; r < b; ++r)
        for (int c = 0; c < b; ++c) {
          double acc = B[r * b + c];
          for (int q = 0; q < c; ++q) acc -= B[r * b + q] * Lk[c * b + q];
          B[r * b + c] = acc / Lk[c * b + c];
        }
    }
    return true;
  }
  bool factor() {
    bool ok = true;
    for (size_t l = 0; l + 1 < lvl_ptr.size() && ok; ++l) {
      const int c0 = lvl_ptr[l], c1 = lvl_ptr[l + 1];
      int bad = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
      for (int t = c0; t < c1; ++t)
        if (!factor_column(lvl_cols[t])) bad |= 1;
      ok = bad == 0;
    }
    return ok;
  }
  // solve (L L^T) x = rhs, rhs/x indexed by variable
  void solve(const std::vector<double>& rhs, std::vector<double>& x) const {
    const int bb = b * b;
    std::vector<double> y((size_t)N * b);
    for (int v = 0; v < N; ++v)
      for (int i = 0; i < b; ++i) y[(size_t)pos[v] * b + i] = rhs[(size_t)v * b + i];
    for (int k = 0; k < N; ++k) {
      const double* Lk = &L[k][0];
      double* yk = &y[(size_t)k * b];
      for (int i = 0; i < b; ++i) {
        double acc = yk[i];
        for (int q = 0; q < i; ++q) acc -= Lk[i * b + q] * yk[q];
        yk[i] = acc / Lk[i * b + i];
      }
      for (size_t a = 0; a < cols[k].size(); ++a) {
        const double* B = &L[k][(a + 1) * bb];
        double* yu = &y[(size_t)cols[k][a] * b];
        for (int r = 0; r < b; ++r) {
          double acc = 0.0;
          for (int c = 0; c < b; ++c) acc += B[r * b + c] * yk[c];
          yu[r] -= acc;
        }
      }
    }
    for (int k = N - 1; k >= 0; --k) {
      const double* Lk = &L[k][0];
      double* yk = &y[(size_t)k * b];
      for (size_t a = 0; a < cols[k].size(); ++a) {
        const double* B = &L[k][(a + 1) * bb];
        const double* xu = &y[(size_t)cols[k][a] * b];
        for (int c = 0; c < b; ++c) {
          double acc = 0.0;
          for (int r = 0; r < b; ++r) acc += B[r * b + c] * xu[r];
          yk[c] -= acc;
        }
      }
      for (int i = b - 1; i >= 0; --i) {
        double acc = yk[i];
        for (int q = i + 1; q < b; ++q) acc -= Lk[q * b + i] * yk[q];
        yk[i] = acc / Lk[i * b + i];
      }
    }
    x.assign((size_t)N * b, 0.0);
    for (int v = 0; v < N; ++v)
      for (int i = 0; i < b; ++i) x[(size_t)v * b + i] = y[(size_t)pos[v] * b + i];
  }
};

// ---------------------------------------------------------------- chi-square quantile
static inline double chi2_cdf(double x, int k) {
  if (x <= 0.0) return 0.0;
  const double h = 0.5 * x;
  if (k % 2 == 0) {
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < k / 2; ++i) {
      term *= h / i;
      sum += term;
    }
    return 1.0 - std::exp(-h) * sum;
  }
  double p = std::erf(std::sqrt(h));
  double term = std::sqrt(x) * std::sqrt(2.0 / kPi) * std::exp(-h);  // j = 1 term: x^{1/2}/1
  for (int j = 1; j <= (k - 1) / 2; ++j) {
    p -= term;
    term *= x / (2.0 * j + 1.0);
  }
  return p;
}
static inline double chi2inv(double alpha, int k) {
  double lo = 0.0, hi = 1.0;
  while (chi2_cdf(hi, k) < alpha) hi *= 2.0;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (chi2_cdf(mid, k) < alpha) lo = mid;
    else hi = mid;
  }
  return 0.5 * (lo + hi);
}

// ---------------------------------------------------------------- LM / GN
struct LmParamsO {
  bool gauss_newton = false;
  bool diagonal_damping = true;
  int max_iterations = 100;
  double rel_tol = 1e-5, abs_tol = 1e-5, error_tol = 0.0;
  double lambda_initial = 1e-5, lambda_factor = 10.0, lambda_upper = 1e5, lambda_lower = 0.0;
  double min_model_fidelity = 1e-3, min_diag = 1e-6, max_diag = 1e32;
};

struct SolveStats {
  int iterations = 0;
  int linear_solves = 0;
  bool failed = false;
};

// Sampling hook of the CPU timings: when >= 0, every LM / GN run stops after
// this many iterations (default -1: the solver's own limit).
inline int g_lm_max_iterations = -1;

template <class S>
struct NLS {
  using L = typename S::L;
  using Pose = typename S::Pose;
  using Values = std::map<uint64_t, Pose>;
  static constexpr int d = S::d;

  const std::vector<Factor<L>>* graph = nullptr;
  const std::vector<double>* weights = nullptr;
  std::vector<uint64_t> keys;
  std::map<uint64_t, int> index;
  std::vector<std::pair<int, int>> edges;  // variable pairs of between factors (per factor)
  std::vector<int> fi_, fj_;               // variable indices of every factor
  std::vector<int> edge_fac_;              // factor of each edge
  std::vector<int> inc_ptr_, inc_;         // per variable: its factors (factor << 1 | role), factor order
  mutable std::vector<double> lin_part_;   // per-factor linearisation pieces
  BlockChol chol;
  bool symbolic_done = false;

  double w(size_t k) const { return weights ? (*weights)[k] : 1.0; }
  // per-factor terms on the OpenMP threads, summed in factor order (the
  // same additions as a sequential loop)
  double error(const Values& v) const {
    const int64_t F = (int64_t)graph->size();
    std::vector<double> e((size_t)F);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < F; ++k) e[(size_t)k] = factor_error<S>((*graph)[(size_t)k], v, w((size_t)k));
    double s = 0.0;
    for (int64_t k = 0; k < F; ++k) s += e[(size_t)k];
    return s;
  }
  void setup(const Values& v) {
    keys.clear();
    index.clear();
    for (auto& kv : v) {
      index[kv.first] = (int)keys.size();
      keys.push_back(kv.first);
    }
    edges.clear();
    edge_fac_.clear();
    fi_.clear();
    fj_.clear();
    for (auto& f : *graph) {
      fi_.push_back(index.at(f.k1));
      fj_.push_back(f.kind == 0 ? index.at(f.k2) : fi_.back());
      if (f.kind == 0) {
        edges.push_back({fi_.back(), fj_.back()});
        edge_fac_.push_back((int)(fi_.size() - 1));
      }
    }
    // per variable: (factor << 1 | role) in factor order, role 0 = the i
    // (or prior) part, 1 = the j part
    const int nv = (int)keys.size();
    inc_ptr_.assign(nv + 1, 0);
    for (size_t k = 0; k < fi_.size(); ++k) {
      inc_ptr_[fi_[k] + 1]++;
      if ((*graph)[k].kind == 0) inc_ptr_[fj_[k] + 1]++;
    }
    for (int v = 0; v < nv; ++v) inc_ptr_[v + 1] += inc_ptr_[v];
    inc_.assign(inc_ptr_[nv], 0);
    std::vector<int> fill(inc_ptr_.begin(), inc_ptr_.end() - 1);
    for (size_t k = 0; k < fi_.size(); ++k) {
      inc_[fill[fi_[k]]++] = (int)(k << 1);
      if ((*graph)[k].kind == 0) inc_[fill[fj_[k]]++] = (int)(k << 1) | 1;
    }
    if (!symbolic_done) {
      chol.symbolic((int)keys.size(), d, edges);
      symbolic_done = true;
    }
  }
  // H (diag blocks Hd, per-between-factor blocks He), g, and 0.5|b|^2
  // Per factor (OpenMP threads): its Hessian blocks and gradient pieces;
  // then added into H and g in factor order, so every sum sees the same
  // additions in the same order as a sequential pass.
  void linearize(const Values& v, std::vector<double>& Hd, std::vector<double>& He, std::vector<double>& g) const {
    const int n = (int)keys.size();
    constexpr int dd = d * d, rec = 3 * dd + 2 * d;
    const int64_t F = (int64_t)graph->size();
    Hd.assign((size_t)n * dd, 0.0);
    He.assign(edges.size() * dd, 0.0);
    g.assign((size_t)n * d, 0.0);
    std::vector<double>& part = lin_part_;
    part.resize((size_t)F * rec);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < F; ++k) {
      const auto& f = (*graph)[(size_t)k];
      double* P = &part[(size_t)k * rec];
      double r[d], Ji[d * d], Jj[d * d];
      if (f.kind == 0) {
        linearize_factor<S>(f, v.at(f.k1), v.at(f.k2), w((size_t)k), r, Ji, Jj);
        for (int a = 0; a < d; ++a)
          for (int b = 0; b < d; ++b) {
            double hii = 0, hjj = 0, hij = 0;
            for (int q = 0; q < d; ++q) {
              hii += Ji[q * d + a] * Ji[q * d + b];
              hjj += Jj[q * d + a] * Jj[q * d + b];
              hij += Ji[q * d + a] * Jj[q * d + b];
            }
            P[a * d + b] = hii;
            P[dd + a * d + b] = hjj;
            P[2 * dd + a * d + b] = hij;
          }
        for (int a = 0; a < d; ++a) {
          double gi = 0, gj = 0;
          for (int q = 0; q < d; ++q) {
            gi += Ji[q * d + a] * r[q];
            gj += Jj[q * d + a] * r[q];
          }
          P[3 * dd + a] = gi;
          P[3 * dd + d + a] = gj;
        }
      } else {
        linearize_factor<S>(f, v.at(f.k1), v.at(f.k1), w((size_t)k), r, Ji, nullptr);
        for (int a = 0; a < d; ++a)
          for (int b = 0; b < d; ++b) {
            double h = 0;
            for (int q = 0; q < d; ++q) h += Ji[q * d + a] * Ji[q * d + b];
            P[a * d + b] = h;
          }
        for (int a = 0; a < d; ++a) {
          double gi = 0;
          for (int q = 0; q < d; ++q) gi += Ji[q * d + a] * r[q];
          P[3 * dd + a] = gi;
        }
      }
    }
    // He: one factor per edge slot; Hd and g: per variable, its factors'
    // pieces in factor order (the incidence lists ascend by factor, the i
    // part before the j part), the additions of a sequential pass
    const int64_t E = (int64_t)edges.size();
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < E; ++e) {
      const double* P = &part[(size_t)edge_fac_[(size_t)e] * rec];
      for (int t = 0; t < dd; ++t) He[(size_t)e * dd + t] += P[2 * dd + t];
    }
#pragma omp parallel for schedule(static)
    for (int v = 0; v < n; ++v) {
      double* H = &Hd[(size_t)v * dd];
      double* gv = &g[(size_t)v * d];
      for (int u = inc_ptr_[v]; u < inc_ptr_[v + 1]; ++u) {
        const int k = inc_[u] >> 1, role = inc_[u] & 1;
        const double* P = &part[(size_t)k * rec];
        for (int t = 0; t < dd; ++t) H[t] += P[role * dd + t];
        for (int a = 0; a < d; ++a) gv[a] += P[3 * dd + role * d + a];
      }
    }
  }
  // delta^T H delta computed from the blocks
  double quad(const std::vector<double>& Hd, const std::vector<double>& He, const std::vector<double>& x) const {
    double s = 0.0;
    const int n = (int)keys.size();
    for (int i = 0; i < n; ++i)
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) s += x[i * d + a] * Hd[(size_t)i * d * d + a * d + b] * x[i * d + b];
    for (size_t e = 0; e < edges.size(); ++e) {
      const int i = edges[e].first, j = edges[e].second;
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) s += 2.0 * x[i * d + a] * He[e * d * d + a * d + b] * x[j * d + b];
    }
    return s;
  }
  Values retract(const Values& v, const std::vector<double>& delta) const {
    std::vector<Pose> nv(keys.size());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)keys.size(); ++i)
      nv[(size_t)i] = L::compose(v.at(keys[(size_t)i]), S::exp(&delta[(size_t)i * d]));
    Values out;
    for (size_t i = 0; i < keys.size(); ++i) out.emplace_hint(out.end(), keys[i], nv[i]);  // keys ascend
    return out;
  }

  // GTSAM LevenbergMarquardtOptimizer / GaussNewtonOptimizer restated
  Values optimize(const Values& init, const LmParamsO& p_in, SolveStats* st) {
    LmParamsO p = p_in;
    if (g_lm_max_iterations >= 0) p.max_iterations = g_lm_max_iterations;
    setup(init);
    Values cur = init;
    double cur_err = error(cur);
    double lambda = p.lambda_initial;
    int iters = 0;
    if (cur_err <= p.error_tol || p.max_iterations <= 0) return cur;
    std::vector<double> Hd, He, g, Hdd, x, rhs;
    double new_err = cur_err;
    do {
      const double current_error = new_err;
      linearize(cur, Hd, He, g);
      const int n = (int)keys.size();
      rhs.assign((size_t)n * d, 0.0);
      for (size_t i = 0; i < rhs.size(); ++i) rhs[i] = -g[i];
      if (p.gauss_newton) {
        chol.load(Hd, edges, He);
        if (st) st->linear_solves++;
        if (!chol.factor()) {
          if (st) st->failed = true;
          return cur;
        }
        chol.solve(rhs, x);
        cur = retract(cur, x);
        cur_err = error(cur);
        ++iters;
      } else {
        std::vector<double> diag((size_t)n * d);
        for (int i = 0; i < n; ++i)
          for (int a = 0; a < d; ++a) {
            double h = Hd[(size_t)i * d * d + a * d + a];
            diag[i * d + a] = p.diagonal_damping ? std::min(std::max(h, p.min_diag), p.max_diag) : 1.0;
          }
        while (true) {
          Hdd = Hd;
          for (int i = 0; i < n; ++i)
            for (int a = 0; a < d; ++a) Hdd[(size_t)i * d * d + a * d + a] += lambda * diag[i * d + a];
          chol.load(Hdd, edges, He);
          if (st) st->linear_solves++;
          bool solved = chol.factor();
          bool success = false, stop_search = false;
          Values newv;
          double nerr = 0;
          if (solved) {
            chol.solve(rhs, x);
            double gd = 0.0;
            for (size_t i = 0; i < x.size(); ++i) gd += g[i] * x[i];
            const double old_lin = cur_err;  // 0.5|b|^2 equals the current error for Gaussian factors
            const double lin_change = -gd - 0.5 * quad(Hd, He, x);
            if (lin_change >= 0.0) {
              newv = retract(cur, x);
              nerr = error(newv);
              const double cost_change = cur_err - nerr;
              if (lin_change > std::numeric_limits<double>::epsilon() * old_lin) {
                success = (cost_change / lin_change) > p.min_model_fidelity;
              } else {
                success = true;
              }
              if (std::fabs(cost_change) < p.rel_tol * cur_err) stop_search = true;
            }
          }
          if (success) {
            cur = newv;
            cur_err = nerr;
            lambda = std::max(p.lambda_lower, lambda / p.lambda_factor);
            ++iters;
            break;
          } else if (!stop_search) {
            lambda *= p.lambda_factor;
            if (lambda >= p.lambda_upper) break;
          } else {
            break;
          }
        }
      }
      new_err = cur_err;
      const double abs_dec = current_error - new_err;
      const double rel_dec = abs_dec / current_error;
      bool converged = (new_err <= p.error_tol) || (p.rel_tol != 0.0 && rel_dec <= p.rel_tol) || (abs_dec <= p.abs_tol);
      if (iters >= p.max_iterations || converged || !std::isfinite(current_error)) break;
    } while (true);
    if (st) st->iterations += iters;
    return cur;
  }
};

// ---------------------------------------------------------------- GNC-TLS
struct GncParamsO {
  int threshold_mode = 1;  // 0 COST, 1 PROBABILITY
  double threshold = 0.9;
  int max_iterations = 100;
  double mu_step = 1.4, rel_cost_tol = 1e-5, weights_tol = 1e-4;
  bool fix_prev_inliers = false, bias_odom = false;
};

template <class S>
struct GncResult {
  std::map<uint64_t, typename S::Pose> values;
  std::vector<double> weights;
  int outer_iterations = 0;
  SolveStats stats;
};

template <class S>
GncResult<S> gnc_tls(const std::vector<Factor<typename S::L>>& graph, const std::map<uint64_t, typename S::Pose>& init,
                     size_t n_known, const GncParamsO& gp, const LmParamsO& lp,
                     const std::vector<double>* init_weights = nullptr, int max_outer_override = -1,
                     bool lm_from_previous = false) {
  GncResult<S> out;
  const size_t nf = graph.size();
  std::vector<double> barc(nf, 1.0);
  for (size_t k = 0; k < nf; ++k)
    barc[k] = (gp.threshold_mode == 0) ? gp.threshold : 0.5 * chi2inv(gp.threshold, S::d);
  std::vector<double> weights(nf, 1.0);
  if (init_weights) weights = *init_weights;
  NLS<S> nls;
  nls.graph = &graph;
  nls.weights = &weights;
  auto result = nls.optimize(init, lp, &out.stats);
  // mu initialisation from the residuals at the initial values
  double mu = std::numeric_limits<double>::infinity();
  std::vector<double> r0(nf);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)nf; ++k) r0[(size_t)k] = factor_error<S>(graph[(size_t)k], init, 1.0);
  for (size_t k = 0; k < nf; ++k) {
    const double rk = r0[k];
    if (2.0 * rk - barc[k] > 0.0) mu = std::min(mu, barc[k] / (2.0 * rk - barc[k]));
  }
  if (mu >= 0.0 && mu < 1e-6) mu = 1e-6;
  if (!(mu > 0.0) || std::isinf(mu)) mu = -1.0;
  double prev_cost = nls.error(result);
  const size_t n_unknown = nf - n_known;
  const int max_outer = max_outer_override >= 0 ? max_outer_override : gp.max_iterations;
  if (n_unknown == 0 || mu <= 0.0) {
    out.values = result;
    out.weights = weights;
    return out;
  }
  for (int it = 0; it < max_outer; ++it) {
    out.outer_iterations = it + 1;
#pragma omp parallel for schedule(static)
    for (int64_t kk = 0; kk < (int64_t)nf; ++kk) {
      const size_t k = (size_t)kk;
      if (k < n_known) {
        weights[k] = 1.0;
        continue;
      }
      const double u2 = factor_error<S>(graph[k], result, 1.0);
      const double ub = (mu + 1.0) / mu * barc[k];
      const double lb = mu / (mu + 1.0) * barc[k];
      double wk = std::sqrt(barc[k] * mu * (mu + 1.0) / u2) - mu;
      if (u2 >= ub || wk < 0.0) wk = 0.0;
      else if (u2 <= lb || wk > 1.0) wk = 1.0;
      weights[k] = wk;
    }
    result = nls.optimize(lm_from_previous ? result : init, lp, &out.stats);
    const double cost = nls.error(result);
    bool conv = std::fabs(cost - prev_cost) / std::max(prev_cost, 1e-7) < gp.rel_cost_tol;
    if (!conv) {
      conv = true;
      for (size_t k = 0; k < nf; ++k)
        if (std::fabs(weights[k] - std::round(weights[k])) > gp.weights_tol) {
          conv = false;
          break;
        }
    }
    if (conv) break;
    mu *= gp.mu_step;
    prev_cost = cost;
  }
  out.values = result;
  out.weights = weights;
  return out;
}

// Warm-started GNC-TLS schedule (no counterpart in the reference; the
// library's GNC warm start restated for parity). probs[k] is a predicted
// inlier probability for every factor k >= n_known. Steps:
//  1. weights: known factors 1, others 1 when probs[k] >= 0.5 else 0;
//     LM from the initial values with those weights;
//  2. TLS weight update at mu (first mu = warm_mu, which skips the
//     continuation from mu ~ 0); when the new weights are binary within
//     weights_tol and equal to the weights of the last solve, the estimate is
//     a fixed point of the TLS rule and the schedule ends; otherwise LM from
//     the previous estimate with the new weights, mu *= mu_step, repeat (at
//     most max_iterations updates);
//  3. a fixed point reached from a start that admitted outliers can be a poor
//     local minimum of the TLS cost, in which most of the predicted inliers
//     end up rejected; the result is therefore certified only when at least
//     kWarmKeep of the predicted inliers are inliers at the fixed point.
// certified = false (no fixed point within max_iterations, or the prediction
// contradicted) sends the caller back to the plain schedule.
constexpr double kWarmKeep = 0.75;

template <class S>
GncResult<S> gnc_tls_warm(const std::vector<Factor<typename S::L>>& graph,
                          const std::map<uint64_t, typename S::Pose>& init, size_t n_known, const GncParamsO& gp,
                          const LmParamsO& lp, const std::vector<double>& probs, double warm_mu, bool* certified) {
  GncResult<S> out;
  const size_t nf = graph.size();
  std::vector<double> barc(nf, 1.0);
  for (size_t k = 0; k < nf; ++k)
    barc[k] = (gp.threshold_mode == 0) ? gp.threshold : 0.5 * chi2inv(gp.threshold, S::d);
  std::vector<double> weights(nf, 1.0);
  size_t predicted = 0;
  for (size_t k = n_known; k < nf; ++k) {
    weights[k] = (k < probs.size() && probs[k] >= 0.5) ? 1.0 : 0.0;
    predicted += weights[k] == 1.0;
  }
  const std::vector<double> first = weights;
  NLS<S> nls;
  nls.graph = &graph;
  nls.weights = &weights;
  auto result = nls.optimize(init, lp, &out.stats);
  double mu = warm_mu;
  bool fixed_point = nf == n_known;
  std::vector<double> wnew(nf, 1.0);
  for (int it = 0; it < gp.max_iterations && !fixed_point; ++it) {
    out.outer_iterations = it + 1;
    bool same = true;
    for (size_t k = n_known; k < nf; ++k) {
      const double u2 = factor_error<S>(graph[k], result, 1.0);
      const double ub = (mu + 1.0) / mu * barc[k];
      const double lb = mu / (mu + 1.0) * barc[k];
      double wk = std::sqrt(barc[k] * mu * (mu + 1.0) / u2) - mu;
      if (u2 >= ub || wk < 0.0) wk = 0.0;
      else if (u2 <= lb || wk > 1.0) wk = 1.0;
      wnew[k] = wk;
      if (std::fabs(wk - std::round(wk)) > gp.weights_tol || std::round(wk) != weights[k]) same = false;
    }
    if (same) {
      fixed_point = true;
      break;
    }
    for (size_t k = n_known; k < nf; ++k) weights[k] = wnew[k];
    result = nls.optimize(result, lp, &out.stats);
    mu *= gp.mu_step;
  }
  size_t kept = 0;
  for (size_t k = n_known; k < nf; ++k) kept += (first[k] == 1.0 && weights[k] == 1.0);
  *certified = fixed_point && (double)kept >= kWarmKeep * (double)predicted;
  out.values = result;
  out.weights = weights;
  return out;
}

}  // namespace oracle

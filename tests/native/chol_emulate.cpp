// Sequential CPU emulation of the direct solve's phases (the GPU kernel
// k_chol_solve in kimera-rpgo_gb300/csrc/chol_kernels.cu), driven by the same
// symbolic plan (make_chol_plan). Test infrastructure only: it checks the
// plan (elimination order, block structure, update lists, Hessian gathers,
// levels, the dense-tail tiling) and the phase order against a dense solve.
// Items of one phase are independent, so running them one after another
// gives what the GPU computes, up to the order of floating-point sums.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "chol_plan.hpp"

using rpgo::CholPlan;

namespace {

struct Emu {
  const CholPlan& p;
  int d, dd, ntp;
  const double *Hd, *fH, *damp;
  double lam;
  const double* lam_v = nullptr;  // per-variable damping (joint batch), else lam
  std::vector<double> L, Ldiag, M, Ldd, y;
  int fail = 0;
  Emu(const CholPlan& pl) : p(pl), d(pl.d), dd(pl.d * pl.d), ntp(pl.n_tiles * pl.tile) {}
  double& m(int r, int c) { return M[(size_t)c * ntp + r]; }

  double diag_entry(int v, int r, int c) {
    double s = Hd[(size_t)v * dd + r * d + c];
    if (r == c) s += (lam_v ? lam_v[v] : lam) * damp[(size_t)v * d + r];
    return s;
  }
  double offdiag_entry(const std::vector<int32_t>& src, int beg, int end, int r, int c) {
    double s = 0.0;
    for (int u = beg; u < end; ++u) {
      const int32_t x = src[u];
      const double* H = fH + (size_t)(x >> 1) * dd;
      s += (x & 1) ? H[c * d + r] : H[r * d + c];
    }
    return s;
  }
  double pairs(const std::vector<int32_t>& src, int beg, int end, int r, int c, double s) {
    for (int u = beg; u < end; ++u) {
      const double* A = &L[(size_t)src[2 * u] * dd + r * d];
      const double* B = &L[(size_t)src[2 * u + 1] * dd + c * d];
      double acc = 0.0;
      for (int t = 0; t < d; ++t) acc += A[t] * B[t];
      s -= acc;
    }
    return s;
  }
  void chol_small(std::vector<double>& C) {
    for (int c = 0; c < d; ++c) {
      double s = C[c * d + c];
      for (int t = 0; t < c; ++t) s -= C[c * d + t] * C[c * d + t];
      if (!(s > 0.0)) {
        fail = 1;
        s = 1.0;
      }
      const double l = std::sqrt(s);
      C[c * d + c] = l;
      for (int r = c + 1; r < d; ++r) {
        double v = C[r * d + c];
        for (int t = 0; t < c; ++t) v -= C[r * d + t] * C[c * d + t];
        C[r * d + c] = v / l;
      }
    }
  }
  std::vector<double> Spart;  // task partial sums
  void run_task(int t) {
    const int* tk = &p.tasks[4 * (size_t)t];
    const int kind = tk[3] & 3, slot = tk[3] >> 4;
    if (kind < 2) {
      const int q = tk[0], j = p.blk_col[q], i = p.blk_row[q];
      const int nc = d == 6 ? 3 : d, c0 = ((tk[3] >> 2) & 1) * nc;
      for (int r = 0; r < d; ++r)
        for (int c = c0; c < c0 + nc; ++c) {
          double s = 0.0;
          if (kind == 1)
            s = i == j ? diag_entry(p.perm[j], r, c) : offdiag_entry(p.a_src, p.a_ptr[q], p.a_ptr[q + 1], r, c);
          Spart[(size_t)slot * dd + r * d + c] = pairs(p.upd_src, tk[1], tk[2], r, c, s);
        }
    } else {
      for (int r = 0; r < d; ++r) {
        double b = 0.0;
        for (int u = tk[1]; u < tk[2]; ++u) {
          const int q = p.row_blk[2 * u], k = p.row_blk[2 * u + 1];
          for (int c = 0; c < d; ++c) b += L[(size_t)q * dd + r * d + c] * y[(size_t)k * d + c];
        }
        Spart[(size_t)slot * dd + r * d] = b;
      }
    }
  }
  void sparse_S(int q) {
    const int j = p.blk_col[q], i = p.blk_row[q];
    for (int e = 0; e < dd; ++e) {
      double s = 0.0;
      if (p.btask[2 * q + 1] == 0)  // no update pairs, no task: the Hessian block itself
        s = i == j ? diag_entry(p.perm[j], e / d, e % d) : offdiag_entry(p.a_src, p.a_ptr[q], p.a_ptr[q + 1], e / d, e % d);
      for (int t = p.btask[2 * q]; t < p.btask[2 * q] + p.btask[2 * q + 1]; ++t) s += Spart[(size_t)t * dd + e];
      L[(size_t)q * dd + e] = s;
    }
  }
  void sparse_scale(int q) {
    const int j = p.blk_col[q], i = p.blk_row[q];
    std::vector<double> C(L.begin() + (size_t)p.col_ptr[j] * dd, L.begin() + (size_t)(p.col_ptr[j] + 1) * dd);
    chol_small(C);
    if (i == j) {
      for (int e = 0; e < dd; ++e) Ldiag[(size_t)j * dd + e] = (e / d >= e % d) ? C[e] : 0.0;
      return;
    }
    for (int r = 0; r < d; ++r) {
      std::vector<double> x(d);
      for (int c = 0; c < d; ++c) {
        double v = L[(size_t)q * dd + r * d + c];
        for (int t = 0; t < c; ++t) v -= x[t] * C[c * d + t];
        x[c] = v / C[c * d + c];
      }
      for (int c = 0; c < d; ++c) L[(size_t)q * dd + r * d + c] = x[c];
    }
  }
  void sparse_forward(int j) {
    std::vector<double> b(d);
    for (int r = 0; r < d; ++r) {
      b[r] = y[(size_t)j * d + r];
      for (int t = p.ftask[2 * j]; t < p.ftask[2 * j] + p.ftask[2 * j + 1]; ++t) b[r] -= Spart[(size_t)t * dd + r * d];
    }
    const double* Lj = &Ldiag[(size_t)j * dd];
    for (int c = 0; c < d; ++c) {
      const double yc = b[c] / Lj[c * d + c];
      y[(size_t)j * d + c] = yc;
      for (int r = c + 1; r < d; ++r) b[r] -= Lj[r * d + c] * yc;
    }
  }
  void sparse_backward(int j) {
    std::vector<double> b(d);
    for (int r = 0; r < d; ++r) {
      b[r] = y[(size_t)j * d + r];
      for (int q = p.col_ptr[j] + 1; q < p.col_ptr[j + 1]; ++q)
        for (int c = 0; c < d; ++c) b[r] -= L[(size_t)q * dd + c * d + r] * y[(size_t)p.blk_row[q] * d + c];
    }
    const double* Lj = &Ldiag[(size_t)j * dd];
    for (int c = d - 1; c >= 0; --c) {
      const double xc = b[c] / Lj[c * d + c];
      y[(size_t)j * d + c] = xc;
      for (int r = 0; r < c; ++r) b[r] -= Lj[c * d + r] * xc;
    }
  }
  static void tail_coords(int t, int& bi, int& bj) {
    int i = (int)((std::sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while (i * (i + 1) / 2 > t) --i;
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    bi = i;
    bj = t - i * (i + 1) / 2;
  }
  void tail_S(int t) {
    int bi, bj;
    tail_coords(t, bi, bj);
    for (int e = 0; e < dd; ++e) {
      const int r = e / d, c = e % d;
      double s = bi == bj ? diag_entry(p.perm[p.n_sparse + bi], r, c)
                          : offdiag_entry(p.ta_src, p.ta_ptr[t], p.ta_ptr[t + 1], r, c);
      m(bi * d + r, bj * d + c) = pairs(p.tupd_src, p.tupd_ptr[t], p.tupd_ptr[t + 1], r, c, s);
    }
  }
  void tail_rhs(int t) {
    for (int r = 0; r < d; ++r) {
      double b = 0.0;
      for (int w = p.ttask_ptr[t]; w < p.ttask_ptr[t + 1]; ++w)
      for (int u = p.ttasks[3 * w + 1]; u < p.ttasks[3 * w + 2]; ++u) {
        const int q = p.trow_blk[2 * u], k = p.trow_blk[2 * u + 1];
        for (int c = 0; c < d; ++c) b += L[(size_t)q * dd + r * d + c] * y[(size_t)k * d + c];
      }
      y[(size_t)(p.n_sparse + t) * d + r] -= b;
    }
  }
  // tile helpers (TB = plan.tile)
  void load(int ti, int tj, std::vector<double>& S) {
    const int TB = p.tile;
    S.assign((size_t)TB * TB, 0.0);
    for (int r = 0; r < TB; ++r)
      for (int c = 0; c < TB; ++c) S[r * TB + c] = m(ti * TB + r, tj * TB + c);
  }
  void column_item(int i, int k) {
    const int TB = p.tile;
    std::vector<double> C, B, A, E;
    load(k, k, C);
    if (k > 0) load(k, k - 1, B);
    if (i > k) {
      load(i, k, A);
      if (k > 0) load(i, k - 1, E);
    }
    if (k > 0) {
      for (int r = 0; r < TB; ++r)
        for (int c = 0; c <= r; ++c) {
          double acc = 0.0;
          for (int t = 0; t < TB; ++t) acc += B[r * TB + t] * B[c * TB + t];
          C[r * TB + c] -= acc;
        }
      if (i > k)
        for (int r = 0; r < TB; ++r)
          for (int c = 0; c < TB; ++c) {
            double acc = 0.0;
            for (int t = 0; t < TB; ++t) acc += E[r * TB + t] * B[c * TB + t];
            A[r * TB + c] -= acc;
          }
    }
    for (int c = 0; c < TB; ++c) {
      double piv = C[c * TB + c];
      if (!(piv > 0.0)) {
        fail = 1;
        piv = 1.0;
      }
      C[c * TB + c] = std::sqrt(piv);
      for (int r = c + 1; r < TB; ++r) C[r * TB + c] /= C[c * TB + c];
      for (int q = c + 1; q < TB; ++q)
        for (int r = q; r < TB; ++r) C[r * TB + q] -= C[r * TB + c] * C[q * TB + c];
    }
    if (i == k) {
      for (int r = 0; r < TB; ++r)
        for (int c = 0; c < TB; ++c) Ldd[(size_t)k * TB * TB + r * TB + c] = c <= r ? C[r * TB + c] : 0.0;
    } else {
      for (int r = 0; r < TB; ++r)
        for (int c = 0; c < TB; ++c) {
          double v = A[r * TB + c];
          for (int t = 0; t < c; ++t) v -= A[r * TB + t] * C[c * TB + t];
          A[r * TB + c] = v / C[c * TB + c];
        }
      for (int r = 0; r < TB; ++r)
        for (int c = 0; c < TB; ++c) m(i * TB + r, k * TB + c) = A[r * TB + c];
    }
  }
  void trailing_item(int i, int j, int k) {
    const int TB = p.tile;
    std::vector<double> A, B;
    load(i, k - 1, A);
    load(j, k - 1, B);
    for (int r = 0; r < TB; ++r)
      for (int c = 0; c < TB; ++c) {
        if (i == j && c > r) continue;
        double acc = 0.0;
        for (int t = 0; t < TB; ++t) acc += A[r * TB + t] * B[c * TB + t];
        m(i * TB + r, j * TB + c) -= acc;
      }
  }
  void forward_item(double* yt, int k) {
    const int TB = p.tile;
    std::vector<double> b(TB);
    for (int r = 0; r < TB; ++r) {
      b[r] = yt[k * TB + r];
      for (int c = 0; c < k * TB; ++c) b[r] -= m(k * TB + r, c) * yt[c];
    }
    const double* Lk = &Ldd[(size_t)k * TB * TB];
    for (int c = 0; c < TB; ++c) {
      const double yc = b[c] / Lk[c * TB + c];
      yt[k * TB + c] = yc;
      for (int r = c + 1; r < TB; ++r) b[r] -= Lk[r * TB + c] * yc;
    }
  }
  void backward_item(double* yt, int k) {
    const int TB = p.tile;
    std::vector<double> b(TB);
    for (int c = 0; c < TB; ++c) {
      b[c] = yt[k * TB + c];
      for (int r = (k + 1) * TB; r < ntp; ++r) b[c] -= m(r, k * TB + c) * yt[r];
    }
    const double* Lk = &Ldd[(size_t)k * TB * TB];
    for (int c = TB - 1; c >= 0; --c) {
      const double xc = b[c] / Lk[c * TB + c];
      yt[k * TB + c] = xc;
      for (int r = 0; r < c; ++r) b[r] -= Lk[c * TB + r] * xc;
    }
  }
};

}  // namespace

namespace {

int emulate(const CholPlan& p, int N, int d, const double* Hd, const double* fH, const double* rhs, double lam,
            const double* lam_v, const double* damp, double* x_out, int32_t* info) {
  Emu e(p);
  e.Hd = Hd;
  e.fH = fH;
  e.damp = damp;
  e.lam = lam;
  e.lam_v = lam_v;
  const int dd = d * d, ns = p.n_sparse, nt = p.T * d, ntp = e.ntp, TB = p.tile;
  e.L.assign((size_t)p.n_blocks() * dd, 0.0);
  e.Ldiag.assign((size_t)ns * dd, 0.0);
  e.M.assign((size_t)ntp * ntp, std::nan(""));
  e.Ldd.assign((size_t)p.n_tiles * TB * TB, 0.0);
  e.y.assign((size_t)ns * d + ntp, 0.0);
  // 1. init
  for (int q = 0; q < N * d; ++q) e.y[q] = rhs[(size_t)p.perm[q / d] * d + q % d];
  for (int c = nt; c < ntp; ++c)
    for (int r = 0; r < ntp; ++r) {
      e.m(r, c) = (r == c) ? 1.0 : 0.0;
      if (r < nt) e.m(c, r) = 0.0;
    }
  // 2. sparse levels
  const int levels = p.levels();
  e.Spart.assign((size_t)p.n_slots * dd, 0.0);
  for (int l = 0; l < levels; ++l) {
    // (A) the level's update tasks, (B) its columns
    for (int t = p.lvl_task_ptr[l]; t < p.lvl_task_ptr[l + 1]; ++t) e.run_task(t);
    for (int w = p.lvl_col_ptr[l]; w < p.lvl_col_ptr[l + 1]; ++w) {
      // one column: S of its blocks, L_jj and L_ij, its forward substitution
      const int j = p.lvl_cols[w];
      for (int q = p.col_ptr[j]; q < p.col_ptr[j + 1]; ++q) e.sparse_S(q);
      for (int q = p.col_ptr[j]; q < p.col_ptr[j + 1]; ++q) e.sparse_scale(q);
      e.sparse_forward(j);
    }
  }
  // 3. tail
  for (int t = 0; t < p.n_tail_blocks(); ++t) e.tail_S(t);
  double* yt = e.y.data() + (size_t)ns * d;
  const int nT = p.n_tiles;
  for (int kk = 0; kk <= nT; ++kk) {
    for (int i = kk; i < nT; ++i) e.column_item(i, kk);
    const int mm = nT - kk - 1;
    if (kk >= 1 && mm > 0)
      for (int u = 0; u < mm * (mm + 1) / 2; ++u) {
        int ii, jj;
        Emu::tail_coords(u, ii, jj);
        e.trailing_item(kk + 1 + ii, kk + 1 + jj, kk);
      }
    if (kk >= 1) e.forward_item(yt, kk - 1);
    if (kk == 0)
      for (int t = 0; t < p.T; ++t) e.tail_rhs(t);
  }
  // 4. backward
  for (int kk = nT - 1; kk >= 0; --kk) e.backward_item(yt, kk);
  for (int l = levels - 1; l >= 0; --l)
    for (int w = p.lvl_col_ptr[l]; w < p.lvl_col_ptr[l + 1]; ++w) e.sparse_backward(p.lvl_cols[w]);
  for (int q = 0; q < N * d; ++q) x_out[(size_t)p.perm[q / d] * d + q % d] = e.y[q];
  info[0] = ns;
  info[1] = p.T;
  info[2] = levels;
  info[3] = nT;
  info[4] = e.fail;
  return 0;
}

}  // namespace

extern "C" int chol_emulate(int N, int d, int F, const int32_t* kind, const int32_t* vi, const int32_t* vj,
                            const double* Hd, const double* fH, const double* rhs, double lam, const double* damp,
                            double* x_out, int32_t* info) {
  std::vector<int32_t> k(kind, kind + F), a(vi, vi + F), b(vj, vj + F);
  CholPlan p = rpgo::make_chol_plan(N, d, k, a, b);
  return emulate(p, N, d, Hd, fH, rhs, lam, nullptr, damp, x_out, info);
}

// The joint batch's plan: G independent systems (system g: Ns[g] variables
// and Fs[g] factors, contiguous in the union arrays, indices global), each
// planned without a dense tail and merged; system g damped by lam_g[g].
extern "C" int chol_emulate_joint(int G, const int32_t* Ns, const int32_t* Fs, int d, const int32_t* kind,
                                  const int32_t* vi, const int32_t* vj, const double* Hd, const double* fH,
                                  const double* rhs, const double* lam_g, const double* damp, double* x_out,
                                  int32_t* info) {
  std::vector<CholPlan> plans(G);
  std::vector<int32_t> foff(G + 1, 0);
  std::vector<double> lam_v;
  int v0 = 0;
  for (int g = 0; g < G; ++g) {
    const int f0 = foff[g];
    foff[g + 1] = f0 + Fs[g];
    std::vector<int32_t> k(kind + f0, kind + f0 + Fs[g]), a(Fs[g]), b(Fs[g]);
    for (int f = 0; f < Fs[g]; ++f) {
      a[f] = vi[f0 + f] - v0;
      b[f] = vj[f0 + f] - v0;
    }
    plans[g] = rpgo::make_chol_plan(Ns[g], d, k, a, b, false);
    lam_v.insert(lam_v.end(), Ns[g], lam_g[g]);
    v0 += Ns[g];
  }
  CholPlan p = rpgo::merge_chol_plans(plans, foff);
  return emulate(p, v0, d, Hd, fH, rhs, 0.0, lam_v.data(), damp, x_out, info);
}

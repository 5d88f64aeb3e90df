// CPU FP64 oracle — TEST INFRASTRUCTURE ONLY.
//
// Restatement of Kimera-RPGO's PCM outlier rejection:
//   include/KimeraRPGO/outlier/Pcm.h:148-281   removeOutliers (classification)
//   include/KimeraRPGO/outlier/Pcm.h:414-502   parseAndIncrementAdjMatrix
//   include/KimeraRPGO/outlier/Pcm.h:516-557   updateOdom
//   include/KimeraRPGO/outlier/Pcm.h:564-629   odometry consistency check
//   include/KimeraRPGO/outlier/Pcm.h:638-718   pairwise loop consistency check
//   include/KimeraRPGO/outlier/Pcm.h:725-768   incrementAdjMatrix
//   include/KimeraRPGO/outlier/Pcm.h:851-1005  findInliers[Incremental], buildGraphToOptimize
//   include/KimeraRPGO/utils/GraphUtils.h:37-58 Trajectory::getBetween
//   include/KimeraRPGO/max_clique_finder/graphIO.cpp:188-257 dense -> CSR
//   include/KimeraRPGO/max_clique_finder/findCliqueHeu.cpp:32-209 greedy clique
//   src/utils/GraphUtils.cpp:19-44 findMaxCliqueHeu[Incremental]
// Landmarks (special symbols), multi-robot frame alignment and the edit API
// (remove / ignore / revive) are outside the restated path.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <unordered_map>
#include <vector>

#include "oracle_math.hpp"

namespace oracle {

// ---------------------------------------------------------------- Lie traits
struct Lie3 {
  using Pose = P3;
  static constexpr int dim = 6, rdim = 3, tdim = 3, stride = 12;
  static Pose identity() { return p3_identity(); }
  static Pose compose(const Pose& a, const Pose& b) { return p3_compose(a, b); }
  static Pose inverse(const Pose& a) { return p3_inverse(a); }
  static Pose between(const Pose& a, const Pose& b) { return p3_between(a, b); }
  static void congruence(const Pose& T, const double* S, double* C) { p3_congruence(T, S, C); }
  static void logmap(const Pose& T, double* xi) { p3_logmap(T, xi); }
  static double rot_trace(const double* cov) { return (cov[0] + cov[7]) + cov[14]; }
  static Pose load(const double* p) {
    Pose q;
    for (int i = 0; i < 9; ++i) q.R[i] = p[i];
    for (int i = 0; i < 3; ++i) q.t[i] = p[9 + i];
    return q;
  }
  static void store(const Pose& q, double* p) {
    for (int i = 0; i < 9; ++i) p[i] = q.R[i];
    for (int i = 0; i < 3; ++i) p[9 + i] = q.t[i];
  }
};
struct Lie2 {
  using Pose = P2;
  static constexpr int dim = 3, rdim = 1, tdim = 2, stride = 4;
  static Pose identity() { return p2_identity(); }
  static Pose compose(const Pose& a, const Pose& b) { return p2_compose(a, b); }
  static Pose inverse(const Pose& a) { return p2_inverse(a); }
  static Pose between(const Pose& a, const Pose& b) { return p2_between(a, b); }
  static void congruence(const Pose& T, const double* S, double* C) { p2_congruence(T, S, C); }
  static void logmap(const Pose& T, double* xi) { p2_logmap(T, xi); }
  static double rot_trace(const double* cov) { return cov[0]; }
  static Pose load(const double* p) { return P2{p[0], p[1], p[2], p[3]}; }
  static void store(const Pose& q, double* p) {
    p[0] = q.c; p[1] = q.s; p[2] = q.x; p[3] = q.y;
  }
};

// ---------------------------------------------------------------- PoseWithCovariance
template <class L>
struct PWC {
  typename L::Pose pose = L::identity();
  double cov[L::dim * L::dim] = {0};
  bool rot_info = true;

  // GeometryUtils.h:91-115
  static PWC from_factor(const typename L::Pose& measured, const double* covariance) {
    PWC out;
    out.pose = measured;
    constexpr int n = L::dim;
    for (int i = 0; i < n * n; ++i) out.cov[i] = covariance[i];
    out.rot_info = true;
    if (std::isnan(L::rot_trace(covariance))) {
      out.rot_info = false;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          out.cov[n * i + j] = (i >= L::rdim && j >= L::rdim) ? covariance[n * i + j] : 0.0;
    }
    return out;
  }
  // GeometryUtils.h:119-129
  PWC compose(const PWC& other) const {
    PWC out;
    constexpr int n = L::dim;
    out.pose = L::compose(pose, other.pose);
    double C[n * n];
    L::congruence(L::inverse(other.pose), cov, C);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j <= i; ++j) {
        const double v = C[n * i + j] + other.cov[n * i + j];
        out.cov[n * i + j] = v;
        out.cov[n * j + i] = v;
      }
    out.rot_info = rot_info && other.rot_info;
    return out;
  }
  // GeometryUtils.h:133-139 (the covariance is deliberately not transformed)
  PWC inverse() const {
    PWC out;
    out.pose = L::inverse(pose);
    for (int i = 0; i < L::dim * L::dim; ++i) out.cov[i] = cov[i];
    out.rot_info = rot_info;
    return out;
  }
  // GeometryUtils.h:143-170
  PWC between(const PWC& other) const {
    PWC out;
    constexpr int n = L::dim;
    const typename L::Pose res = L::between(pose, other.pose);
    out.pose = res;
    double C[n * n];
    L::congruence(L::inverse(res), cov, C);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j <= i; ++j) {
        const double v = other.cov[n * i + j] - C[n * i + j];
        out.cov[n * i + j] = v;
        out.cov[n * j + i] = v;
      }
    if (!llt_ok(out.cov, n)) {
      const typename L::Pose res2 = L::between(other.pose, pose);
      L::congruence(L::inverse(res2), other.cov, C);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j) {
          const double v = cov[n * i + j] - C[n * i + j];
          out.cov[n * i + j] = v;
          out.cov[n * j + i] = v;
        }
    }
    out.rot_info = rot_info && other.rot_info;
    return out;
  }
  // GeometryUtils.h:172-186
  double mahalanobis_norm() const {
    constexpr int n = L::dim;
    double xi[n];
    L::logmap(pose, xi);
    if (!rot_info) {
      constexpr int m = L::tdim, r = L::rdim;
      double B[m * m];
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) B[m * i + j] = cov[n * (r + i) + (r + j)];
      return std::sqrt(quad_inv(B, m, xi + r));
    }
    return std::sqrt(quad_inv(cov, n, xi));
  }
};

// ---------------------------------------------------------------- PoseWithNode
template <class L>
struct PWN {
  typename L::Pose pose = L::identity();
  int node = 0;
  bool rot_info = true;

  // GeometryUtils.h:221-234
  static PWN from_factor(const typename L::Pose& measured, const double* covariance) {
    PWN out;
    out.pose = measured;
    out.rot_info = !std::isnan(L::rot_trace(covariance));
    out.node = 1;
    return out;
  }
  PWN compose(const PWN& other) const {
    PWN out;
    out.pose = L::compose(pose, other.pose);
    out.node = node + other.node;
    out.rot_info = rot_info && other.rot_info;
    return out;
  }
  PWN inverse() const {
    PWN out;
    out.pose = L::inverse(pose);
    out.node = node;
    out.rot_info = rot_info;
    return out;
  }
  PWN between(const PWN& other) const {
    PWN out;
    out.pose = L::between(pose, other.pose);
    out.node = std::abs(other.node - node);
    out.rot_info = rot_info && other.rot_info;
    return out;
  }
  static double norm_slice(const double* v, int m) {
    double acc = v[0] * v[0];
    for (int i = 1; i < m; ++i) acc = fmad(v[i], v[i], acc);
    return std::sqrt(acc);
  }
  // GeometryUtils.h:274-288 (Pose2: tail(2) is (v_y, omega), head(1) is v_x)
  double avg_trans_norm() const {
    double xi[L::dim];
    L::logmap(pose, xi);
    return norm_slice(xi + L::rdim, L::tdim) / static_cast<double>(node);
  }
  double avg_rot_norm() const {
    if (!rot_info) return 0.0;
    double xi[L::dim];
    L::logmap(pose, xi);
    return norm_slice(xi, L::rdim) / static_cast<double>(node);
  }
};

static inline char key_chr(uint64_t k) { return static_cast<char>(static_cast<unsigned char>(k >> 56)); }
static inline uint64_t symbol(char c, uint64_t idx) {
  return (static_cast<uint64_t>(static_cast<unsigned char>(c)) << 56) | idx;
}

// ---------------------------------------------------------------- Trajectory
template <class U>
struct Trajectory {
  std::map<uint64_t, U> poses;
  // GraphUtils.h:37-58 (std::map::operator[] inserts a default entry)
  U getBetween(uint64_t ka, uint64_t kb) {
    if (key_chr(ka) == key_chr(kb)) return poses[ka].between(poses[kb]);
    const uint64_t a0 = symbol(key_chr(ka), 0), b0 = symbol(key_chr(kb), 0);
    U pa = poses[a0].between(poses[ka]);
    U pb = poses[b0].between(poses[kb]);
    U pab = poses[a0].between(poses[b0]);
    U r = pa.inverse().compose(pab);
    return r.compose(pb);
  }
};

// ---------------------------------------------------------------- max clique (FMC heuristic)
// CSR exactly as CGraphIO::ReadEigenAdjacencyMatrix builds it: neighbour
// lists in ascending order, diagonal ignored.
struct Csr {
  std::vector<int> off, adj;
  int max_deg = -1;
};
static inline Csr csr_from_bits(const std::vector<uint32_t>& bits, int n, int words) {
  Csr g;
  g.off.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    // set bits of row i in ascending column order (columns >= n ignored)
    for (int w = 0; w < words && 32 * w < n; ++w) {
      uint32_t x = bits[(size_t)i * words + w];
      while (x) {
        const int j = 32 * w + __builtin_ctz(x);
        x &= x - 1u;
        if (j < n && j != i) g.adj.push_back(j);
      }
    }
    g.off[i + 1] = (int)g.adj.size();
  }
  for (int i = 0; i < n; ++i) g.max_deg = std::max(g.max_deg, g.off[i + 1] - g.off[i]);
  return g;
}

// findCliqueHeu.cpp:32-117 and 119-209: candidates first..n-1, running best
// seeded with max_clq; the winning work buffer is returned whole, so its
// first max_clq slots may hold stale (non-clique) vertices. This is the
// reference's loop structure, including its linear search of S[a] in the
// neighbour list of m (the cost the CPU baseline times).
static inline int fmc_heuristic_scan(const Csr& g, int first, int max_clq, std::vector<int>* best) {
  const int n = (int)g.off.size() - 1;
  auto deg = [&](int v) { return g.off[v + 1] - g.off[v]; };
  std::vector<int> S(std::max(g.max_deg, 0) + 1, 0), S1(std::max(g.max_deg, 0) + 1, 0);
  for (int v = first; v < n; ++v) {
    if (max_clq > deg(v)) continue;
    int npos = 0;
    S[npos++] = v;
    for (int e = g.off[v]; e < g.off[v + 1]; ++e)
      if (max_clq <= deg(g.adj[e])) S[npos++] = g.adj[e];
    int icc = 0;
    while (npos > 0) {
      ++icc;
      const int m = S[npos - 1];
      int n1 = 0;
      for (int a = 0; a < npos; ++a) {
        for (int e = g.off[m]; e < g.off[m + 1]; ++e) {
          if (S[a] == g.adj[e] && max_clq <= deg(g.adj[e])) {
            S1[n1++] = S[a];
            break;
          }
        }
      }
      for (int a = 0; a < n1; ++a) S[a] = S1[a];
      npos = n1;
    }
    if (max_clq < icc) {
      *best = S;
      max_clq = icc;
    }
  }
  return max_clq;
}

// The same heuristic with the linear search replaced by a membership stamp:
// before each round, every neighbour u of m gets stamp[u] = round id, so
// "S[a] occurs in N(m)" is one lookup. The scan's `break` on the first match
// only ends the search, so the kept elements, their order, the round count
// and every write to S are those of fmc_heuristic_scan: O(|S| + deg(m)) per
// round instead of O(|S| deg(m)).
static inline int fmc_heuristic_marked(const Csr& g, int first, int max_clq, std::vector<int>* best) {
  const int n = (int)g.off.size() - 1;
  auto deg = [&](int v) { return g.off[v + 1] - g.off[v]; };
  std::vector<int> S(std::max(g.max_deg, 0) + 1, 0), S1(std::max(g.max_deg, 0) + 1, 0);
  std::vector<int64_t> stamp(std::max(n, 1), -1);
  int64_t round_id = 0;
  for (int v = first; v < n; ++v) {
    if (max_clq > deg(v)) continue;
    int npos = 0;
    S[npos++] = v;
    for (int e = g.off[v]; e < g.off[v + 1]; ++e)
      if (max_clq <= deg(g.adj[e])) S[npos++] = g.adj[e];
    int icc = 0;
    while (npos > 0) {
      ++icc;
      const int m = S[npos - 1];
      ++round_id;
      for (int e = g.off[m]; e < g.off[m + 1]; ++e) stamp[g.adj[e]] = round_id;
      int n1 = 0;
      for (int a = 0; a < npos; ++a)
        if (stamp[S[a]] == round_id && max_clq <= deg(S[a])) S1[n1++] = S[a];
      for (int a = 0; a < n1; ++a) S[a] = S1[a];
      npos = n1;
    }
    if (max_clq < icc) {
      *best = S;
      max_clq = icc;
    }
  }
  return max_clq;
}

// Inner-loop iterations the reference's linear search (fmc_heuristic_scan)
// performs on g: per round and per element S[a], the entries of N(m) it
// compares before the match that keeps S[a] (position + 1), or all deg(m)
// when S[a] is not kept. Same control flow as fmc_heuristic_marked, so it
// costs O(|S| + deg(m)) per round; used to price the linear search at sizes
// where running it is out of reach.
static inline double fmc_scan_ops(const Csr& g, int first, int max_clq) {
  const int n = (int)g.off.size() - 1;
  auto deg = [&](int v) { return g.off[v + 1] - g.off[v]; };
  std::vector<int> S(std::max(g.max_deg, 0) + 1, 0), S1(std::max(g.max_deg, 0) + 1, 0);
  std::vector<int64_t> stamp(std::max(n, 1), -1);
  std::vector<int> where(std::max(n, 1), 0);
  int64_t round_id = 0;
  double ops = 0.0;
  for (int v = first; v < n; ++v) {
    if (max_clq > deg(v)) continue;
    int npos = 0;
    S[npos++] = v;
    for (int e = g.off[v]; e < g.off[v + 1]; ++e)
      if (max_clq <= deg(g.adj[e])) S[npos++] = g.adj[e];
    int icc = 0;
    while (npos > 0) {
      ++icc;
      const int m = S[npos - 1];
      ++round_id;
      for (int e = g.off[m]; e < g.off[m + 1]; ++e) {
        stamp[g.adj[e]] = round_id;
        where[g.adj[e]] = e - g.off[m];
      }
      int n1 = 0;
      int64_t cnt = 0;
      for (int a = 0; a < npos; ++a) {
        if (stamp[S[a]] == round_id && max_clq <= deg(S[a])) {
          S1[n1++] = S[a];
          cnt += where[S[a]] + 1;
        } else {
          cnt += deg(m);
        }
      }
      ops += (double)cnt;
      for (int a = 0; a < n1; ++a) S[a] = S1[a];
      npos = n1;
    }
    if (max_clq < icc) max_clq = icc;
  }
  return ops;
}

// The same heuristic on bit rows, for dense matrices. A candidate's list S is
// kept as v (always first) followed by a bitset of the other members, whose
// ascending order is the order of the reference's list: the kept elements
// keep their order, so "S <- elements of S adjacent to m" is S_bits &= N(m)
// (v stays: m is a neighbour of v; the degree filter of the round is already
// in S_bits), and m = S[last] is the highest set bit (v once S_bits is
// empty). The reference's work buffer is rebuilt for a winning candidate:
// the initial fill writes positions [0, n_0), round r writes [0, n_r), so
// position p ends with element p of the last list longer than p.
// Candidates are evaluated in windows on the OpenMP threads with the running
// best fixed; the first improving candidate of a window (in order) wins and
// the scan restarts after it, so every decision is the sequential scan's.
// ops_out (optional): the reference's linear-search inner iterations,
// estimated per round: a kept element costs its position in N(m) plus one
// (counted to its 64-bit word, inside the word at the word's mean), any
// other element all of N(m).
struct BitRows {
  int n = 0, w64 = 0;
  std::vector<uint64_t> row;  // n x w64
  std::vector<int> deg;
  BitRows(const std::vector<uint32_t>& bits, int n_, int words) : n(n_), w64((n_ + 63) / 64) {
    row.assign((size_t)n * w64, 0ull);
    deg.assign(n, 0);
    for (int i = 0; i < n; ++i) {
      uint64_t* r = &row[(size_t)i * w64];
      for (int w = 0; w < words && 32 * w < n; ++w) r[w >> 1] |= (uint64_t)bits[(size_t)i * words + w] << (32 * (w & 1));
      if (n % 64) r[w64 - 1] &= (~0ull) >> (64 - n % 64);
      r[i >> 6] &= ~(1ull << (i & 63));  // the diagonal is not an edge
      int d = 0;
      for (int w = 0; w < w64; ++w) d += __builtin_popcountll(r[w]);
      deg[i] = d;
    }
  }
  const uint64_t* of(int i) const { return &row[(size_t)i * w64]; }
};

// Rounds of candidate v with running best max_clq (dmask: vertices of degree
// >= max_clq); S: w64 words of scratch. n_sizes (optional): list length after
// each round, [0] the initial fill; keep (optional): each round's member set.
// Returns the round count icc.
static inline int fmc_bits_candidate(const BitRows& g, int v, const std::vector<uint64_t>& dmask,
                                     std::vector<uint64_t>& S, std::vector<int>* n_sizes,
                                     std::vector<std::vector<uint64_t>>* keep, double* ops) {
  const int W = g.w64;
  const uint64_t* nv = g.of(v);
  int cnt = 0, hi = -1;
  for (int w = 0; w < W; ++w) {
    S[w] = nv[w] & dmask[w];
    if (S[w]) {
      cnt += __builtin_popcountll(S[w]);
      hi = w;
    }
  }
  if (n_sizes) n_sizes->assign(1, 1 + cnt);
  if (keep) keep->assign(1, std::vector<uint64_t>(S.begin(), S.end()));
  int icc = 0;
  int npos = 1 + cnt;
  while (npos > 0) {
    ++icc;
    if (cnt == 0) {  // m = v, not adjacent to itself: the list empties
      if (ops) *ops += (double)g.deg[v];
      npos = 0;
      if (n_sizes) n_sizes->push_back(0);
      break;
    }
    const int m = 64 * hi + 63 - __builtin_clzll(S[hi]);
    const uint64_t* nm = g.of(m);
    int kept = 0, nh = -1;
    double rank_sum = 0.0;
    int prefix = 0;
    for (int w = 0; w <= hi; ++w) {
      const int pn = __builtin_popcountll(nm[w]);
      S[w] &= nm[w];
      if (S[w]) {
        const int kw = __builtin_popcountll(S[w]);
        kept += kw;
        nh = w;
        if (ops) rank_sum += (double)kw * ((double)prefix + 0.5 * (double)pn);
      }
      prefix += pn;
    }
    if (ops) {
      // the search for a kept element stops at its position in N(m), v's
      // included; the others (m among them) scan all of N(m)
      int vrank = 0;
      for (int w = 0; w < (v >> 6); ++w) vrank += __builtin_popcountll(nm[w]);
      vrank += __builtin_popcountll(nm[v >> 6] & ((1ull << (v & 63)) - 1ull));
      *ops += rank_sum + (double)kept + (double)(vrank + 1) + (double)(cnt - kept) * (double)g.deg[m];
    }
    cnt = kept;
    hi = nh;
    npos = 1 + cnt;
    if (n_sizes) n_sizes->push_back(npos);
    if (keep) keep->push_back(std::vector<uint64_t>(S.begin(), S.begin() + W));
  }
  return icc;
}

static inline int fmc_heuristic_bits(const BitRows& g, int first, int max_clq, std::vector<int>* best,
                                     double* ops_out = nullptr) {
  const int n = g.n, W = g.w64;
  std::vector<uint64_t> dmask(W, 0ull);
  auto build_mask = [&](int m) {
    std::fill(dmask.begin(), dmask.end(), 0ull);
    for (int i = 0; i < n; ++i)
      if (m <= g.deg[i]) dmask[i >> 6] |= 1ull << (i & 63);
  };
  build_mask(max_clq);
  double ops = 0.0;
  int v = std::max(first, 0);
  const int window = 64;
  std::vector<int> res(window);
  std::vector<double> wops(window);
  while (v < n) {
    const int cnt = std::min(window, n - v);
#pragma omp parallel
    {
      std::vector<uint64_t> S(W);
#pragma omp for schedule(dynamic, 1)
      for (int k = 0; k < cnt; ++k) {
        const int c = v + k;
        wops[k] = 0.0;
        if (max_clq > g.deg[c]) {
          res[k] = -1;
          continue;
        }
        res[k] = fmc_bits_candidate(g, c, dmask, S, nullptr, nullptr, ops_out ? &wops[k] : nullptr);
      }
    }
    int improved = -1;
    for (int k = 0; k < cnt; ++k) {
      if (ops_out) ops += wops[k];
      if (res[k] > max_clq) {
        improved = k;
        break;
      }
    }
    if (improved < 0) {
      v += cnt;
      continue;
    }
    const int c = v + improved;
    // the winner again, keeping its rounds, to rebuild its work buffer;
    // positions [0, icc) lie inside its own initial fill, so no earlier
    // candidate's writes survive there
    std::vector<uint64_t> S(W);
    std::vector<int> sizes;
    std::vector<std::vector<uint64_t>> rounds;
    const int icc = fmc_bits_candidate(g, c, dmask, S, &sizes, &rounds, nullptr);
    std::vector<int> out((size_t)std::max(icc, 0), 0);
    // list r (0 = the initial fill) is final on positions [sizes[r + 1], sizes[r])
    for (size_t r = 0; r + 1 < sizes.size(); ++r) {
      const int lo = sizes[r + 1], hi2 = std::min(sizes[r], icc);
      if (lo >= hi2) continue;
      // element p of list r: p = 0 is c, p >= 1 the p-th member in ascending order
      int p = 0;
      if (lo == 0) out[p++] = c;
      p = std::max(p, lo);
      int rank = 0;
      const std::vector<uint64_t>& R = rounds[r];
      for (int w = 0; w < W && p < hi2; ++w) {
        uint64_t x = R[w];
        const int pc = __builtin_popcountll(x);
        if (rank + pc < p) {
          rank += pc;
          continue;
        }
        while (x && p < hi2) {
          const int b = __builtin_ctzll(x);
          x &= x - 1;
          ++rank;
          if (rank >= p) out[p++] = 64 * w + b;
        }
      }
    }
    *best = out;
    max_clq = icc;
    build_mask(max_clq);
    v = c + 1;
  }
  if (ops_out) *ops_out = ops;
  return max_clq;
}

// Which form the oracle runs: 0 = the reference's linear search (default),
// 1 = the membership-stamp form, 2 = the bit-row form (identical results;
// 1 and 2 are for checks at large sizes).
inline int g_clique_impl = 0;
static inline int fmc_heuristic(const Csr& g, int first, int max_clq, std::vector<int>* best) {
  return g_clique_impl == 1 ? fmc_heuristic_marked(g, first, max_clq, best)
                            : fmc_heuristic_scan(g, first, max_clq, best);
}
// the heuristic of a bit-packed matrix (n x words uint32) in the selected form
static inline int fmc_from_bits(const std::vector<uint32_t>& bits, int n, int words, int first, int max_clq,
                                std::vector<int>* best) {
  if (g_clique_impl == 2) return fmc_heuristic_bits(BitRows(bits, n, words), first, max_clq, best);
  return fmc_heuristic(csr_from_bits(bits, n, words), first, max_clq, best);
}

// ---------------------------------------------------------------- factor records
template <class L>
struct Factor {
  int kind = 0;  // 0 between, 1 prior
  uint64_t k1 = 0, k2 = 0;
  typename L::Pose measured = L::identity();
  double cov[L::dim * L::dim] = {0};
  double sqrt_info[L::dim * L::dim] = {0};
  int64_t src = -1;  // index in the input batch (checks only)
};

// ObservationId (TypeUtils.h:44-58) with the same symmetric equality and
// hash (TypeUtils.h:80-88), so std::unordered_map iterates in the same
// order as the reference's.
struct ObsId {
  char id1, id2;
  bool operator==(const ObsId& o) const {
    return (id1 == o.id1 && id2 == o.id2) || (id2 == o.id1 && id1 == o.id2);
  }
};
struct ObsIdHash {
  size_t operator()(const ObsId& id) const {
    std::hash<char> h;
    return h(id.id1) + h(id.id2) + h(id.id1) * h(id.id2);
  }
};

template <class L>
struct Group {
  std::vector<Factor<L>> factors;
  std::vector<Factor<L>> consistent;
  int n = 0, words = 0;
  int adj_rows = 1;  // rows of adj_matrix: 1 for a fresh Measurements (TypeUtils.h:16-33)
  std::vector<uint32_t> bits;  // n x words, symmetric
  void grow(int new_n) {
    const int nw = (new_n + 31) / 32;
    std::vector<uint32_t> nb((size_t)new_n * nw, 0u);
    for (int i = 0; i < n; ++i)
      for (int w = 0; w < words; ++w) nb[(size_t)i * nw + w] = bits[(size_t)i * words + w];
    bits.swap(nb);
    n = new_n;
    words = nw;
  }
  void set(int i, int j) {
    bits[(size_t)i * words + (j >> 5)] |= 1u << (j & 31);
    bits[(size_t)j * words + (i >> 5)] |= 1u << (i & 31);
  }
  // adj_matrix.block(0, 0, m, m)
  void shrink(int m) {
    const int nw = (m + 31) / 32;
    std::vector<uint32_t> nb((size_t)m * nw, 0u);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j)
        if (bits[(size_t)i * words + (j >> 5)] >> (j & 31) & 1u) nb[(size_t)i * nw + (j >> 5)] |= 1u << (j & 31);
    bits.swap(nb);
    n = m;
    words = nw;
  }
};

struct PcmParamsO {
  double odom_threshold = 10.0, lc_threshold = 5.0;
  double odom_trans_threshold = 0.05, odom_rot_threshold = 0.005;
  double dist_trans_threshold = 0.01, dist_rot_threshold = 0.001;
  bool incremental = false;
  std::vector<char> special;  // special (landmark) symbols
};

// U = PWC<L> (Pcm2D/Pcm3D) or PWN<L> (PcmSimple2D/PcmSimple3D)
template <class L, class U>
struct Pcm {
  static constexpr bool kSimple = !std::is_same<U, PWC<L>>::value;
  PcmParamsO params;
  bool odom_check = true, lc_check = true;
  std::vector<Factor<L>> nfg_odom, nfg_special;
  std::unordered_map<ObsId, Group<L>, ObsIdHash> loop_closures;
  std::unordered_map<uint64_t, Group<L>> landmarks;  // landmarks_ (Pcm.h)
  std::vector<ObsId> in_order;   // loop_closures_in_order_ (Pcm.h:112)
  std::vector<char> robot_order; // robot_order_ (Pcm.h:128)
  std::vector<char> ignored;     // ignored_prefixes_ (Pcm.h:117)
  std::unordered_map<char, Trajectory<U>> trajectories;
  size_t total_lc = 0, total_good_lc = 0;
  bool warned_missing = false;
  // checks at large sizes: parse, odometry-check and group the closures but
  // leave the consistency matrix and the clique to sample_rows
  bool defer_lc = false;

  explicit Pcm(const PcmParamsO& p) : params(p) {
    if (p.odom_threshold < 0 || p.odom_rot_threshold < 0 || p.odom_trans_threshold < 0) odom_check = false;
    if (p.lc_threshold < 0 || p.dist_rot_threshold < 0 || p.dist_trans_threshold < 0) lc_check = false;
  }

  bool check_odom(const U& r) const {
    if constexpr (kSimple) {
      return r.avg_trans_norm() < params.odom_trans_threshold && r.avg_rot_norm() < params.odom_rot_threshold;
    } else {
      return r.mahalanobis_norm() < params.odom_threshold;
    }
  }
  bool check_loop(const U& r) const {
    if constexpr (kSimple) {
      return r.avg_trans_norm() < params.dist_trans_threshold && r.avg_rot_norm() < params.dist_rot_threshold;
    } else {
      return r.mahalanobis_norm() < params.lc_threshold;
    }
  }
  // Pcm.h:604-629
  bool is_odom_consistent(const Factor<L>& f) {
    if (!odom_check) return true;
    U pij = trajectories[key_chr(f.k1)].getBetween(f.k1, f.k2);
    U pji = U::from_factor(f.measured, f.cov).inverse();
    return check_odom(pij.compose(pji));
  }
  // Pcm.h:670-718
  bool are_loops_consistent(const Factor<L>& ab, const Factor<L>& cd) {
    if (!lc_check) return true;
    uint64_t ka = ab.k1, kb = ab.k2, kc = cd.k1, kd = cd.k2;
    U a_lc_b = U::from_factor(ab.measured, ab.cov);
    U c_lc_d = U::from_factor(cd.measured, cd.cov);
    if (key_chr(ka) != key_chr(kc)) std::swap(kc, kd);
    U a_odom_c = trajectories[key_chr(ka)].getBetween(ka, kc);
    U b_odom_d = trajectories[key_chr(kb)].getBetween(kb, kd);
    U a_path_d = a_odom_c.compose(c_lc_d);
    U d_path_b = a_path_d.inverse().compose(a_lc_b);
    U loop = d_path_b.compose(b_odom_d);
    return check_loop(loop);
  }
  // Pcm.h:516-557
  template <class ValuesMap>
  void update_odom(const Factor<L>& f, const ValuesMap& values) {
    nfg_odom.push_back(f);
    const char prefix = key_chr(f.k2);
    U delta = U::from_factor(f.measured, f.cov);
    if (trajectories.find(prefix) == trajectories.end()) {
      U init;
      init.pose = values.at(f.k1);
      trajectories[prefix].poses[f.k1] = init;
      robot_order.push_back(prefix);
    }
    U prev = trajectories[prefix].poses[f.k1];
    trajectories[prefix].poses[f.k2] = prev.compose(delta);
  }
  // Pcm.h:506-511
  bool is_special(char c) const {
    return std::find(params.special.begin(), params.special.end(), c) != params.special.end();
  }
  uint64_t landmark_key(const Factor<L>& f) const { return is_special(key_chr(f.k1)) ? f.k1 : f.k2; }
  // Pcm.h:775-844 for the newest observation of a landmark. Observations
  // stored landmark -> pose are warned about and left inconsistent with every
  // other (the reference abandons the whole matrix update there).
  void increment_landmark(Group<L>& g, uint64_t lk) {
    const int num_lc = (int)g.factors.size();
    g.grow(num_lc);
    g.adj_rows = num_lc;
    if (num_lc < 2) return;
    const Factor<L>& fj = g.factors[num_lc - 1];
    const U j_pose_l = U::from_factor(fj.measured, fj.cov);
    for (int i = 0; i < num_lc - 1; ++i) {
      const Factor<L>& fi = g.factors[i];
      if (fi.k1 == lk || fj.k1 == lk) continue;
      const U i_pose_l = U::from_factor(fi.measured, fi.cov);
      U i_odom_j = trajectories[key_chr(fi.k1)].getBetween(fi.k1, fj.k1);
      U i_path_l = i_odom_j.compose(j_pose_l);
      U loop = i_path_l.inverse().compose(i_pose_l);
      if (check_loop(loop)) g.set(i, num_lc - 1);
    }
  }
  // findMaxCliqueHeu over a landmark's adjacency (Pcm.h:878-897)
  size_t landmark_inliers(Group<L>& g) {
    g.consistent.clear();
    if (g.n < g.adj_rows) g.grow(g.adj_rows);
    std::vector<int> idx;
    const int sz = fmc_from_bits(g.bits, g.adj_rows, g.words, 0, -1, &idx);
    for (int i = 0; i < sz; ++i)
      if (idx[i] < (int)g.factors.size()) g.consistent.push_back(g.factors[idx[i]]);
    return g.consistent.size();
  }

  // Pcm.h:725-768 for every new member of the group against all earlier ones.
  // The pair tests are independent: with OpenMP threads, each new row j is
  // filled by one thread (bits i < j of row j), then one pass mirrors them;
  // the matrix is the same as the sequential fill's.
  void increment_adjacency(Group<L>& g, int old_n) {
    g.grow((int)g.factors.size());
    g.adj_rows = g.n;
    const int n = g.n, words = g.words;
#pragma omp parallel for schedule(dynamic, 4)
    for (int j = old_n; j < n; ++j)
      for (int i = 0; i < j; ++i)
        if (are_loops_consistent(g.factors[i], g.factors[j])) g.bits[(size_t)j * words + (i >> 5)] |= 1u << (i & 31);
    for (int i = 0; i < n; ++i)
      for (int j = std::max(i + 1, old_n); j < n; ++j)
        if (g.bits[(size_t)j * words + (i >> 5)] >> (i & 31) & 1u) g.bits[(size_t)i * words + (j >> 5)] |= 1u << (j & 31);
  }

  template <class ValuesMap>
  void parse_and_increment(const std::vector<Factor<L>>& lcs, const ValuesMap& values,
                           std::unordered_map<ObsId, size_t, ObsIdHash>* num_new) {
    // the reference grows each group one closure at a time; doing all checks
    // of a batch after the appends gives the same matrix because the pair
    // test depends only on the two closures and the (fixed) trajectories.
    std::unordered_map<ObsId, int, ObsIdHash> old_sizes;
    std::vector<ObsId> touched;
    for (const auto& f : lcs) {
      if (!values.count(f.k1) || !values.count(f.k2)) continue;
      const char c1 = key_chr(f.k1), c2 = key_chr(f.k2);
      if (is_special(c1) || is_special(c2)) {
        // landmark re-observation (Pcm.h:440-454)
        const uint64_t lk = landmark_key(f);
        Group<L>& lg = landmarks[lk];
        lg.factors.push_back(f);
        ++total_lc;
        increment_landmark(lg, lk);
        continue;
      }
      bool ok = true;
      if (c1 == c2) ok = is_odom_consistent(f);
      if (!ok) continue;
      ObsId id{c1, c2};
      auto it = num_new->find(id);
      if (it == num_new->end()) num_new->insert({id, 1});
      else it->second++;
      Group<L>& g = loop_closures[id];
      if (!old_sizes.count(id)) {
        old_sizes[id] = (int)g.factors.size();
        touched.push_back(id);
      }
      g.factors.push_back(f);
      in_order.push_back(id);
      ++total_lc;
    }
    if (lc_check && !defer_lc)
      for (const auto& id : touched) increment_adjacency(loop_closures[id], old_sizes[id]);
  }

  void find_inliers() {
    total_good_lc = 0;
    for (auto& kv : loop_closures) {
      Group<L>& g = kv.second;
      size_t num;
      if (lc_check) {
        g.consistent.clear();
        std::vector<int> idx;
        const int sz = fmc_from_bits(g.bits, g.n, g.words, 0, -1, &idx);
        // indices past the closures (an adjacency kept larger by a removal)
        // are dropped; the reference would index past its factor list
        for (int i = 0; i < sz; ++i)
          if (idx[i] < (int)g.factors.size()) g.consistent.push_back(g.factors[idx[i]]);
        num = g.consistent.size();
      } else {
        g.consistent = g.factors;
        num = g.factors.size();
      }
      total_good_lc += num;
    }
    for (auto& kv : landmarks) total_good_lc += landmark_inliers(kv.second);
  }
  void find_inliers_incremental(const std::unordered_map<ObsId, size_t, ObsIdHash>& num_new) {
    total_good_lc = 0;
    for (const auto& kv : num_new) {
      Group<L>& g = loop_closures[kv.first];
      const size_t prev = g.consistent.size();
      std::vector<int> idx;
      const int first = g.n - (int)kv.second;
      int num = fmc_from_bits(g.bits, g.n, g.words, first, (int)prev, &idx);
      if ((size_t)num > prev) {
        g.consistent.clear();
        for (int i = 0; i < num; ++i)
          if (idx[i] < (int)g.factors.size()) g.consistent.push_back(g.factors[idx[i]]);
      }
    }
    for (const auto& kv : loop_closures) total_good_lc += kv.second.consistent.size();
    for (auto& kv : landmarks) total_good_lc += landmark_inliers(kv.second);
  }
  // Pcm.h:977-1005
  std::vector<Factor<L>> build_graph() const {
    std::vector<Factor<L>> out(nfg_odom);
    out.insert(out.end(), nfg_special.begin(), nfg_special.end());
    auto is_ignored = [this](char c) { return std::find(ignored.begin(), ignored.end(), c) != ignored.end(); };
    for (const auto& kv : loop_closures) {
      if (is_ignored(kv.first.id1) || is_ignored(kv.first.id2)) continue;
      out.insert(out.end(), kv.second.consistent.begin(), kv.second.consistent.end());
    }
    for (const auto& kv : landmarks) out.insert(out.end(), kv.second.consistent.begin(), kv.second.consistent.end());
    return out;
  }

  // Pcm.h:299-342 (a group with no closure left returns false; the reference
  // would index its empty factor list)
  bool remove_last(const ObsId& id, uint64_t* k1, uint64_t* k2, std::vector<Factor<L>>* out) {
    auto it = loop_closures.find(id);
    if (it == loop_closures.end()) return false;
    Group<L>& g = it->second;
    const int num_lc = g.adj_rows;
    if (num_lc <= 0 || g.factors.empty()) return false;
    *k1 = g.factors.back().k1;
    *k2 = g.factors.back().k2;
    g.factors.pop_back();
    if (g.factors.size() < 2) {
      g.consistent = g.factors;
    } else {
      const int m = num_lc - 1;
      g.adj_rows = m;
      g.consistent.clear();
      if (lc_check && g.n >= m) {
        g.shrink(m);
        std::vector<int> idx;
        const int sz = fmc_from_bits(g.bits, g.n, g.words, 0, -1, &idx);
        for (int i = 0; i < sz; ++i)
          if (idx[i] < (int)g.factors.size()) g.consistent.push_back(g.factors[idx[i]]);
      } else if (m > 0) {
        g.consistent.push_back(g.factors[0]);  // greedy clique of an edgeless graph
      }
    }
    *out = build_graph();
    return true;
  }
  // Pcm.h:347-353
  bool remove_last_in_order(uint64_t* k1, uint64_t* k2, std::vector<Factor<L>>* out) {
    if (in_order.empty()) return false;
    const ObsId id = in_order.back();
    in_order.pop_back();
    return remove_last(id, k1, k2, out);
  }
  // Pcm.h:357-376
  void ignore_prefix(char c, std::vector<Factor<L>>* out) {
    if (std::find(ignored.begin(), ignored.end(), c) == ignored.end()) ignored.push_back(c);
    *out = build_graph();
  }
  void revive_prefix(char c, std::vector<Factor<L>>* out) {
    ignored.erase(std::remove(ignored.begin(), ignored.end(), c), ignored.end());
    *out = build_graph();
  }
  // Pcm.h:386-408
  void remove_priors_with_prefix(char c, std::vector<Factor<L>>* out) {
    std::vector<Factor<L>> kept;
    for (const auto& f : nfg_special)
      if (f.kind != 1 || key_chr(f.k1) != c) kept.push_back(f);
    nfg_special.swap(kept);
    *out = build_graph();
  }

  // Rows of a group's consistency matrix as incrementAdjMatrix (Pcm.h:725-768)
  // fills it: bit (r, c), r != c, is are_loops_consistent(factor min(r, c),
  // factor max(r, c)). out: rows.size() x ceil(n / 32) words. Words are
  // independent, so they are spread over the OpenMP threads. lower_only:
  // columns c < r only (the pairs that new row r adds, as the reference
  // evaluates them).
  void sample_rows(Group<L>& g, const std::vector<int>& rows, std::vector<uint32_t>* out, bool lower_only = false) {
    const int n = (int)g.factors.size(), words = (n + 31) / 32;
    out->assign(rows.size() * (size_t)words, 0u);
    const int64_t tasks = (int64_t)rows.size() * words;
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t t = 0; t < tasks; ++t) {
      const int r = rows[t / words], w = (int)(t % words);
      uint32_t x = 0u;
      for (int b = 0; b < 32; ++b) {
        const int c = 32 * w + b;
        if (c >= n || c == r || (lower_only && c > r)) continue;
        const int i = std::min(r, c), j = std::max(r, c);
        if (are_loops_consistent(g.factors[i], g.factors[j])) x |= 1u << b;
      }
      (*out)[t] = x;
    }
  }

  // Pcm.h:148-281. values: the solver's value map, already extended by the
  // caller with new_values. Returns do_optimize.
  template <class ValuesMap, class KeySet>
  bool remove_outliers(const std::vector<Factor<L>>& new_factors, const KeySet& new_keys, const ValuesMap& values,
                       std::vector<Factor<L>>* out_graph) {
    if (new_factors.empty()) return false;
    bool do_optimize = false;
    std::vector<Factor<L>> lcs;
    for (const auto& f : new_factors) {
      if (f.kind == 0) {
        if (is_special(key_chr(f.k1)) || is_special(key_chr(f.k2))) {
          if (new_keys.count(f.k1) || new_keys.count(f.k2)) {
            // first observation of a landmark (Pcm.h:209-220)
            Group<L> g;
            g.factors.push_back(f);
            g.consistent.push_back(f);
            landmarks[landmark_key(f)] = g;
            ++total_lc;
          } else if (f.k1 != f.k2) {
            lcs.push_back(f);
          }
        } else if (f.k1 + 1 == f.k2 && new_keys.count(f.k2)) {
          update_odom(f, values);
        } else if (f.k1 != f.k2) {
          lcs.push_back(f);
        }
      } else {
        nfg_special.push_back(f);
        do_optimize = true;
      }
    }
    if (!lcs.empty()) {
      std::unordered_map<ObsId, size_t, ObsIdHash> num_new;
      parse_and_increment(lcs, values, &num_new);
      if (defer_lc) {
        // nothing: sample_rows evaluates the requested rows
      } else if (params.incremental) {
        find_inliers_incremental(num_new);
      } else {
        find_inliers();
      }
      do_optimize = true;
    }
    *out_graph = build_graph();
    return do_optimize;
  }
};

}  // namespace oracle

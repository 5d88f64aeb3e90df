// Symbolic analysis for the direct solve; see chol_plan.hpp.
#include "chol_plan.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <exception>
#include <functional>
#include <queue>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>

namespace rpgo {
namespace {

// time model of the solve kernel (per grid-barrier phase, per FP64 flop)
constexpr double kPhaseUs = 8.0;
constexpr double kUsPerFlop = 5e-6;

// Elimination game on the variable graph: eliminating u records its current
// neighbours (the structure of its column of L, as variables) and joins them
// into a clique.
struct Elimination {
  std::vector<std::vector<int32_t>>& adj;
  std::vector<char> alive;
  std::vector<int32_t> order;
  std::vector<std::vector<int32_t>> col_vars;
  std::vector<int32_t> merged;
  explicit Elimination(std::vector<std::vector<int32_t>>& a) : adj(a), alive(a.size(), 1), col_vars(a.size()) {
    order.reserve(a.size());
  }
  template <class OnDegree>
  void eliminate(int u, OnDegree&& on_degree) {
    alive[u] = 0;
    order.push_back(u);
    std::vector<int32_t> nb;
    nb.swap(adj[u]);
    for (int w : nb) {
      // adj[w] <- (adj[w] \ {u}) U (nb \ {w})
      const std::vector<int32_t>& a = adj[w];
      merged.clear();
      merged.reserve(a.size() + nb.size());
      size_t i = 0, j = 0;
      while (i < a.size() || j < nb.size()) {
        int32_t x;
        if (j >= nb.size() || (i < a.size() && a[i] < nb[j])) x = a[i++];
        else if (i >= a.size() || nb[j] < a[i]) x = nb[j++];
        else {
          x = a[i++];
          ++j;
        }
        if (x != u && x != w) merged.push_back(x);
      }
      adj[w].assign(merged.begin(), merged.end());
      on_degree(w);
    }
    col_vars[u] = std::move(nb);
  }
};

// Elimination order:
//  1. the interior of every chain of degree-2 variables (odometry between loop
//     closures, dangling trajectory ends) by cyclic reduction: alternate chain
//     variables first, then alternate survivors, ... This costs no more fill
//     than eliminating the chain from one end and makes the elimination tree
//     log2(length) deep over the chain instead of length deep;
//  2. the remaining variables by minimum degree (ties by the smaller index).
void order_variables(int N, std::vector<std::vector<int32_t>>& adj, std::vector<int32_t>* order,
                     std::vector<std::vector<int32_t>>* col_vars) {
  Elimination el(adj);
  // 1. chains of variables of degree <= 2
  std::vector<char> in_chain(N, 0), seen(N, 0);
  for (int u = 0; u < N; ++u) in_chain[u] = adj[u].size() <= 2;
  std::vector<std::pair<int, int>> keyed;  // (cyclic-reduction level, variable)
  std::vector<int32_t> path;
  for (int s = 0; s < N; ++s) {
    if (!in_chain[s] || seen[s]) continue;
    // walk to one end of the chain through chain variables
    int prev = -1, cur = s;
    while (true) {
      int nxt = -1;
      for (int w : adj[cur])
        if (w != prev && in_chain[w] && w != s) {
          nxt = w;
          break;
        }
      if (nxt < 0) break;
      prev = cur;
      cur = nxt;
    }
    // collect the chain from that end
    path.clear();
    prev = -1;
    while (cur >= 0 && !seen[cur]) {
      seen[cur] = 1;
      path.push_back(cur);
      int nxt = -1;
      for (int w : adj[cur])
        if (w != prev && in_chain[w] && !seen[w]) {
          nxt = w;
          break;
        }
      prev = cur;
      cur = nxt;
    }
    for (size_t t = 0; t < path.size(); ++t) {
      const unsigned pos1 = (unsigned)t + 1;
      keyed.push_back({__builtin_ctz(pos1), path[t]});
    }
  }
  std::stable_sort(keyed.begin(), keyed.end(),
                   [](const std::pair<int, int>& a, const std::pair<int, int>& b) { return a.first < b.first; });
  for (const auto& kv : keyed) el.eliminate(kv.second, [](int) {});
  // 2. minimum degree on what remains
  using Entry = std::pair<int32_t, int32_t>;  // (degree, variable)
  std::priority_queue<Entry, std::vector<Entry>, std::greater<Entry>> pq;
  for (int u = 0; u < N; ++u)
    if (el.alive[u]) pq.push({(int32_t)adj[u].size(), u});
  auto push = [&](int w) { pq.push({(int32_t)adj[w].size(), w}); };
  while (!pq.empty()) {
    const Entry e = pq.top();
    pq.pop();
    const int u = e.second;
    if (!el.alive[u] || e.first != (int32_t)adj[u].size()) continue;
    el.eliminate(u, push);
  }
  *order = std::move(el.order);
  *col_vars = std::move(el.col_vars);
}

// Nested dissection by breadth-first level structures: a connected set is
// split at the level of a breadth-first search from a pseudo-peripheral
// variable whose variables (those with a neighbour in the next level) form
// the smallest separator that leaves at least a quarter of the set on each
// side; both halves are ordered recursively, the separator last. Pose graphs
// whose closures are local (a thick chain) have separators a few variables
// wide, so the elimination tree stays about log2(N) separators deep where
// minimum degree, eliminating such a band from one end, makes it about N deep.
// One recursion gives the orders for two leaf sizes (`out` for `leaf`, `out2`
// for the larger `leaf2`): sets above leaf2 split the same way in both.
struct NestedDissection {
  const std::vector<std::vector<int32_t>>& adj;
  int leaf, leaf2;
  std::vector<int32_t> inset, vis, level;
  int set_id = 0, bfs_id = 0;
  std::vector<int32_t> out, out2;
  NestedDissection(const std::vector<std::vector<int32_t>>& a, int lf, int lf2)
      : adj(a), leaf(lf), leaf2(lf2), inset(a.size(), 0), vis(a.size(), 0), level(a.size(), 0) {}

  // breadth-first search inside the current set; returns the visit order
  void bfs(int root, std::vector<int32_t>* q) {
    ++bfs_id;
    q->clear();
    q->push_back(root);
    vis[root] = bfs_id;
    level[root] = 0;
    for (size_t h = 0; h < q->size(); ++h) {
      const int u = (*q)[h];
      for (int w : adj[u])
        if (inset[w] == set_id && vis[w] != bfs_id) {
          vis[w] = bfs_id;
          level[w] = level[u] + 1;
          q->push_back(w);
        }
    }
  }

  // two: the set is still above leaf2 for the second order; the two halves
  // of a large set in the first kParDepth splits are ordered concurrently
  // (a second instance on its own thread, its orders inserted before the
  // other half's: the same orders as one thread's); up to 16 threads
  static constexpr int kParDepth = 4, kParMin = 2048;
  void run(std::vector<int32_t> nodes, bool two, int split = 0) {
    if (two && (int)nodes.size() <= leaf2) {
      std::vector<int32_t> sorted = nodes;
      std::sort(sorted.begin(), sorted.end());
      out2.insert(out2.end(), sorted.begin(), sorted.end());
      two = false;
    }
    if ((int)nodes.size() <= leaf) {
      std::sort(nodes.begin(), nodes.end());
      out.insert(out.end(), nodes.begin(), nodes.end());
      return;
    }
    ++set_id;
    for (int u : nodes) inset[u] = set_id;
    std::vector<int32_t> q;
    bfs(nodes[0], &q);
    if (q.size() < nodes.size()) {
      // several components: order each on its own
      std::vector<std::vector<int32_t>> comps;
      const int sid = set_id;
      comps.push_back(q);
      ++bfs_id;
      const int mark = bfs_id;
      for (int u : q) vis[u] = mark;
      for (int u : nodes) {
        if (vis[u] == mark) continue;
        set_id = sid;
        std::vector<int32_t> c;
        bfs(u, &c);
        for (int w : c) vis[w] = mark;
        comps.push_back(std::move(c));
      }
      for (auto& c : comps) run(std::move(c), two, split);
      return;
    }
    // pseudo-peripheral root: repeat the search from the farthest variable
    int root = nodes[0], depth = 0;
    for (int sweep = 0; sweep < 4; ++sweep) {
      const int far = q.back();
      if (level[far] <= depth && sweep > 0) break;
      depth = level[far];
      root = far;
      bfs(root, &q);
    }
    // q and level now hold the search from root
    const int L = level[q.back()] + 1;
    std::vector<int32_t> cnt(L + 1, 0);
    for (int u : q) cnt[level[u]]++;
    const int n = (int)q.size();
    int best_m = -1, best = 1 << 30, below = 0;
    for (int m = 0; m < L; ++m) {
      const int above = n - below - cnt[m];
      if (m > 0 && m + 1 < L && 4 * below >= n && 4 * above >= n && cnt[m] < best) {
        best = cnt[m];
        best_m = m;
      }
      below += cnt[m];
    }
    if (best_m < 0) {
      // no balanced level split (a star or a tiny diameter): keep the set whole
      std::sort(nodes.begin(), nodes.end());
      out.insert(out.end(), nodes.begin(), nodes.end());
      if (two) out2.insert(out2.end(), nodes.begin(), nodes.end());
      return;
    }
    std::vector<int32_t> A, B, S;
    for (int u : q) {
      const int l = level[u];
      if (l < best_m) A.push_back(u);
      else if (l > best_m) B.push_back(u);
      else {
        bool touches_next = false;
        for (int w : adj[u])
          if (inset[w] == set_id && level[w] == best_m + 1) {
            touches_next = true;
            break;
          }
        (touches_next ? S : A).push_back(u);
      }
    }
    if (split < kParDepth && (int)(A.size() + B.size()) > kParMin) {
      NestedDissection other(adj, leaf, leaf2);
      std::exception_ptr err;
      std::thread t([&] {
        try {
          other.run(std::move(A), two, split + 1);
        } catch (...) {
          err = std::current_exception();
        }
      });
      const size_t at = out.size(), at2 = out2.size();
      try {
        run(std::move(B), two, split + 1);
      } catch (...) {
        t.join();
        throw;
      }
      t.join();
      if (err) std::rethrow_exception(err);
      out.insert(out.begin() + at, other.out.begin(), other.out.end());
      out2.insert(out2.begin() + at2, other.out2.begin(), other.out2.end());
    } else {
      run(std::move(A), two, split + 1);
      run(std::move(B), two, split + 1);
    }
    std::sort(S.begin(), S.end());
    out.insert(out.end(), S.begin(), S.end());
    if (two) out2.insert(out2.end(), S.begin(), S.end());
  }
};

// Symbolic elimination in a given order: the same column structures as the
// elimination game (the neighbours of each variable when it is eliminated),
// from the elimination tree in time linear in the factor's size. Column j's
// structure is its later neighbours together with its children's structures
// less j itself (a child c's parent is the first variable of c's structure).
// Output: column j (elimination position) holds positions
// idx[ptr[j] .. ptr[j + 1]), unsorted.
void eliminate_in_order(const std::vector<std::vector<int32_t>>& adj, const std::vector<int32_t>& order,
                        std::vector<int32_t>* ptr, std::vector<int32_t>* idx) {
  const int N = (int)order.size();
  std::vector<int32_t> pos(adj.size(), -1), mark(N, -1), first_child(N, -1), next_sibling(N, -1);
  for (int j = 0; j < N; ++j) pos[order[j]] = j;
  ptr->assign(N + 1, 0);
  idx->clear();
  idx->reserve((size_t)8 * N);
  for (int j = 0; j < N; ++j) {
    const size_t b = idx->size();
    for (int w : adj[order[j]]) {
      const int x = pos[w];
      if (x > j && mark[x] != j) {
        mark[x] = j;
        idx->push_back(x);
      }
    }
    for (int ch = first_child[j]; ch >= 0; ch = next_sibling[ch])
      for (int q = (*ptr)[ch]; q < (*ptr)[ch + 1]; ++q) {
        const int x = (*idx)[q];
        if (x != j && mark[x] != j) {
          mark[x] = j;
          idx->push_back(x);
        }
      }
    (*ptr)[j + 1] = (int32_t)idx->size();
    if (idx->size() > b) {
      const int parent = *std::min_element(idx->begin() + b, idx->end());
      next_sibling[j] = first_child[parent];
      first_child[parent] = j;
    }
  }
}

int find_block(const CholPlan& p, int col, int row) {
  if (row == col) return p.col_ptr[col];
  const auto b = p.blk_row.begin() + p.col_ptr[col] + 1, e = p.blk_row.begin() + p.col_ptr[col + 1];
  const auto it = std::lower_bound(b, e, row);
  if (it == e || *it != row)
    throw std::logic_error("chol plan: block (" + std::to_string(row) + ", " + std::to_string(col) +
                           ") outside the symbolic structure");
  return (int)(it - p.blk_row.begin());
}

}  // namespace

CholPlan make_chol_plan(int N, int d, const std::vector<int32_t>& kind, const std::vector<int32_t>& vi,
                        const std::vector<int32_t>& vj, bool dense_tail) {
  CholPlan p;
  p.N = N;
  p.d = d;
  const size_t F = kind.size();
  std::vector<std::vector<int32_t>> adj(N);
  for (size_t f = 0; f < F; ++f)
    if (kind[f] == 0 && vi[f] != vj[f]) {
      adj[vi[f]].push_back(vj[f]);
      adj[vj[f]].push_back(vi[f]);
    }
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  // Candidate orders, kept by a model of the solve kernel's time: every
  // grid-barrier phase (three per sparse level, two per dense tile) costs
  // about kPhaseUs, every FP64 flop of the factorisation kUsPerFlop.
  struct Candidate {
    std::vector<int32_t> perm, pos;
    std::vector<int32_t> cptr, cidx;  // column j's rows (positions), ascending
    int T = 0;
    double cost = 0.0;
  };
  // cptr / cidx: column structures by elimination position, unsorted
  auto make_candidate = [&](std::vector<int32_t>&& perm, std::vector<int32_t>&& cptr, std::vector<int32_t>&& cidx) {
    Candidate c;
    c.perm = std::move(perm);
    c.pos.assign(N, 0);
    for (int j = 0; j < N; ++j) c.pos[c.perm[j]] = j;
    c.cptr = std::move(cptr);
    c.cidx = std::move(cidx);
    for (int j = 0; j < N; ++j) std::sort(c.cidx.begin() + c.cptr[j], c.cidx.begin() + c.cptr[j + 1]);
    auto size = [&](int j) { return c.cptr[j + 1] - c.cptr[j]; };
    // dense tail: the trailing columns whose structure is complete
    while (dense_tail && c.T < N && size(N - 1 - c.T) == c.T) ++c.T;
    const int ns = N - c.T;
    std::vector<int32_t> lvl(ns, 0);
    int L = 0;
    double pairs = 0.0;
    for (int j = 0; j < ns; ++j) {
      L = std::max(L, lvl[j] + 1);
      if (size(j) > 0 && c.cidx[c.cptr[j]] < ns) lvl[c.cidx[c.cptr[j]]] = std::max(lvl[c.cidx[c.cptr[j]]], lvl[j] + 1);
      const double m = (double)size(j);
      pairs += m * (m + 1) / 2;
    }
    const double nt = (double)c.T * d, dd3 = (double)d * d * d;
    const double tiles = std::ceil(nt / p.tile);
    const double flops = 2.0 * dd3 * pairs + nt * nt * nt / 3.0;
    c.cost = (3.0 * L + 2.0 * tiles + 4.0) * kPhaseUs + flops * kUsPerFlop;
    return c;
  };
  // the three candidates are independent: minimum degree and the second
  // nested-dissection order run on their own threads
  std::vector<Candidate> cands(3);
  std::exception_ptr err[2];
  std::thread t_md([&] {
    try {
      std::vector<std::vector<int32_t>> a = adj, col_vars;
      std::vector<int32_t> perm;
      order_variables(N, a, &perm, &col_vars);
      std::vector<int32_t> pos(N), cptr(N + 1, 0), cidx;
      for (int j = 0; j < N; ++j) pos[perm[j]] = j;
      for (int j = 0; j < N; ++j) cptr[j + 1] = cptr[j] + (int32_t)col_vars[perm[j]].size();
      cidx.reserve(cptr[N]);
      for (int j = 0; j < N; ++j)
        for (int v : col_vars[perm[j]]) cidx.push_back(pos[v]);
      cands[0] = make_candidate(std::move(perm), std::move(cptr), std::move(cidx));
    } catch (...) {
      err[0] = std::current_exception();
    }
  });
  {
    // nested dissection with leaves of 4 and of 32 variables
    NestedDissection nd(adj, 4, 32);
    std::vector<int32_t> all(N);
    for (int u = 0; u < N; ++u) all[u] = u;
    try {
      nd.run(std::move(all), true);
    } catch (...) {
      t_md.join();
      throw;
    }
    std::thread t_nd([&] {
      try {
        std::vector<int32_t> cptr, cidx;
        eliminate_in_order(adj, nd.out2, &cptr, &cidx);
        cands[2] = make_candidate(std::move(nd.out2), std::move(cptr), std::move(cidx));
      } catch (...) {
        err[1] = std::current_exception();
      }
    });
    try {
      std::vector<int32_t> cptr, cidx;
      eliminate_in_order(adj, nd.out, &cptr, &cidx);
      cands[1] = make_candidate(std::move(nd.out), std::move(cptr), std::move(cidx));
    } catch (...) {
      t_nd.join();
      t_md.join();
      throw;
    }
    t_nd.join();
  }
  t_md.join();
  for (auto& e : err)
    if (e) std::rethrow_exception(e);
  size_t best = 0;
  for (size_t c = 1; c < cands.size(); ++c)
    if (cands[c].cost < cands[best].cost) best = c;
  p.perm = std::move(cands[best].perm);
  p.pos = std::move(cands[best].pos);
  const std::vector<int32_t> cptr = std::move(cands[best].cptr), cidx = std::move(cands[best].cidx);
  const int T = cands[best].T;
  p.T = T;
  p.n_sparse = N - T;
  const int ns = p.n_sparse;
  p.n_tiles = (T * d + p.tile - 1) / p.tile;

  // sparse blocks
  p.col_ptr.assign(ns + 1, 0);
  for (int j = 0; j < ns; ++j) p.col_ptr[j + 1] = p.col_ptr[j] + 1 + (cptr[j + 1] - cptr[j]);
  p.blk_row.resize(p.col_ptr[ns]);
  p.blk_col.resize(p.col_ptr[ns]);
  for (int j = 0; j < ns; ++j) {
    int q = p.col_ptr[j];
    p.blk_row[q] = j;
    p.blk_col[q] = j;
    for (int e = cptr[j]; e < cptr[j + 1]; ++e) {
      const int r = cidx[e];
      ++q;
      p.blk_row[q] = r;
      p.blk_col[q] = j;
    }
  }
  // elimination-tree levels of the sparse columns
  std::vector<int32_t> lvl(ns, 0);
  int L = 0;
  for (int j = 0; j < ns; ++j) {
    L = std::max(L, lvl[j] + 1);
    if (cptr[j + 1] > cptr[j] && cidx[cptr[j]] < ns) lvl[cidx[cptr[j]]] = std::max(lvl[cidx[cptr[j]]], lvl[j] + 1);
  }
  p.lvl_col_ptr.assign(L + 1, 0);
  for (int j = 0; j < ns; ++j) p.lvl_col_ptr[lvl[j] + 1] += 1;
  for (int l = 0; l < L; ++l) p.lvl_col_ptr[l + 1] += p.lvl_col_ptr[l];
  p.lvl_cols.resize(ns);
  {
    std::vector<int32_t> cc(p.lvl_col_ptr.begin(), p.lvl_col_ptr.end() - 1);
    for (int j = 0; j < ns; ++j) p.lvl_cols[cc[lvl[j]]++] = j;
    // each level's columns by descending block count (consecutive columns go
    // to the lane groups of one warp on wide levels: similar loops); columns
    // of a level are independent, so the order changes no result
    for (int l = 0; l < L; ++l)
      std::stable_sort(p.lvl_cols.begin() + p.lvl_col_ptr[l], p.lvl_cols.begin() + p.lvl_col_ptr[l + 1],
                       [&](int32_t a, int32_t b) {
                         return p.col_ptr[a + 1] - p.col_ptr[a] > p.col_ptr[b + 1] - p.col_ptr[b];
                       });
  }

  // updates: for each sparse column k and rows ra <= rb of it, target (rb, ra)
  // -= L(rb, k) L(ra, k)^T; lists are filled in ascending k
  const int nblk = p.n_blocks(), ntb = p.n_tail_blocks();
  p.upd_ptr.assign(nblk + 1, 0);
  p.tupd_ptr.assign(ntb + 1, 0);
  auto tail_index = [ns](int rb, int ra) {
    const int bi = rb - ns, bj = ra - ns;
    return bi * (bi + 1) / 2 + bj;
  };
  double pairs = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<int32_t> fill_s, fill_t;
    if (pass == 1) {
      for (int q = 0; q < nblk; ++q) p.upd_ptr[q + 1] += p.upd_ptr[q];
      for (int t = 0; t < ntb; ++t) p.tupd_ptr[t + 1] += p.tupd_ptr[t];
      p.upd_src.resize((size_t)2 * p.upd_ptr[nblk]);
      p.tupd_src.resize((size_t)2 * p.tupd_ptr[ntb]);
      fill_s.assign(p.upd_ptr.begin(), p.upd_ptr.end() - 1);
      fill_t.assign(p.tupd_ptr.begin(), p.tupd_ptr.end() - 1);
    }
    for (int k = 0; k < ns; ++k) {
      const int b0 = p.col_ptr[k] + 1, m = p.col_ptr[k + 1] - b0;
      for (int a = 0; a < m; ++a) {
        const int ra = p.blk_row[b0 + a];
        for (int b = a; b < m; ++b) {
          const int rb = p.blk_row[b0 + b];
          if (ra < ns) {
            const int tgt = find_block(p, ra, rb);
            if (pass == 0) {
              p.upd_ptr[tgt + 1]++;
            } else {
              const int s = fill_s[tgt]++;
              p.upd_src[2 * s] = b0 + b;
              p.upd_src[2 * s + 1] = b0 + a;
            }
          } else {
            const int tgt = tail_index(rb, ra);
            if (pass == 0) {
              p.tupd_ptr[tgt + 1]++;
            } else {
              const int s = fill_t[tgt]++;
              p.tupd_src[2 * s] = b0 + b;
              p.tupd_src[2 * s + 1] = b0 + a;
            }
          }
          if (pass == 0) pairs += 1.0;
        }
      }
    }
  }

  // Hessian off-diagonal blocks per target
  p.a_ptr.assign(nblk + 1, 0);
  p.ta_ptr.assign(ntb + 1, 0);
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<int32_t> fill_s, fill_t;
    if (pass == 1) {
      for (int q = 0; q < nblk; ++q) p.a_ptr[q + 1] += p.a_ptr[q];
      for (int t = 0; t < ntb; ++t) p.ta_ptr[t + 1] += p.ta_ptr[t];
      p.a_src.resize(p.a_ptr[nblk]);
      p.ta_src.resize(p.ta_ptr[ntb]);
      fill_s.assign(p.a_ptr.begin(), p.a_ptr.end() - 1);
      fill_t.assign(p.ta_ptr.begin(), p.ta_ptr.end() - 1);
    }
    for (size_t f = 0; f < F; ++f) {
      if (kind[f] != 0 || vi[f] == vj[f]) continue;
      const int pi = p.pos[vi[f]], pj = p.pos[vj[f]];
      const int r = std::max(pi, pj), c = std::min(pi, pj);
      const int32_t src = (int32_t)(2 * f + (pi == r ? 0 : 1));
      if (c < ns) {
        const int tgt = find_block(p, c, r);
        if (pass == 0) p.a_ptr[tgt + 1]++;
        else p.a_src[fill_s[tgt]++] = src;
      } else {
        const int tgt = tail_index(r, c);
        if (pass == 0) p.ta_ptr[tgt + 1]++;
        else p.ta_src[fill_t[tgt]++] = src;
      }
    }
  }

  // row lists for the forward solve
  p.row_ptr.assign(ns + 1, 0);
  p.trow_ptr.assign(T + 1, 0);
  for (int q = 0; q < nblk; ++q) {
    const int r = p.blk_row[q];
    if (r == p.blk_col[q]) continue;
    if (r < ns) p.row_ptr[r + 1]++;
    else p.trow_ptr[r - ns + 1]++;
  }
  for (int j = 0; j < ns; ++j) p.row_ptr[j + 1] += p.row_ptr[j];
  for (int t = 0; t < T; ++t) p.trow_ptr[t + 1] += p.trow_ptr[t];
  p.row_blk.resize((size_t)2 * p.row_ptr[ns]);
  p.trow_blk.resize((size_t)2 * p.trow_ptr[T]);
  {
    std::vector<int32_t> fr(p.row_ptr.begin(), p.row_ptr.end() - 1), ft(p.trow_ptr.begin(), p.trow_ptr.end() - 1);
    for (int q = 0; q < nblk; ++q) {
      const int r = p.blk_row[q];
      if (r == p.blk_col[q]) continue;
      if (r < ns) {
        const int u = fr[r]++;
        p.row_blk[2 * u] = q;
        p.row_blk[2 * u + 1] = p.blk_col[q];
      } else {
        const int u = ft[r - ns]++;
        p.trow_blk[2 * u] = q;
        p.trow_blk[2 * u + 1] = p.blk_col[q];
      }
    }
  }
  // tasks, level by level: every block of a level's columns (its Hessian
  // block and update chunks), then the row sums of the level's columns
  p.chunk = 32 / d;
  p.row_chunk = 4 * (32 / d);
  p.lvl_task_ptr.assign(L + 1, 0);
  p.btask.assign((size_t)2 * nblk, 0);
  p.ftask.assign((size_t)2 * ns, 0);
  p.tasks.clear();
  {
    const int halves = d == 6 ? 2 : 1;
    {
      size_t n = 0;  // tasks, for the reservation
      for (int q = 0; q < nblk; ++q) n += (size_t)halves * ((p.upd_ptr[q + 1] - p.upd_ptr[q] + p.chunk - 1) / p.chunk);
      for (int j = 0; j < ns; ++j) n += (size_t)((p.row_ptr[j + 1] - p.row_ptr[j] + p.row_chunk - 1) / p.row_chunk);
      p.tasks.reserve(4 * n);
    }
    std::vector<int32_t> lt;
    int slot = 0;
    for (int l = 0; l < L; ++l) {
      for (int w = p.lvl_col_ptr[l]; w < p.lvl_col_ptr[l + 1]; ++w) {
        const int j = p.lvl_cols[w];
        for (int q = p.col_ptr[j]; q < p.col_ptr[j + 1]; ++q) {
          p.btask[2 * q] = slot;
          // blocks without update pairs (every block of the leaves, which
          // also have no row sums) get no task: the column's own phase reads
          // their Hessian blocks directly, and the leaves' level has no task
          // phase
          if (l == 0 || p.upd_ptr[q] == p.upd_ptr[q + 1]) continue;
          int u = p.upd_ptr[q];
          do {
            const int e = std::min(u + p.chunk, p.upd_ptr[q + 1]);
            const int kind = u == p.upd_ptr[q] ? 1 : 0;
            const int diag = q == p.col_ptr[j] ? 1 : 0;
            for (int h = 0; h < halves; ++h)
              p.tasks.insert(p.tasks.end(), {q, u, e, kind | h << 2 | diag << 3 | slot << 4});
            ++slot;
            u = e;
          } while (u < p.upd_ptr[q + 1]);
          p.btask[2 * q + 1] = slot - p.btask[2 * q];
        }
        p.ftask[2 * j] = slot;
        for (int u = p.row_ptr[j]; u < p.row_ptr[j + 1]; u += p.row_chunk) {
          p.tasks.insert(p.tasks.end(), {j, u, std::min(u + p.row_chunk, p.row_ptr[j + 1]), 2 | slot << 4});
          ++slot;
        }
        p.ftask[2 * j + 1] = slot - p.ftask[2 * j];
      }
      // the level's tasks by descending work (a block chunk's pairs weigh
      // three row entries; the Hessian block of a first chunk one more), so
      // that the lane groups of a warp, which take consecutive tasks on wide
      // levels, get similar loops; the order of independent tasks changes no
      // result
      // (a stable counting sort: the weights are small integers)
      const int t0 = p.lvl_task_ptr[l], t1 = (int)p.tasks.size() / 4;
      auto work = [&](int t) {
        const int kind = p.tasks[4 * t + 3] & 3, n = p.tasks[4 * t + 2] - p.tasks[4 * t + 1];
        return kind == 2 ? n : 3 * n + (kind == 1 ? 1 : 0);
      };
      int wmax = 0;
      for (int t = t0; t < t1; ++t) wmax = std::max(wmax, work(t));
      std::vector<int32_t> at((size_t)wmax + 2, 0);  // at[wmax - w + 1]: tasks of weight w
      for (int t = t0; t < t1; ++t) at[(size_t)(wmax - work(t)) + 1]++;
      for (int w = 1; w <= wmax + 1; ++w) at[w] += at[w - 1];
      lt.assign(p.tasks.begin() + 4 * (size_t)t0, p.tasks.begin() + 4 * (size_t)t1);
      for (int t = 0; t < t1 - t0; ++t) {
        const int x = lt[4 * t + 3] & 3, n = lt[4 * t + 2] - lt[4 * t + 1];
        const int w = x == 2 ? n : 3 * n + (x == 1 ? 1 : 0);
        const int dst = t0 + at[wmax - w]++;
        for (int k = 0; k < 4; ++k) p.tasks[4 * (size_t)dst + k] = lt[4 * t + k];
      }
      p.lvl_task_ptr[l + 1] = t1;
    }
    p.n_slots = slot;
  }
  p.ttask_ptr.assign(T + 1, 0);
  p.ttasks.clear();
  for (int t = 0; t < T; ++t) {
    for (int u = p.trow_ptr[t]; u < p.trow_ptr[t + 1]; u += p.row_chunk)
      p.ttasks.insert(p.ttasks.end(), {t, u, std::min(u + p.row_chunk, p.trow_ptr[t + 1])});
    p.ttask_ptr[t + 1] = (int)p.ttasks.size() / 3;
  }
  const double dd3 = (double)d * d * d, nt = (double)T * d;
  p.flops = 2.0 * dd3 * pairs + ns * dd3 / 3.0 + (nblk - ns) * dd3 + nt * nt * nt / 3.0;
  {
    const double dd = (double)d * d, nA = (double)p.a_src.size() + p.ta_src.size();
    const double factor = 8.0 * dd * (nblk + ns) + 8.0 * nt * (nt + 1) / 2.0;  // L (+ diagonal factors)
    p.bytes = 8.0 * dd * (N + nA)   // Hessian diagonal and off-diagonal blocks
              + 2.0 * factor        // factor written, then read by its updates
              + 2.0 * factor        // read by the forward and the backward substitution
              + 8.0 * d * N * 6.0;  // gradient, damping, rhs / solution, step, model change
  }
  return p;
}

CholPlan merge_chol_plans(const std::vector<CholPlan>& plans, const std::vector<int32_t>& foff) {
  CholPlan u;
  const int G = (int)plans.size();
  if (G == 0) return u;
  u.d = plans[0].d;
  u.tile = plans[0].tile;
  u.chunk = plans[0].chunk;
  u.row_chunk = plans[0].row_chunk;
  int L = 0;
  for (const CholPlan& p : plans) {
    if (p.T != 0 || p.d != u.d || p.chunk != u.chunk || p.row_chunk != u.row_chunk)
      throw std::logic_error("merge_chol_plans: plans with dense tails or different block sizes");
    L = std::max(L, p.levels());
    u.N += p.N;
    u.flops += p.flops;
    u.bytes += p.bytes;
  }
  u.n_sparse = u.N;
  u.T = 0;
  u.n_tiles = 0;
  // offsets of each plan's positions, blocks, slots, update pairs, Hessian
  // sources and row entries in the merged arrays
  std::vector<int32_t> voff(G + 1, 0), boff(G + 1, 0), soff(G + 1, 0), uoff(G + 1, 0), aoff(G + 1, 0),
      roff(G + 1, 0);
  for (int g = 0; g < G; ++g) {
    const CholPlan& p = plans[g];
    voff[g + 1] = voff[g] + p.N;
    boff[g + 1] = boff[g] + p.n_blocks();
    soff[g + 1] = soff[g] + p.n_slots;
    uoff[g + 1] = uoff[g] + p.upd_ptr.back();
    aoff[g + 1] = aoff[g] + p.a_ptr.back();
    roff[g + 1] = roff[g] + p.row_ptr.back();
  }
  u.n_slots = soff[G];
  const int nb = boff[G];
  u.perm.resize(u.N);
  u.pos.resize(u.N);
  u.col_ptr.assign(u.N + 1, 0);
  u.blk_row.resize(nb);
  u.blk_col.resize(nb);
  u.upd_ptr.assign(nb + 1, 0);
  u.upd_src.resize((size_t)2 * uoff[G]);
  u.a_ptr.assign(nb + 1, 0);
  u.a_src.resize(aoff[G]);
  u.row_ptr.assign(u.N + 1, 0);
  u.row_blk.resize((size_t)2 * roff[G]);
  u.btask.resize((size_t)2 * nb);
  u.ftask.resize((size_t)2 * u.N);
  for (int g = 0; g < G; ++g) {
    const CholPlan& p = plans[g];
    const int v0 = voff[g], b0 = boff[g], s0 = soff[g], u0 = uoff[g], a0 = aoff[g], r0 = roff[g];
    for (int j = 0; j < p.N; ++j) {
      u.perm[v0 + j] = p.perm[j] + v0;
      u.pos[v0 + j] = p.pos[j] + v0;
      u.col_ptr[v0 + j + 1] = p.col_ptr[j + 1] + b0;
      u.row_ptr[v0 + j + 1] = p.row_ptr[j + 1] + r0;
      u.ftask[2 * (v0 + j)] = p.ftask[2 * j] + s0;
      u.ftask[2 * (v0 + j) + 1] = p.ftask[2 * j + 1];
    }
    for (int q = 0; q < p.n_blocks(); ++q) {
      u.blk_row[b0 + q] = p.blk_row[q] + v0;
      u.blk_col[b0 + q] = p.blk_col[q] + v0;
      u.upd_ptr[b0 + q + 1] = p.upd_ptr[q + 1] + u0;
      u.a_ptr[b0 + q + 1] = p.a_ptr[q + 1] + a0;
      u.btask[2 * (b0 + q)] = p.btask[2 * q] + s0;
      u.btask[2 * (b0 + q) + 1] = p.btask[2 * q + 1];
    }
    for (size_t k = 0; k < p.upd_src.size(); ++k) u.upd_src[(size_t)2 * u0 + k] = p.upd_src[k] + b0;
    // Hessian sources 2 f + transposed: factor f of plan g is factor foff[g] + f
    for (size_t k = 0; k < p.a_src.size(); ++k) u.a_src[a0 + k] = p.a_src[k] + 2 * foff[g];
    for (size_t k = 0; k < p.row_blk.size(); k += 2) {
      u.row_blk[(size_t)2 * r0 + k] = p.row_blk[k] + b0;
      u.row_blk[(size_t)2 * r0 + k + 1] = p.row_blk[k + 1] + v0;
    }
  }
  // levels: every plan's level l, then the level's columns by descending
  // block count and its tasks by descending work (as make_chol_plan orders a
  // level; a stable counting sort, the keys being small); independent items,
  // so the order changes no result
  u.lvl_col_ptr.assign(L + 1, 0);
  u.lvl_task_ptr.assign(L + 1, 0);
  u.lvl_cols.reserve(u.N);
  std::vector<int32_t> cols_l, cnt;
  std::vector<std::array<int32_t, 4>> tasks_l;
  auto task_work = [](const std::array<int32_t, 4>& x) {
    const int kind = x[3] & 3, n = x[2] - x[1];
    return kind == 2 ? n : 3 * n + (kind == 1 ? 1 : 0);
  };
  for (int l = 0; l < L; ++l) {
    cols_l.clear();
    tasks_l.clear();
    for (int g = 0; g < G; ++g) {
      const CholPlan& p = plans[g];
      if (l >= p.levels()) continue;
      const int v0 = voff[g], b0 = boff[g], s0 = soff[g], u0 = uoff[g], r0 = roff[g];
      for (int w = p.lvl_col_ptr[l]; w < p.lvl_col_ptr[l + 1]; ++w) cols_l.push_back(p.lvl_cols[w] + v0);
      for (int t = p.lvl_task_ptr[l]; t < p.lvl_task_ptr[l + 1]; ++t) {
        const int32_t* tk = &p.tasks[4 * (size_t)t];
        const int kind = tk[3] & 3, low = tk[3] & 15, slot = tk[3] >> 4;
        if (kind < 2) tasks_l.push_back({tk[0] + b0, tk[1] + u0, tk[2] + u0, low | (slot + s0) << 4});
        else tasks_l.push_back({tk[0] + v0, tk[1] + r0, tk[2] + r0, low | (slot + s0) << 4});
      }
    }
    // columns by descending block count
    int kmax = 0;
    for (int32_t c : cols_l) kmax = std::max(kmax, u.col_ptr[c + 1] - u.col_ptr[c]);
    cnt.assign(kmax + 2, 0);
    for (int32_t c : cols_l) cnt[kmax - (u.col_ptr[c + 1] - u.col_ptr[c]) + 1]++;
    for (int k = 1; k <= kmax + 1; ++k) cnt[k] += cnt[k - 1];
    const size_t c_begin = u.lvl_cols.size();
    u.lvl_cols.resize(c_begin + cols_l.size());
    for (int32_t c : cols_l) u.lvl_cols[c_begin + cnt[kmax - (u.col_ptr[c + 1] - u.col_ptr[c])]++] = c;
    // tasks by descending work
    int wmax = 0;
    for (const auto& x : tasks_l) wmax = std::max(wmax, task_work(x));
    cnt.assign(wmax + 2, 0);
    for (const auto& x : tasks_l) cnt[wmax - task_work(x) + 1]++;
    for (int k = 1; k <= wmax + 1; ++k) cnt[k] += cnt[k - 1];
    const size_t t_begin = u.tasks.size() / 4;
    u.tasks.resize(u.tasks.size() + 4 * tasks_l.size());
    for (const auto& x : tasks_l) {
      const size_t t = t_begin + cnt[wmax - task_work(x)]++;
      for (int k = 0; k < 4; ++k) u.tasks[4 * t + k] = x[k];
    }
    u.lvl_col_ptr[l + 1] = (int32_t)u.lvl_cols.size();
    u.lvl_task_ptr[l + 1] = (int32_t)(u.tasks.size() / 4);
  }
  u.tupd_ptr.assign(1, 0);
  u.ta_ptr.assign(1, 0);
  u.trow_ptr.assign(1, 0);
  u.ttask_ptr.assign(1, 0);
  return u;
}

}  // namespace rpgo

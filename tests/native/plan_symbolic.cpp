// Test harness (CPU): compiles the plan builder in this translation unit to
// reach its internal helpers, and compares the elimination-tree symbolic
// analysis of a given order with the elimination game (the neighbours of each
// variable when it is eliminated). Loaded by tests/test_plan_symbolic_cpu.py.
#include "../../kimera-rpgo_gb300/csrc/chol_plan.cpp"

#include <algorithm>
#include <cstdint>
#include <vector>

extern "C" {

// n variables, m edges (ei[k], ej[k]), elimination order `order` (a
// permutation of 0..n-1). Returns 0 when every column's structure agrees (as
// sets of variables), else 1 + the first differing position.
int plan_symbolic_check(int n, int m, const int32_t* ei, const int32_t* ej, const int32_t* order) {
  std::vector<std::vector<int32_t>> adj((size_t)n);
  for (int k = 0; k < m; ++k)
    if (ei[k] != ej[k]) {
      adj[ei[k]].push_back(ej[k]);
      adj[ej[k]].push_back(ei[k]);
    }
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  const std::vector<int32_t> ord(order, order + n);
  std::vector<int32_t> ptr, idx;
  rpgo::eliminate_in_order(adj, ord, &ptr, &idx);
  std::vector<std::vector<int32_t>> game_adj = adj;
  rpgo::Elimination el(game_adj);
  for (int u : ord) el.eliminate(u, [](int) {});
  for (int j = 0; j < n; ++j) {
    std::vector<int32_t> a, b = el.col_vars[ord[j]];
    for (int q = ptr[j]; q < ptr[j + 1]; ++q) a.push_back(ord[idx[q]]);
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    if (a != b) return 1 + j;
  }
  return 0;
}

// Plan of n variables of dimension d over the given edges (and a prior on
// variable 0): writes the number of levels to *levels and returns 0 when the
// tasks of every level are in non-increasing order of weight (a block chunk's
// pairs weigh three row entries, the Hessian block of a first chunk one more)
// and every slot appears in exactly one level's tasks, else 1.
int plan_task_order_check(int n, int d, int m, const int32_t* ei, const int32_t* ej, int* levels) {
  std::vector<int32_t> kind, vi, vj;
  for (int k = 0; k < m; ++k) {
    kind.push_back(0);
    vi.push_back(ei[k]);
    vj.push_back(ej[k]);
  }
  kind.push_back(1);
  vi.push_back(0);
  vj.push_back(0);
  const rpgo::CholPlan p = rpgo::make_chol_plan(n, d, kind, vi, vj);
  *levels = (int)p.lvl_task_ptr.size() - 1;
  std::vector<int> seen((size_t)p.n_slots, 0);
  for (int l = 0; l + 1 < (int)p.lvl_task_ptr.size(); ++l) {
    int prev = 1 << 30;
    for (int t = p.lvl_task_ptr[l]; t < p.lvl_task_ptr[l + 1]; ++t) {
      const int kd = p.tasks[4 * t + 3] & 3, cnt = p.tasks[4 * t + 2] - p.tasks[4 * t + 1];
      const int w = kd == 2 ? cnt : 3 * cnt + (kd == 1 ? 1 : 0);
      if (w > prev) return 1;
      prev = w;
      const int slot = p.tasks[4 * t + 3] >> 4;
      if (slot < 0 || slot >= p.n_slots) return 1;
      seen[slot]++;
    }
  }
  const int halves = d == 6 ? 2 : 1;
  for (int slot = 0; slot < p.n_slots; ++slot) {
    // a block chunk's slot appears once per half, a row chunk's once
    if (seen[slot] != halves && seen[slot] != 1) return 1;
  }
  return 0;
}
}

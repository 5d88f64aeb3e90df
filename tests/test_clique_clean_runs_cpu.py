"""The clique kernel's clean-run batches (clique_kernels.cu) take the same
rounds as the reference's greedy walk (findCliqueHeu.cpp:32-209, as the
oracle restates it): a walk from candidate v keeps [v] + B, every round takes
m = max(B) and keeps B & N(m); a round whose m is adjacent to every element
of B below it only removes m, so up to 32 such rounds are checked on the
rows of B's highest elements and the leading clean run is committed at once.
Both forms are restated here in plain Python on random graphs with planted
cliques and compared: the same score (rounds + 1, or the early stop when
rounds + |B| + 1 <= best) and the same work buffer, stale slots included.
No GPU."""
import random

import numpy as np
import pytest


def _walk_plain(adj, v, best, deg):
    n = len(adj)
    B = [u for u in range(n) if adj[v][u] and u != v and deg[u] >= best]
    buf = [-7] * (n + 1)
    buf[0] = v
    r = 0
    while True:
        if not B:
            return r + 1, buf
        if r + len(B) + 1 <= best:
            return -2, buf
        m = B[-1]
        nxt = [u for u in B if adj[m][u] and u != m]
        # slots (|B'|, |B|] <- the |B| - |B'| largest elements of B, ascending
        need = len(B) - len(nxt)
        for i, u in enumerate(B[len(B) - need:]):
            buf[len(nxt) + 1 + i] = u
        B = nxt
        r += 1


def _walk_clean_runs(adj, v, best, deg, batch=32):
    n = len(adj)
    B = [u for u in range(n) if adj[v][u] and u != v and deg[u] >= best]
    buf = [-7] * (n + 1)
    buf[0] = v
    r, try_at, misses = 0, 0, 0
    while True:
        if not B:
            return r + 1, buf
        if r + len(B) + 1 <= best:
            return -2, buf
        if r >= try_at:
            top = B[::-1][:batch]
            k = 0
            for u in top:  # u clean: every element of B below u is a neighbour
                if all(adj[u][x] for x in B if x < u):
                    k += 1
                else:
                    break
            if k:
                for l in range(k):  # round l removes top[l]: slot |B| - l
                    buf[len(B) - l] = top[l]
                B = [x for x in B if x < top[k - 1]]
                r += k
                misses = 0
                try_at = r + 1 if k < len(top) else r
                continue
            misses = min(misses + 1, 6)
            try_at = r + (1 << misses)
        m = B[-1]
        nxt = [u for u in B if adj[m][u] and u != m]
        need = len(B) - len(nxt)
        for i, u in enumerate(B[len(B) - need:]):
            buf[len(nxt) + 1 + i] = u
        B = nxt
        r += 1


@pytest.mark.parametrize("seed", range(4))
def test_clean_run_batches_take_the_same_rounds(seed):
    rng = random.Random(seed)
    for _ in range(40):
        n = rng.randint(5, 90)
        p = rng.choice([0.1, 0.5, 0.9, 0.97])
        A = np.zeros((n, n), bool)
        for i in range(n):
            for j in range(i + 1, n):
                if rng.random() < p:
                    A[i, j] = A[j, i] = True
        S = rng.sample(range(n), rng.randint(0, n))
        for i in S:
            for j in S:
                if i != j:
                    A[i, j] = True
        deg = A.sum(1)
        best = rng.choice([0, 3, int(deg.max() // 2)])
        for v in range(n):
            if deg[v] < best:
                continue
            a = _walk_plain(A, v, best, deg)
            b = _walk_clean_runs(A, v, best, deg, batch=rng.choice([1, 4, 32]))
            assert a[0] == b[0]
            if a[0] > 0:
                assert a[1] == b[1]

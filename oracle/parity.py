"""GPU result against the CPU FP64 oracle — TEST INFRASTRUCTURE ONLY.

Used by tests/ and by bench.py's CPU-baseline leg as the checker; the
product path never imports it. `check(graph, params, gpu)` compares one
`rpgo_update` of `graph` on the GPU (a `capi.RobustSolver` after the update)
with the oracle, stage by stage, so that every stage is checked at sizes
where the oracle's own end-to-end run is too slow:

  * consistency matrix (Pcm.h:725-768): the oracle's whole matrix
    (`rows=None`), or a seeded sample of whole rows, against the GPU's bits;
  * greedy clique (findCliqueHeu.cpp:32-117): the oracle's clique of the
    GPU's matrix against the closures the GPU kept, in the same order;
  * solve (RobustSolver.cpp:115-306): the oracle's GNC-TLS / LM over the
    GPU's filtered factor list (known inliers = odometry + priors) against
    the GPU's GNC weights and estimate.

With bit-equal matrices the chain is the oracle's whole update; bit
equality of the sampled rows is the evidence for the rest of the matrix.
"""
from __future__ import annotations

import time

import numpy as np

from . import rpgo_oracle as O


def _ate(a, b, dim):
    if dim == 3:
        d = a[:, 9:12] - b[:, 9:12]
    else:
        d = a[:, 2:4] - b[:, 2:4]
    return float(np.sqrt(np.mean(np.sum(d * d, axis=1)))) if len(d) else 0.0


def _max_rel(a, b):
    if not len(a):
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b))))


def check(graph, params, gpu, rows=256, seed=0, solve=True, threads=0, keep=False):
    """Stage-by-stage comparison of a GPU update of `graph` with the oracle.

    rows: None for the oracle's whole consistency matrix, else the number of
    seeded whole rows to evaluate (single-group graphs). Returns a dict of
    booleans, errors and the oracle's wall time per stage (with keep, also
    the oracle solver of the solve stage under "_oracle")."""
    before_impl = O.set_clique_impl(2)
    before_thr = O.set_threads(0)
    if threads:
        O.set_threads(threads)
    out = {}
    try:
        dim = 3 if graph.dim == 3 else 2
        t0 = time.perf_counter()
        n, src, _ = O.OracleSolver(params).pcm_rows(graph, [])
        A = gpu.adjacency(0)
        gn = 0 if A is None else A.shape[0]
        out["closures_checked"] = int(n)
        if rows is None or rows >= n:
            sel = np.arange(n, dtype=np.int32)
        else:
            sel = np.sort(np.random.default_rng(seed).choice(n, int(rows), replace=False)).astype(np.int32)
        _, _, bits = O.OracleSolver(params).pcm_rows(graph, sel)
        out["adjacency_rows_checked"] = int(len(sel))
        out["adjacency_bit_exact"] = bool(gn == n and (n == 0 or np.array_equal(bits, A[sel])))
        out["oracle_rows_s"] = time.perf_counter() - t0
        # greedy clique of the GPU's matrix on the oracle
        t0 = time.perf_counter()
        c = gpu.counts()
        n_known = int(c.num_odom + c.num_special)
        kind, k1, k2, _ = gpu.factors()
        if n:
            size, idx = O.max_clique_heu(A, n)
            kept = [int(src[i]) for i in idx[:size] if i < n]
        else:
            kept = []
        exp = np.array([[graph.kind[j], graph.key1[j], graph.key2[j]] for j in kept], dtype=np.uint64).reshape(-1, 3)
        got = np.stack([kind[n_known:].astype(np.uint64), k1[n_known:], k2[n_known:]], axis=1)
        out["clique_equal"] = bool(exp.shape == got.shape and np.array_equal(exp, got))
        out["clique_size"] = int(len(kept))
        out["oracle_clique_s"] = time.perf_counter() - t0
        if solve:
            t0 = time.perf_counter()
            fg = O.filtered_graph(graph, kind, k1, k2)
            o = O.OracleSolver(params)
            rc = o.solve_graph(fg, n_known)
            out["oracle_solve_rc"] = int(rc)
            wo, wg = o.gnc_weights(), gpu.gnc_weights()
            out["inlier_set_identical"] = bool(len(wo) == len(wg) and np.array_equal(np.round(wo), np.round(wg)))
            ko, po = o.estimate()
            kg, pg = gpu.estimate()
            same_keys = bool(np.array_equal(ko, kg))
            out["ate_vs_oracle_m"] = _ate(pg, po, dim) if same_keys else None
            out["max_rel_pose_err"] = _max_rel(pg, po) if same_keys else None
            st = o.stats()
            out["oracle_solves"] = int(st["linear_solves"])
            out["oracle_gnc_iterations"] = int(st["gnc_iterations"])
            out["oracle_solve_s"] = time.perf_counter() - t0
            if keep:
                out["_oracle"] = o
    finally:
        O.set_clique_impl(before_impl)
        O.set_threads(before_thr)
    return out


def passed(report, ate_tol=1e-4, rel_tol=1e-6):
    """True when every check of `report` holds."""
    ok = report["adjacency_bit_exact"] and report["clique_equal"]
    if "inlier_set_identical" in report:
        ok = ok and report["oracle_solve_rc"] == 0 and report["inlier_set_identical"]
        ok = ok and report["ate_vs_oracle_m"] is not None and report["ate_vs_oracle_m"] <= ate_tol
        ok = ok and report["max_rel_pose_err"] <= rel_tol
    return bool(ok)

"""ctypes front-end of the CPU FP64 oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check and bench.py's CPU-baseline leg load this
module; the product path never does. The shared library is built from
oracle/*.cpp by oracle/Makefile into oracle/_build/liboracle.so.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


class Params(C.Structure):
    _fields_ = [
        ("solver", C.c_int32), ("outlier_removal", C.c_int32), ("verbosity", C.c_int32), ("dim", C.c_int32),
        ("odom_threshold", C.c_double), ("lc_threshold", C.c_double),
        ("odom_trans_threshold", C.c_double), ("odom_rot_threshold", C.c_double),
        ("dist_trans_threshold", C.c_double), ("dist_rot_threshold", C.c_double),
        ("incremental", C.c_int32),
        ("use_gnc", C.c_int32), ("gnc_threshold_mode", C.c_int32), ("gnc_inlier_threshold", C.c_double),
        ("gnc_max_iterations", C.c_int32), ("gnc_mu_step", C.c_double), ("gnc_relative_cost_tol", C.c_double),
        ("gnc_weights_tol", C.c_double), ("gnc_fix_prev_inliers", C.c_int32), ("gnc_bias_odom", C.c_int32),
        ("lm_diagonal_damping", C.c_int32), ("linear_solver", C.c_int32),
        ("gnc_warm_start", C.c_int32), ("gnc_warm_mu", C.c_double),
        ("num_special_symbols", C.c_int32), ("special_symbols", C.c_char * 16),
        ("multirobot_align_method", C.c_int32), ("multirobot_align_gnc_prob", C.c_double),
    ]


class FactorBatch(C.Structure):
    _fields_ = [("count", C.c_int64), ("kind", C.c_void_p), ("key_front", C.c_void_p), ("key_back", C.c_void_p),
                ("measured", C.c_void_p), ("covariance", C.c_void_p), ("sqrt_information", C.c_void_p)]


class ValueBatch(C.Structure):
    _fields_ = [("count", C.c_int64), ("key", C.c_void_p), ("pose", C.c_void_p)]


class Counts(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("num_factors", "num_values", "num_lc", "num_lc_inliers", "num_odom",
                                          "num_special", "num_gnc_weights", "last_do_optimize")]


def build(force: bool = False) -> str:
    # make rebuilds only when a source is newer than the library
    subprocess.check_call(["make", "-s", "-C", _HERE] + (["-B"] if force else []))
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        _lib.oracle_create.restype = C.c_void_p
        _lib.oracle_create.argtypes = [C.POINTER(Params)]
        _lib.oracle_destroy.argtypes = [C.c_void_p]
        _lib.oracle_update.argtypes = [C.c_void_p, C.POINTER(FactorBatch), C.POINTER(ValueBatch), C.c_int32]
        _lib.oracle_get_counts.argtypes = [C.c_void_p, C.POINTER(Counts)]
        _lib.oracle_get_estimate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        _lib.oracle_get_gnc_weights.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        _lib.oracle_get_factors.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        _lib.oracle_get_adjacency.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64,
                                              C.POINTER(C.c_int64)]
        _lib.oracle_get_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                          C.POINTER(C.c_int64)]
        _lib.oracle_get_times.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.oracle_set_warm_probs.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        _lib.oracle_force_optimize.argtypes = [C.c_void_p]
        _lib.oracle_set_threads.argtypes = [C.c_int]
        _lib.oracle_set_temp.argtypes = [C.c_void_p, C.POINTER(FactorBatch), C.POINTER(ValueBatch), C.c_int]
        _lib.oracle_clear_temp.argtypes = [C.c_void_p]
        _lib.oracle_temp_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        _lib.oracle_temp_values.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        _lib.oracle_temp_weights.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
        _lib.oracle_remove_last_loop_closure.argtypes = [C.c_void_p, C.c_int, C.c_char, C.c_char,
                                                         C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                                         C.POINTER(C.c_int)]
        _lib.oracle_ignore_prefix.argtypes = [C.c_void_p, C.c_char, C.c_int]
        _lib.oracle_ignored_prefixes.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        _lib.oracle_remove_priors_with_prefix.argtypes = [C.c_void_p, C.c_char, C.c_int]
        _lib.oracle_get_warm_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        _lib.oracle_pwc_op.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]
        _lib.oracle_pwc_mahalanobis.restype = C.c_double
        _lib.oracle_pwc_mahalanobis.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        _lib.oracle_pwn_norms.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        _lib.oracle_logmap.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
        _lib.oracle_atan2.restype = C.c_double
        _lib.oracle_atan2.argtypes = [C.c_double, C.c_double]
        _lib.oracle_chi2inv.restype = C.c_double
        _lib.oracle_chi2inv.argtypes = [C.c_double, C.c_int]
        _lib.oracle_pairwise_adjacency.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 9 + [
            C.c_double, C.c_double, C.c_void_p]
        _lib.oracle_max_clique_heu.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        _lib.oracle_set_clique_impl.argtypes = [C.c_int]
        _lib.oracle_pcm_rows.argtypes = [C.c_void_p, C.POINTER(FactorBatch), C.POINTER(ValueBatch), C.c_void_p,
                                         C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.c_void_p,
                                         C.c_int64, C.c_int]
        _lib.oracle_clique_scan_ops.restype = C.c_double
        _lib.oracle_clique_scan_ops.argtypes = [C.c_int, C.c_void_p, C.c_int]
        _lib.oracle_set_lm_max_iterations.argtypes = [C.c_int]
        _lib.oracle_solve_graph.argtypes = [C.c_void_p, C.POINTER(FactorBatch), C.POINTER(ValueBatch), C.c_int64]
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


def params_struct(p) -> Params:
    """Accepts any object with the rpgo_params field names (e.g. the product's
    RobustSolverParams mirror)."""
    s = Params()
    for name, _ in Params._fields_:
        setattr(s, name, getattr(p, name))
    return s


class _Batch:
    def __init__(self, g):
        self.a = g.arrays()
        a = self.a
        self.f = FactorBatch(len(a["kind"]), _ptr(a["kind"]), _ptr(a["key1"]), _ptr(a["key2"]), _ptr(a["measured"]),
                             _ptr(a["cov"]), _ptr(a["sqrt_info"]))
        self.v = ValueBatch(len(a["value_keys"]), _ptr(a["value_keys"]), _ptr(a["value_poses"]))


class OracleSolver:
    """RobustSolver restated on the CPU (same call shape as the product)."""

    def __init__(self, params):
        self.dim = 2 if params.outlier_removal in (1, 3) or (params.outlier_removal == 0 and params.dim == 2) else 3
        self._p = params_struct(params)
        self.h = lib().oracle_create(C.byref(self._p))
        if not self.h:
            raise ValueError("bad parameters")

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def update(self, graph, optimize_graph: bool = True) -> int:
        b = _Batch(graph)
        return lib().oracle_update(self.h, C.byref(b.f), C.byref(b.v), int(optimize_graph))

    def counts(self) -> Counts:
        c = Counts()
        lib().oracle_get_counts(self.h, C.byref(c))
        return c

    def size(self) -> int:
        return self.counts().num_factors

    def estimate(self):
        n = self.counts().num_values
        st = 12 if self.dim == 3 else 4
        keys = np.zeros(n, dtype=np.uint64)
        poses = np.zeros((n, st))
        rc = lib().oracle_get_estimate(self.h, _ptr(keys), _ptr(poses), n)
        assert rc == 0
        return keys, poses

    def gnc_weights(self):
        n = self.counts().num_gnc_weights
        w = np.zeros(n)
        lib().oracle_get_gnc_weights(self.h, _ptr(w), n)
        return w

    def factors(self):
        n = self.counts().num_factors
        st = 12 if self.dim == 3 else 4
        kind = np.zeros(n, dtype=np.int32)
        k1 = np.zeros(n, dtype=np.uint64)
        k2 = np.zeros(n, dtype=np.uint64)
        meas = np.zeros((n, st))
        lib().oracle_get_factors(self.h, _ptr(kind), _ptr(k1), _ptr(k2), _ptr(meas), n)
        return kind, k1, k2, meas

    def adjacency(self, group: int = 0):
        n = C.c_int64(0)
        rc = lib().oracle_get_adjacency(self.h, group, None, 0, C.byref(n))
        if rc != 0:
            return None
        words = (n.value + 31) // 32
        out = np.zeros(n.value * words, dtype=np.uint32)
        lib().oracle_get_adjacency(self.h, group, _ptr(out), out.size, C.byref(n))
        return out.reshape(n.value, words)

    def stats(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        lib().oracle_get_stats(self.h, C.byref(a), C.byref(b), C.byref(c))
        p, s = C.c_double(), C.c_double()
        lib().oracle_get_times(self.h, C.byref(p), C.byref(s))
        wr, wf = C.c_int64(), C.c_int64()
        lib().oracle_get_warm_stats(self.h, C.byref(wr), C.byref(wf))
        return dict(lm_iterations=a.value, linear_solves=b.value, gnc_iterations=c.value, pcm_seconds=p.value,
                    solve_seconds=s.value, warm_runs=wr.value, warm_fallbacks=wf.value)

    # ---- edit API (src/RobustSolver.cpp:371-446)
    def removeLastLoopClosure(self, prefix_1=None, prefix_2=None):
        a, b, r = C.c_uint64(), C.c_uint64(), C.c_int()
        by_id = prefix_1 is not None
        rc = lib().oracle_remove_last_loop_closure(self.h, int(by_id), (prefix_1 or "\0").encode(),
                                                   (prefix_2 or "\0").encode(), C.byref(a), C.byref(b), C.byref(r))
        assert rc == 0, rc
        return (a.value, b.value) if r.value else None

    def ignorePrefix(self, prefix: str) -> int:
        return lib().oracle_ignore_prefix(self.h, prefix.encode(), 0)

    def revivePrefix(self, prefix: str) -> int:
        return lib().oracle_ignore_prefix(self.h, prefix.encode(), 1)

    def getIgnoredPrefixes(self):
        buf = C.create_string_buffer(64)
        n = lib().oracle_ignored_prefixes(self.h, buf, 64)
        return [chr(c) for c in buf.raw[:n]]

    def removePriorFactorsWithPrefix(self, prefix: str, optimize_graph: bool = True) -> int:
        return lib().oracle_remove_priors_with_prefix(self.h, prefix.encode(), int(optimize_graph))

    def force_optimize(self) -> int:
        """forceUpdate() with no new factors: re-run the solve."""
        return lib().oracle_force_optimize(self.h)

    # temporary factors and values (GenericSolver.h:46-65)
    def updateTempFactorsValues(self, graph) -> int:
        b = _Batch(graph)
        return lib().oracle_set_temp(self.h, C.byref(b.f), C.byref(b.v), 0)

    def replaceTempFactorsValues(self, graph) -> int:
        b = _Batch(graph)
        return lib().oracle_set_temp(self.h, C.byref(b.f), C.byref(b.v), 1)

    def clearTempFactorsValues(self) -> int:
        return lib().oracle_clear_temp(self.h)

    def temp_sizes(self):
        """(getTempFactorsUnsafe().size(), getTempValues().size())"""
        nf, nv = C.c_int64(), C.c_int64()
        lib().oracle_temp_sizes(self.h, C.byref(nf), C.byref(nv))
        return nf.value, nv.value

    def getTempValues(self):
        n = self.temp_sizes()[1]
        keys = np.zeros(n, dtype=np.uint64)
        poses = np.zeros((n, 12 if self.dim == 3 else 4))
        assert lib().oracle_temp_values(self.h, _ptr(keys), _ptr(poses), n) == 0
        return keys, poses

    def getGncTempWeights(self):
        n = C.c_int64()
        lib().oracle_temp_weights(self.h, None, 0, C.byref(n))
        w = np.zeros(n.value)
        assert lib().oracle_temp_weights(self.h, _ptr(w), n.value, C.byref(n)) == 0
        return w

    def pcm_rows(self, graph, rows, lower_only=False):
        """On a fresh solver: classify, odometry-check and group the closures
        of `graph` (one batch) without the consistency matrix; returns (n,
        src, bits): the first group's size, the index in `graph` of each of
        its closures (group order), and rows `rows` of its consistency matrix
        (len(rows) x ceil(n / 32) words), evaluated on the OpenMP threads;
        lower_only: columns below the diagonal only (each pair once)."""
        b = _Batch(graph)
        r = np.ascontiguousarray(rows, dtype=np.int32)
        nf = max(graph.num_factors, 1)
        flat = np.zeros(max(len(r), 1) * ((nf + 31) // 32), dtype=np.uint32)
        src = np.zeros(nf, dtype=np.int64)
        n = C.c_int64(0)
        rc = lib().oracle_pcm_rows(self.h, C.byref(b.f), C.byref(b.v), _ptr(r), len(r), _ptr(flat), flat.size,
                                   C.byref(n), _ptr(src), src.size, int(lower_only))
        assert rc == 0, rc
        words = (n.value + 31) // 32
        bits = flat[:len(r) * words].reshape(len(r), words)
        return n.value, src[:n.value], bits

    def solve_graph(self, graph, n_known: int) -> int:
        """On a fresh solver: the solve stage alone (RobustSolver::optimize)
        over `graph`'s factors and values, with factors [0, n_known) as the
        GNC known inliers."""
        b = _Batch(graph)
        return lib().oracle_solve_graph(self.h, C.byref(b.f), C.byref(b.v), int(n_known))

    def set_warm_probs(self, probs):
        """Inlier probabilities for the next warm-started GNC solve, one per
        factor of the graph to optimise (known inliers are ignored)."""
        self._warm = np.ascontiguousarray(probs, dtype=np.float64)
        lib().oracle_set_warm_probs(self.h, _ptr(self._warm), self._warm.size)


def set_clique_impl(impl: int) -> int:
    """0: the reference's linear-search greedy clique (default); 1: the
    membership-stamp form; 2: the bit-row form on the OpenMP threads (both
    with identical results, for large checks). Returns the previous
    setting."""
    return lib().oracle_set_clique_impl(int(impl))


def filtered_graph(graph, kind, key1, key2):
    """The factor graph a solver's outlier rejection produced, rebuilt from
    its factor list (kind, key1, key2 in graph order) with the measurements
    and noise models of the matching factors of the input `graph`. The greedy
    clique can list a closure twice (stale buffer slots, as in the
    reference): a repeated factor reuses its input."""
    from rpgo_gb300.graph import Graph

    src = {}
    for i in range(graph.num_factors):
        src.setdefault((int(graph.kind[i]), int(graph.key1[i]), int(graph.key2[i])), []).append(i)
    g = Graph(graph.dim)
    used = {}
    for kd, a, b in zip(kind, key1, key2):
        key = (int(kd), int(a), int(b))
        j = src[key][min(used.get(key, 0), len(src[key]) - 1)]
        used[key] = used.get(key, 0) + 1
        g.kind.append(graph.kind[j])
        g.key1.append(graph.key1[j])
        g.key2.append(graph.key2[j])
        g.measured.append(graph.measured[j])
        g.cov.append(graph.cov[j])
        g.sqrt_info.append(graph.sqrt_info[j])
    g.value_keys, g.value_poses = list(graph.value_keys), list(graph.value_poses)
    return g


def clique_scan_ops(adj_words: np.ndarray, n: int, exact: bool = True) -> float:
    """Inner-loop iterations of the reference's linear-search greedy clique
    on this adjacency, not run: counted exactly (O(|S| + deg) per round), or
    with exact=False estimated on bit rows (each kept element's position in
    the neighbour list to its 64-bit word; for large dense matrices)."""
    adj = np.ascontiguousarray(adj_words, dtype=np.uint32)
    return lib().oracle_clique_scan_ops(int(n), _ptr(adj), int(bool(exact)))


def set_lm_max_iterations(n: int) -> int:
    """Cap every LM / GN run at n iterations (-1: the solver's own limit);
    returns the previous cap. For bounded CPU timing samples."""
    return lib().oracle_set_lm_max_iterations(int(n))


def set_threads(n: int = 0) -> int:
    """OpenMP threads of the oracle's pair tests (0: keep); returns the count."""
    return lib().oracle_set_threads(int(n))


# ------------------------------------------------------------------ math hooks
def pwc_op(dim, op, pa, ca, ria=1, pb=None, cb=None, rib=1):
    st, d = (12, 6) if dim == 3 else (4, 3)
    pa = np.ascontiguousarray(pa, dtype=np.float64)
    ca = np.ascontiguousarray(ca, dtype=np.float64)
    pb = np.ascontiguousarray(pb if pb is not None else pa, dtype=np.float64)
    cb = np.ascontiguousarray(cb if cb is not None else ca, dtype=np.float64)
    po = np.zeros(st)
    co = np.zeros((d, d))
    ri = C.c_int(0)
    lib().oracle_pwc_op(dim, op, _ptr(pa), _ptr(ca), ria, _ptr(pb), _ptr(cb), rib, _ptr(po), _ptr(co), C.byref(ri))
    return po, co, ri.value


def pwc_mahalanobis(dim, pose, cov, rot_info=1) -> float:
    pose = np.ascontiguousarray(pose, dtype=np.float64)
    cov = np.ascontiguousarray(cov, dtype=np.float64)
    return lib().oracle_pwc_mahalanobis(dim, _ptr(pose), _ptr(cov), rot_info)


def pwn_norms(dim, pose, node, rot_info=1):
    pose = np.ascontiguousarray(pose, dtype=np.float64)
    out = np.zeros(2)
    lib().oracle_pwn_norms(dim, _ptr(pose), node, rot_info, _ptr(out))
    return float(out[0]), float(out[1])


def logmap(dim, pose):
    pose = np.ascontiguousarray(pose, dtype=np.float64)
    xi = np.zeros(6 if dim == 3 else 3)
    lib().oracle_logmap(dim, _ptr(pose), _ptr(xi))
    return xi


def atan2(y, x) -> float:
    return lib().oracle_atan2(float(y), float(x))


def chi2inv(alpha, k) -> float:
    return lib().oracle_chi2inv(float(alpha), int(k))


def pairwise_adjacency(dim, mode, slot_a, slot_b, flip, z_pose, z_cov, traj_pose, traj_cov, traj_node, traj_rot,
                       th0, th1):
    n = len(slot_a)
    words = (n + 31) // 32
    adj = np.zeros((n, words), dtype=np.uint32)
    args = [np.ascontiguousarray(x) for x in (slot_a, slot_b, flip, z_pose, z_cov, traj_pose, traj_cov, traj_node,
                                              traj_rot)]
    lib().oracle_pairwise_adjacency(dim, mode, n, *[_ptr(a) for a in args], float(th0), float(th1), _ptr(adj))
    return adj


def max_clique_heu(adj_words: np.ndarray, n: int, first: int = 0, seed: int = -1):
    adj = np.ascontiguousarray(adj_words, dtype=np.uint32)
    out = np.zeros(max(n, 1), dtype=np.int32)
    size = np.zeros(1, dtype=np.int32)
    lib().oracle_max_clique_heu(n, _ptr(adj), first, seed, _ptr(out), _ptr(size))
    return int(size[0]), out[: max(int(size[0]), 0)].copy()

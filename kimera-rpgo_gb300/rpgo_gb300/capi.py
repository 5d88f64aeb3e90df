"""ctypes binding of librpgo_gb300.so (the C ABI of include/rpgo_gb300.h).

The library is the CUDA implementation; there is no Python or CPU fallback.
Loading fails loudly when the shared library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librpgo_gb300.so")
_lib = None

OK, ERR_ARG, ERR_CUDA, ERR_KEY, ERR_SOLVER, ERR_UNSUPPORTED, ERR_SIZE = range(7)
CLIQUE_NOALLOC_MAX_N = 4096
CLIQUE_NOALLOC_MAX_WORDS = 128


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


class Timing(C.Structure):
    _fields_ = [("pcm_ms", C.c_double), ("solve_ms", C.c_double)] + [
        (n, C.c_int64) for n in ("pair_checks", "lm_iterations", "linear_solves", "gnc_iterations", "cg_iterations",
                                 "kernel_launches")] + [
        ("pcg_kernel_ms", C.c_double), ("pcg_kernel_launches", C.c_int64), ("pcg_kernel_bytes", C.c_double),
        ("chol_kernel_ms", C.c_double), ("chol_kernel_launches", C.c_int64), ("chol_kernel_flops", C.c_double),
        ("chol_kernel_bytes", C.c_double), ("chol_levels", C.c_int64), ("chol_tail", C.c_int64),
        ("pair_kernel_ms", C.c_double), ("pair_kernel_launches", C.c_int64),
        ("warm_runs", C.c_int64), ("warm_fallbacks", C.c_int64)]


MLP_FEATURES, MLP_PARAMS = 16, 5345


class BatchOut(C.Structure):
    _fields_ = [("poses", C.c_void_p), ("gnc_weights", C.c_void_p), ("num_weights", C.c_void_p),
                ("status", C.c_void_p), ("timing", C.c_void_p)]


# every exported entry point: name -> (restype, argtypes)
_P = C.c_void_p
SIGNATURES = {
    "rpgo_params_default": (None, [C.POINTER(Params)]),
    "rpgo_params_set_no_rejection": (None, [C.POINTER(Params), C.c_int32]),
    "rpgo_params_set_pcm2d": (None, [C.POINTER(Params), C.c_double, C.c_double, C.c_int32]),
    "rpgo_params_set_pcm3d": (None, [C.POINTER(Params), C.c_double, C.c_double, C.c_int32]),
    "rpgo_params_set_pcm_simple2d": (None, [C.POINTER(Params)] + [C.c_double] * 4 + [C.c_int32]),
    "rpgo_params_set_pcm_simple3d": (None, [C.POINTER(Params)] + [C.c_double] * 4 + [C.c_int32]),
    "rpgo_params_set_multirobot_align": (None, [C.POINTER(Params), C.c_int32, C.c_double]),
    "rpgo_params_set_gnc_probability": (None, [C.POINTER(Params), C.c_double, C.c_int32, C.c_double, C.c_double,
                                               C.c_double, C.c_int32, C.c_int32]),
    "rpgo_params_set_gnc_cost": (None, [C.POINTER(Params), C.c_double, C.c_int32, C.c_double, C.c_double,
                                        C.c_double, C.c_int32, C.c_int32]),
    "rpgo_create": (_P, [C.POINTER(Params)]),
    "rpgo_destroy": (None, [_P]),
    "rpgo_update": (C.c_int, [_P, C.POINTER(FactorBatch), C.POINTER(ValueBatch), C.c_int32]),
    "rpgo_update_dev": (C.c_int, [_P, C.POINTER(FactorBatch), C.POINTER(ValueBatch), C.c_int32]),
    "rpgo_force_update": (C.c_int, [_P, C.POINTER(FactorBatch), C.POINTER(ValueBatch)]),
    "rpgo_load_graph": (C.c_int, [_P, C.POINTER(FactorBatch), C.POINTER(ValueBatch), C.POINTER(FactorBatch)]),
    "rpgo_add_graph": (C.c_int, [_P, C.POINTER(FactorBatch), C.POINTER(ValueBatch), C.POINTER(FactorBatch)]),
    "rpgo_get_counts": (C.c_int, [_P, C.POINTER(Counts)]),
    "rpgo_get_estimate": (C.c_int, [_P, _P, _P, C.c_int64]),
    "rpgo_get_gnc_weights": (C.c_int, [_P, _P, C.c_int64]),
    "rpgo_update_temp_factors_values": (C.c_int, [_P, C.POINTER(FactorBatch), C.POINTER(ValueBatch)]),
    "rpgo_replace_temp_factors_values": (C.c_int, [_P, C.POINTER(FactorBatch), C.POINTER(ValueBatch)]),
    "rpgo_clear_temp_factors_values": (C.c_int, [_P]),
    "rpgo_get_temp_sizes": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "rpgo_get_temp_values": (C.c_int, [_P, _P, _P, C.c_int64]),
    "rpgo_get_gnc_temp_weights": (C.c_int, [_P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "rpgo_get_factors": (C.c_int, [_P, _P, _P, _P, _P, C.c_int64]),
    "rpgo_get_adjacency": (C.c_int, [_P, C.c_int32, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "rpgo_get_timing": (C.c_int, [_P, C.POINTER(Timing)]),
    "rpgo_set_warm_start_probs": (C.c_int, [_P, _P, C.c_int64]),
    "rpgo_remove_last_loop_closure": (C.c_int, [_P, C.c_int32, C.c_char, C.c_char, C.POINTER(C.c_uint64),
                                                C.POINTER(C.c_uint64), C.POINTER(C.c_int32)]),
    "rpgo_ignore_prefix": (C.c_int, [_P, C.c_char]),
    "rpgo_revive_prefix": (C.c_int, [_P, C.c_char]),
    "rpgo_get_ignored_prefixes": (C.c_int, [_P, C.c_char_p, C.c_int32, C.POINTER(C.c_int32)]),
    "rpgo_remove_prior_factors_with_prefix": (C.c_int, [_P, C.c_char, C.c_int32]),
    "rpgo_set_warm_start_model": (C.c_int, [_P, _P]),
    "rpgo_get_closure_features": (C.c_int, [_P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "rpgo_mlp_forward_dev": (C.c_int, [_P, C.c_int64, _P, _P, _P]),
    "rpgo_mlp_train_step_dev": (C.c_int, [_P, _P, _P, C.c_int64, C.c_float, C.c_int64, _P, _P, _P,
                                          C.POINTER(C.c_double), _P]),
    "rpgo_g2o_read": (_P, [C.c_char_p, C.c_int32, C.POINTER(C.c_int32)]),
    "rpgo_g2o_view": (C.c_int, [_P, C.POINTER(FactorBatch), C.POINTER(ValueBatch)]),
    "rpgo_g2o_free": (None, [_P]),
    "rpgo_solve_batch": (C.c_int, [C.POINTER(Params), C.c_int32, _P, _P, C.c_int32, C.c_int32,
                                   C.POINTER(BatchOut)]),
    "rpgo_solve_batch_joint": (C.c_int, [C.POINTER(Params), C.c_int32, _P, _P, C.c_int32, C.c_int32,
                                         C.POINTER(BatchOut)]),
    "rpgo_set_joint_graphs": (C.c_int32, [C.c_int32]),
    "rpgo_joint_graph_rounds": (C.c_int64, []),
    "rpgo_save_data": (C.c_int, [_P, C.c_char_p]),
    "rpgo_trajectory_scan_dev": (C.c_int, [C.c_int32, C.c_int32, C.c_int64] + [_P] * 8 + [_P]),
    "rpgo_odometry_check_dev": (C.c_int, [C.c_int32, C.c_int32, C.c_int64] + [_P] * 8 + [C.c_double, C.c_double,
                                                                                          _P, _P]),
    "rpgo_pairwise_adjacency_dev": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32] + [_P] * 9 + [
        C.c_double, C.c_double, _P, C.c_int32, _P]),
    "rpgo_max_clique_heu_dev": (C.c_int, [C.c_int32, _P, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P]),
    "rpgo_max_clique_heu_dev_noalloc": (C.c_int, [C.c_int32, _P, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P]),
    "rpgo_pairwise_adjacency": (C.c_int, [C.c_int32, C.c_int32, C.c_int32] + [_P] * 5 + [C.c_int32] + [_P] * 4 + [
        C.c_double, C.c_double, _P]),
    "rpgo_max_clique_heu": (C.c_int, [C.c_int32, _P, C.c_int32, C.c_int32, _P, _P]),
    "rpgo_device_info": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.c_int32)]),
    "rpgo_kernel_launch_count": (C.c_int64, []),
    "rpgo_buffer_alloc_count": (C.c_int64, []),
    "rpgo_set_direct_solve_guard": (C.c_double, [C.c_double, C.c_int32]),
}


def load():
    """Load the CUDA library (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with python kimera-rpgo_gb300/build.py")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


def params_struct(p) -> Params:
    s = Params()
    for name, _ in Params._fields_:
        setattr(s, name, getattr(p, name))
    return s


class Batch:
    """A graph in the C ABI's host layout (rpgo_factor_batch / rpgo_value_batch);
    keeps the numpy arrays alive while the C structs point into them. Every
    call that takes a graph also takes a Batch (converted once, reused)."""

    def __init__(self, g):
        self.a = g.arrays()
        a = self.a
        self.f = FactorBatch(len(a["kind"]), _ptr(a["kind"]), _ptr(a["key1"]), _ptr(a["key2"]), _ptr(a["measured"]),
                             _ptr(a["cov"]), _ptr(a["sqrt_info"]))
        self.v = ValueBatch(len(a["value_keys"]), _ptr(a["value_keys"]), _ptr(a["value_poses"]))


def as_batch(g) -> Batch:
    return g if isinstance(g, Batch) else Batch(g)


class DeviceBatch:
    """A graph whose bulk arrays (measurements, covariances, square-root
    informations, value poses) sit in GPU memory (torch tensors on cuda:0);
    kinds and keys stay on the host. For rpgo_update_dev."""

    def __init__(self, g):
        import torch

        self.a = g.arrays()
        a = self.a
        dev = torch.device("cuda", 0)
        self.t = {k: torch.from_numpy(np.ascontiguousarray(a[k])).to(dev)
                  for k in ("measured", "cov", "sqrt_info", "value_poses")}
        torch.cuda.synchronize()
        tp = lambda k: self.t[k].data_ptr() if self.t[k].numel() else None
        self.f = FactorBatch(len(a["kind"]), _ptr(a["kind"]), _ptr(a["key1"]), _ptr(a["key2"]), tp("measured"),
                             tp("cov"), tp("sqrt_info"))
        self.v = ValueBatch(len(a["value_keys"]), _ptr(a["value_keys"]), tp("value_poses"))
        self.bytes = sum(int(x.numel()) * 8 for x in self.t.values())


class RpgoError(RuntimeError):
    pass


class RobustSolver:
    """KimeraRPGO::RobustSolver on the GPU (include/KimeraRPGO/RobustSolver.h)."""

    def __init__(self, params):
        self.dim = 2 if params.outlier_removal in (1, 3) or (params.outlier_removal == 0 and params.dim == 2) else 3
        self._p = params_struct(params)
        self.use_gnc = bool(params.use_gnc)
        self.h = load().rpgo_create(C.byref(self._p))
        if not self.h:
            raise RpgoError("rpgo_create failed (bad parameters or no CUDA device)")

    def __del__(self):
        if getattr(self, "h", None):
            load().rpgo_destroy(self.h)
            self.h = None

    # ---- reference API
    def update(self, graph, optimize_graph: bool = True) -> int:
        b = as_batch(graph)
        return load().rpgo_update(self.h, C.byref(b.f), C.byref(b.v), int(optimize_graph))

    def update_dev(self, dbatch: "DeviceBatch", optimize_graph: bool = True) -> int:
        return load().rpgo_update_dev(self.h, C.byref(dbatch.f), C.byref(dbatch.v), int(optimize_graph))

    def forceUpdate(self, graph) -> int:
        b = as_batch(graph)
        return load().rpgo_force_update(self.h, C.byref(b.f), C.byref(b.v))

    def loadGraph(self, graph, prior) -> int:
        b, p = as_batch(graph), as_batch(prior)
        return load().rpgo_load_graph(self.h, C.byref(b.f), C.byref(b.v), C.byref(p.f))

    def addGraph(self, graph, between) -> int:
        b, p = as_batch(graph), as_batch(between)
        return load().rpgo_add_graph(self.h, C.byref(b.f), C.byref(b.v), C.byref(p.f))

    def counts(self) -> Counts:
        c = Counts()
        load().rpgo_get_counts(self.h, C.byref(c))
        return c

    def size(self) -> int:
        return self.counts().num_factors

    def getNumLC(self) -> int:
        return self.counts().num_lc

    def getNumLCInliers(self) -> int:
        return self.counts().num_lc_inliers

    def estimate(self):
        n = self.counts().num_values
        st = 12 if self.dim == 3 else 4
        keys = np.zeros(n, dtype=np.uint64)
        poses = np.zeros((n, st))
        rc = load().rpgo_get_estimate(self.h, _ptr(keys), _ptr(poses), n)
        if rc:
            raise RpgoError(f"rpgo_get_estimate: {rc}")
        return keys, poses

    calculateEstimate = estimate
    calculateBestEstimate = estimate  # GenericSolver.h:42
    getLinearizationPoint = estimate  # GenericSolver.h:43

    def gnc_weights(self):
        n = self.counts().num_gnc_weights
        w = np.zeros(n)
        load().rpgo_get_gnc_weights(self.h, _ptr(w), n)
        return w

    getGncWeights = gnc_weights

    # temporary factors and values (GenericSolver.h:46-65)
    def updateTempFactorsValues(self, graph) -> int:
        b = as_batch(graph)
        return load().rpgo_update_temp_factors_values(self.h, C.byref(b.f), C.byref(b.v))

    def replaceTempFactorsValues(self, graph) -> int:
        b = as_batch(graph)
        return load().rpgo_replace_temp_factors_values(self.h, C.byref(b.f), C.byref(b.v))

    def clearTempFactorsValues(self) -> int:
        return load().rpgo_clear_temp_factors_values(self.h)

    def temp_sizes(self):
        """(getTempFactorsUnsafe().size(), getTempValues().size())"""
        nf, nv = C.c_int64(), C.c_int64()
        load().rpgo_get_temp_sizes(self.h, C.byref(nf), C.byref(nv))
        return nf.value, nv.value

    def getTempValues(self):
        n = self.temp_sizes()[1]
        keys = np.zeros(n, dtype=np.uint64)
        poses = np.zeros((n, 12 if self.dim == 3 else 4))
        rc = load().rpgo_get_temp_values(self.h, _ptr(keys), _ptr(poses), n)
        if rc:
            raise RpgoError(f"rpgo_get_temp_values: {rc}")
        return keys, poses

    def getGncTempWeights(self):
        n = C.c_int64()
        load().rpgo_get_gnc_temp_weights(self.h, None, 0, C.byref(n))
        w = np.zeros(n.value)
        rc = load().rpgo_get_gnc_temp_weights(self.h, _ptr(w), n.value, C.byref(n))
        if rc:
            raise RpgoError(f"rpgo_get_gnc_temp_weights: {rc}")
        return w

    def factors(self):
        n = self.counts().num_factors
        st = 12 if self.dim == 3 else 4
        kind = np.zeros(n, dtype=np.int32)
        k1 = np.zeros(n, dtype=np.uint64)
        k2 = np.zeros(n, dtype=np.uint64)
        meas = np.zeros((n, st))
        load().rpgo_get_factors(self.h, _ptr(kind), _ptr(k1), _ptr(k2), _ptr(meas), n)
        return kind, k1, k2, meas

    getFactorsUnsafe = factors

    def adjacency(self, group: int = 0):
        n = C.c_int64(0)
        if load().rpgo_get_adjacency(self.h, group, None, 0, C.byref(n)) != 0:
            return None
        words = (n.value + 31) // 32
        out = np.zeros(n.value * words, dtype=np.uint32)
        load().rpgo_get_adjacency(self.h, group, _ptr(out), out.size, C.byref(n))
        return out.reshape(n.value, words)

    def timing(self) -> Timing:
        t = Timing()
        load().rpgo_get_timing(self.h, C.byref(t))
        return t

    def saveData(self, folder: str) -> int:
        return load().rpgo_save_data(self.h, folder.encode())

    # ---- edit API (src/RobustSolver.cpp:371-446)
    def removeLastLoopClosure(self, prefix_1=None, prefix_2=None):
        """Returns (from_key, to_key) of the removed closure, or None."""
        a, b, r = C.c_uint64(), C.c_uint64(), C.c_int32()
        by_id = prefix_1 is not None
        p1 = (prefix_1 or "\0").encode()
        p2 = (prefix_2 or "\0").encode()
        rc = load().rpgo_remove_last_loop_closure(self.h, int(by_id), p1, p2, C.byref(a), C.byref(b), C.byref(r))
        if rc:
            raise RpgoError(f"rpgo_remove_last_loop_closure: {rc}")
        return (a.value, b.value) if r.value else None

    def ignorePrefix(self, prefix: str) -> int:
        return load().rpgo_ignore_prefix(self.h, prefix.encode())

    def revivePrefix(self, prefix: str) -> int:
        return load().rpgo_revive_prefix(self.h, prefix.encode())

    def getIgnoredPrefixes(self):
        n = C.c_int32()
        load().rpgo_get_ignored_prefixes(self.h, None, 0, C.byref(n))
        buf = C.create_string_buffer(max(n.value, 1))
        load().rpgo_get_ignored_prefixes(self.h, buf, n.value, C.byref(n))
        return [chr(c) for c in buf.raw[:n.value]]

    def removePriorFactorsWithPrefix(self, prefix: str, optimize_graph: bool = True) -> int:
        return load().rpgo_remove_prior_factors_with_prefix(self.h, prefix.encode(), int(optimize_graph))

    # ---- GNC warm start (no counterpart in the reference)
    def set_warm_start_model(self, params) -> int:
        """Install a closure network (MLP_PARAMS floats) for the warm start;
        None removes it."""
        if params is None:
            return load().rpgo_set_warm_start_model(self.h, None)
        self._model = np.ascontiguousarray(params, dtype=np.float32)
        assert self._model.size == MLP_PARAMS
        return load().rpgo_set_warm_start_model(self.h, _ptr(self._model))

    def closure_features(self):
        """Features of the closures of the last warm-mode GNC solve (rows of
        MLP_FEATURES floats, graph order)."""
        n = C.c_int64(0)
        load().rpgo_get_closure_features(self.h, None, 0, C.byref(n))
        out = np.zeros((n.value, MLP_FEATURES), dtype=np.float32)
        if n.value:
            load().rpgo_get_closure_features(self.h, _ptr(out), n.value, C.byref(n))
        return out

    def set_warm_start_probs(self, probs) -> int:
        """Inlier probabilities for the next warm-started GNC solve, one per
        factor of the graph it optimises (known inliers are ignored)."""
        self._warm = np.ascontiguousarray(probs, dtype=np.float64)
        return load().rpgo_set_warm_start_probs(self.h, _ptr(self._warm), self._warm.size)


# ------------------------------------------------------------------ stage functions (host arrays)
def read_g2o(path: str, dim: int = 3):
    """rpgo_g2o_read: the graph of a g2o file (factors in file order, then
    the vertices as values), as a Graph."""
    from .graph import Graph

    lib = load()
    st = C.c_int32(0)
    h = lib.rpgo_g2o_read(path.encode(), int(dim), C.byref(st))
    if not h:
        raise RpgoError(f"rpgo_g2o_read({path}): {st.value}")
    try:
        f, v = FactorBatch(), ValueBatch()
        lib.rpgo_g2o_view(h, C.byref(f), C.byref(v))
        stride, d = (12, 6) if dim == 3 else (4, 3)
        n, m = int(f.count), int(v.count)

        def arr(ptr, ctype, count):
            if count == 0:
                return np.zeros(0)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(count,)).copy()

        g = Graph(dim)
        g.kind = [int(x) for x in arr(f.kind, C.c_int32, n)]
        g.key1 = [int(x) for x in arr(f.key_front, C.c_uint64, n)]
        g.key2 = [int(x) for x in arr(f.key_back, C.c_uint64, n)]
        meas = arr(f.measured, C.c_double, n * stride).reshape(n, stride)
        cov = arr(f.covariance, C.c_double, n * d * d).reshape(n, d, d)
        sq = arr(f.sqrt_information, C.c_double, n * d * d).reshape(n, d, d)
        g.measured, g.cov, g.sqrt_info = list(meas), list(cov), list(sq)
        g.value_keys = [int(x) for x in arr(v.key, C.c_uint64, m)]
        g.value_poses = list(arr(v.pose, C.c_double, m * stride).reshape(m, stride))
        return g
    finally:
        lib.rpgo_g2o_free(h)


def solve_batch(params, graphs, workers: int = 0, coop_ctas: int = 0, joint: bool = False, group: int = 0,
                streams: int = 0):
    """rpgo_solve_batch: solve independent graphs concurrently (joint: the
    lock-step rpgo_solve_batch_joint, `streams` concurrent groups of `group`
    graphs; 0 = defaults).
    Returns a list of (status, keys, poses, gnc_weights, timing) per graph,
    the poses in ascending key order as calculateEstimate() gives them."""
    n = len(graphs)
    batches = [as_batch(g) for g in graphs]
    fb = (FactorBatch * max(n, 1))(*[b.f for b in batches])
    vb = (ValueBatch * max(n, 1))(*[b.v for b in batches])
    dim = 2 if params.outlier_removal in (1, 3) or (params.outlier_removal == 0 and params.dim == 2) else 3
    st = 12 if dim == 3 else 4
    nv = [int(b.v.count) for b in batches]
    nf = [int(b.f.count) for b in batches]
    poses = np.zeros((max(sum(nv), 1), st))
    weights = np.zeros(max(sum(nf), 1))
    num_w = np.zeros(max(n, 1), dtype=np.int64)
    status = np.zeros(max(n, 1), dtype=np.int32)
    timing = (Timing * max(n, 1))()
    out = BatchOut(_ptr(poses), _ptr(weights), _ptr(num_w), _ptr(status), C.cast(timing, C.c_void_p))
    p = params_struct(params)
    if joint:
        rc = load().rpgo_solve_batch_joint(C.byref(p), n, C.cast(fb, C.c_void_p), C.cast(vb, C.c_void_p), int(group),
                                           int(streams), C.byref(out))
    else:
        rc = load().rpgo_solve_batch(C.byref(p), n, C.cast(fb, C.c_void_p), C.cast(vb, C.c_void_p), int(workers),
                                     int(coop_ctas), C.byref(out))
    if rc:
        raise RpgoError(f"rpgo_solve_batch{'_joint' if joint else ''}: {rc}")
    res, vo, fo = [], 0, 0
    for g in range(n):
        keys = np.sort(np.asarray(batches[g].a["value_keys"], dtype=np.uint64))
        res.append((int(status[g]), keys, poses[vo:vo + nv[g]].copy(), weights[fo:fo + int(num_w[g])].copy(),
                    timing[g]))
        vo += nv[g]
        fo += nf[g]
    return res


BATCH_CANDIDATES = (
    {"workers": 8}, {"workers": 4}, {"workers": 12}, {"workers": 8, "coop_ctas": 76}, {"workers": 8, "coop_ctas": 19},
    {"joint": True, "streams": 1}, {"joint": True, "streams": 2}, {"joint": True, "streams": 4},
    {"joint": True, "streams": 8}, {"joint": True, "streams": 4, "group": 4},
)


def _config_name(c):
    if c.get("joint"):
        return f"joint_s{c.get('streams', 0)}_g{c.get('group', 0)}"
    return f"workers{c.get('workers', 0)}_ctas{c.get('coop_ctas', 0)}"


def autotune_batch(params, graphs, candidates=BATCH_CANDIDATES, margin=0.05):
    """Pick the configuration of the batched solve that finishes a sample of
    graphs fastest (wall clock, after one warm-up run of the sample): the
    worker form (rpgo_solve_batch: host threads, the CTA budget of each
    direct solve) or the joint form (rpgo_solve_batch_joint: concurrent
    lock-step groups, their size and, through the stream count, each group's
    CTA budget). The first candidate is kept unless another is faster by more
    than `margin` (timing noise on a small sample). Returns (config,
    {name: seconds}); config holds solve_batch's keyword arguments."""
    import time

    solve_batch(params, graphs[:2], workers=2)
    solve_batch(params, graphs[:2], joint=True)
    times = {}
    for c in candidates:
        t0 = time.perf_counter()
        res = solve_batch(params, graphs, **c)
        times[_config_name(c)] = time.perf_counter() - t0
        if any(r[0] != 0 for r in res):
            raise RpgoError(f"batched solve failed with {c}")
    first = _config_name(candidates[0])
    best = min(candidates, key=lambda c: times[_config_name(c)])
    if times[_config_name(best)] > (1.0 - margin) * times[first]:
        best = candidates[0]
    return dict(best), times


def pairwise_adjacency(dim, mode, slot_a, slot_b, flip, z_pose, z_cov, traj_pose, traj_cov, traj_node, traj_rot,
                       th0, th1):
    n = len(slot_a)
    words = (n + 31) // 32
    adj = np.zeros((max(n, 1), max(words, 1)), dtype=np.uint32)
    arrs = [np.ascontiguousarray(x) for x in (slot_a, slot_b, flip, z_pose, z_cov)]
    tr = [np.ascontiguousarray(x) for x in (traj_pose, traj_cov, traj_node, traj_rot)]
    rc = load().rpgo_pairwise_adjacency(dim, mode, n, *[_ptr(a) for a in arrs], len(traj_rot),
                                        *[_ptr(a) for a in tr], float(th0), float(th1), _ptr(adj))
    if rc:
        raise RpgoError(f"rpgo_pairwise_adjacency: {rc}")
    return adj[:n, :words]


def max_clique_heu(adj_words, n, first=0, seed=-1):
    adj = np.ascontiguousarray(adj_words, dtype=np.uint32)
    out = np.zeros(max(n, 1), dtype=np.int32)
    size = np.zeros(1, dtype=np.int32)
    rc = load().rpgo_max_clique_heu(n, _ptr(adj), first, seed, _ptr(out), _ptr(size))
    if rc:
        raise RpgoError(f"rpgo_max_clique_heu: {rc}")
    return int(size[0]), out[: max(int(size[0]), 0)].copy()


def device_info():
    name = C.create_string_buffer(256)
    sm = C.c_int32(0)
    rc = load().rpgo_device_info(name, 256, C.byref(sm))
    if rc:
        raise RpgoError("no CUDA device")
    return name.value.decode(), sm.value


def kernel_launch_count() -> int:
    return int(load().rpgo_kernel_launch_count())


def set_direct_solve_guard(flops: float, prefer: int = 0) -> float:
    """Fill-in guard of the direct solve: plans above `flops` race the direct
    and PCG solvers on the first damped system (prefer 0: keep the faster,
    1: direct, 2: PCG). Returns the previous threshold."""
    return float(load().rpgo_set_direct_solve_guard(float(flops), int(prefer)))


def buffer_alloc_count() -> int:
    """Device and pinned host allocations made by the library's buffers."""
    return int(load().rpgo_buffer_alloc_count())

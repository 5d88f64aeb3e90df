#!/usr/bin/env python
"""PCM + GNC-TLS robust back-end throughput on one GB300 (graphs/s).

Workload (one step = one graph through RobustSolver::update, PCM outlier
rejection then the GNC-TLS / LM solve), default: the seeded 3D random-walk
graph of 50,000 poses with 20,000 loop closures, 30 % of them outliers
(2e8 candidate pair checks), PCM3D thresholds 10 / 5, GNC-TLS at probability
0.9. `--workload walk3d_5000` runs the 5,000-pose graph (1,000 inlier + 333
outlier closures) instead; it is also an extra leg of the default run.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

gb300 arm: `value` = graphs/s with the graph's bulk arrays already resident
in HBM (rpgo_update_dev); `e2e` = graphs/s through rpgo_update from pinned
host buffers with the estimate and GNC weights read back every step. L2 is
flushed (256 MiB write) between timed steps. Multi-GPU: replicas only (each
rank solves its own copy; no collective on the data path). The CPU leg
(rank 0, N = 1) times a bounded single-thread sample of the CPU FP64
restatement of the reference path (oracle/) and checks this run's result
against it stage by stage (`parity`).

reference arm: the CPU FP64 restatement of the reference path (the reference
itself needs GTSAM, absent here) runs the same graph once on every host
thread, cut into K timed slices (the pair tests by row block, then the
clique, then the GNC-TLS solve).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "kimera-rpgo_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "PCM+GNC solve ms and graphs/s vs plain GPU at ATE<=1e-4 m; pair checks/s"
# nominal FP64 rate of one GB300 (no measured FP64 figure exists for this part)
FP64_NOMINAL_GFLOPS = 1250.0
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit())
        mx = max((float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def dist_setup(n_gpus):
    """One process per GPU (replicas: no collective on the data path; the
    process group only times the job). NCCL with CUDA, gloo without."""
    import torch

    if n_gpus > 1 or "WORLD_SIZE" in os.environ and int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        local = int(os.environ.get("LOCAL_RANK", "0"))
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        return dist, dist.get_rank(), dist.get_world_size(), local
    return None, 0, 1, 0


def barrier(dist):
    import torch

    if dist is not None:
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def max_over_ranks(dist, x):
    """The slowest rank's time: the job ends when every replica has."""
    import torch

    if dist is None:
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, ms_per_step_max):
    """Graphs per second of the whole job: every rank solves one graph per
    step, and the step lasts as long as the slowest rank's."""
    return world * 1000.0 / ms_per_step_max




WORKLOADS = {
    "walk3d_50000": ("3d random walk, 50000 poses, 14000 inlier + 6000 outlier loop closures (2e8 candidate pair "
                     "checks), PCM3D(10,5) + GNC-TLS(p=0.9)", 50000, 20000, 0.30),
    "walk3d_5000": ("3d random walk, 5000 poses, 1000 inlier + 333 outlier loop closures, PCM3D(10,5) + "
                    "GNC-TLS(p=0.9)", 5000, 1333, 0.25),
}
DEFAULT_WORKLOAD = "walk3d_50000"
L2_NOTE = "L2 flushed between GPU steps (256 MiB write)"


def bench_config(name, world):
    """The workload as both arms report it (identical dicts)."""
    desc, n_poses, n_lc, out_frac = WORKLOADS[name]
    return {"workload": desc, "graph_poses": n_poses, "loop_closures": n_lc, "outlier_fraction": out_frac,
            "solver": "PCM3D(10,5), then GNC-TLS(p=0.9) over LM", "l2": L2_NOTE,
            "parallelism": "replicas" if world > 1 else "single GPU"}


def make_workload(name=DEFAULT_WORKLOAD):
    from rpgo_gb300 import synth
    from rpgo_gb300.params import QUIET, RobustSolverParams

    s = synth.config_c2() if name == "walk3d_5000" else synth.config_c3()
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    return s, p


# ------------------------------------------------------------------ gb300 arm
class Arm:
    """The graph in HBM and in pinned host memory, with the two step kinds."""

    def __init__(self, s, params):
        import ctypes as C

        import numpy as np
        import torch

        from rpgo_gb300 import capi

        self.s, self.params, self.capi = s, params, capi
        self.lib = capi.load()
        self.dev_batch = capi.DeviceBatch(s.graph)
        arrays = s.graph.arrays()
        self.pinned = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in arrays.items()}

        def pp(k):
            return self.pinned[k].data_ptr() if self.pinned[k].numel() else None

        self.host_f = capi.FactorBatch(len(arrays["kind"]), pp("kind"), pp("key1"), pp("key2"), pp("measured"),
                                       pp("cov"), pp("sqrt_info"))
        self.host_v = capi.ValueBatch(len(arrays["value_keys"]), pp("value_keys"), pp("value_poses"))
        self.h2d = sum(int(t.numel()) * t.element_size() for t in self.pinned.values())
        n_val = len(arrays["value_keys"])
        self.out_keys = np.zeros(n_val, dtype=np.uint64)
        self.out_poses = torch.empty((n_val, 12), dtype=torch.float64).pin_memory()
        self.out_w = torch.empty(s.graph.num_factors, dtype=torch.float64).pin_memory()
        self.C = C

    def step_dev(self, params=None, model=None):
        g = self.capi.RobustSolver(params or self.params)
        if model is not None:
            g.set_warm_start_model(model)
        rc = g.update_dev(self.dev_batch, True)
        assert rc == 0, rc
        return g

    def step_e2e(self):
        C = self.C
        g = self.capi.RobustSolver(self.params)
        rc = self.lib.rpgo_update(g.h, C.byref(self.host_f), C.byref(self.host_v), 1)
        assert rc == 0, rc
        c = g.counts()
        self.lib.rpgo_get_estimate(g.h, self.out_keys.ctypes.data, self.out_poses.data_ptr(), c.num_values)
        self.lib.rpgo_get_gnc_weights(g.h, self.out_w.data_ptr(), self.s.graph.num_factors)
        return g, 8 * c.num_values * 13 + 8 * c.num_gnc_weights


def timed_steps(fn, steps, flush, dist=None):
    """CUDA-event time of each call of fn (after an L2 flush), with a barrier
    and a device synchronisation on both sides; returns (ms list, last result)."""
    import torch

    times, out = [], None
    for _ in range(steps):
        flush.zero_()
        barrier(dist)
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        out = fn()
        t1.record()
        barrier(dist)
        times.append(t0.elapsed_time(t1))
    return times, out


def run_gb300(args):
    import torch

    from rpgo_gb300 import build, capi

    dist, rank, world, local = dist_setup(args.gpus)
    build()
    capi.load()
    s, params = make_workload(args.workload)
    arm = Arm(s, params)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    for _ in range(args.warmup):
        arm.step_dev()
    tims = []

    def step():
        g = arm.step_dev()
        tims.append(g.timing())
        return g

    with ClockSampler(local) as clocks:
        times, g_last = timed_steps(step, args.steps, flush, dist)
        # e2e: pinned host buffers in, estimate + weights out, through rpgo_update
        e2e_times, (g_e2e, d2h) = timed_steps(arm.step_e2e, args.steps, flush, dist)
    ms = max_over_ranks(dist, sum(times) / len(times))
    e2e_ms = max_over_ranks(dist, sum(e2e_times) / len(e2e_times))
    last = tims[-1]
    peak, peak_kind = peaks()
    n_chol = sum(t.chol_kernel_launches for t in tims)
    n_pcg = sum(t.pcg_kernel_launches for t in tims)
    if n_chol:
        kname = "k_chol_solve (direct sparse Cholesky solve, FP64)"
        launch_ms = sum(t.chol_kernel_ms for t in tims) / n_chol
        launch_bytes = sum(t.chol_kernel_bytes for t in tims) / n_chol
        launch_flops = sum(t.chol_kernel_flops for t in tims) / n_chol
        traffic_file = f"chol_traffic_{args.workload}.json"
    else:
        kname = "k_pcg_coop (whole-GPU flexible PCG)"
        launch_ms = sum(t.pcg_kernel_ms for t in tims) / max(1, n_pcg)
        launch_bytes = sum(t.pcg_kernel_bytes for t in tims) / max(1, n_pcg)
        launch_flops = None
        traffic_file = f"pcg_traffic_{args.workload}.json"
    achieved = launch_bytes / (launch_ms * 1e-3) / 1e9 if launch_ms > 0 else 0.0
    pair_ms = sum(t.pair_kernel_ms for t in tims) / max(1, sum(t.pair_kernel_launches for t in tims))
    traffic = None
    tpath = os.path.join(ROOT, "profiles", traffic_file)
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("bytes_per_launch_scaled")
    fp64 = (launch_flops / (launch_ms * 1e-3) / 1e9) if launch_flops and launch_ms > 0 else None
    line = {
        "metric": METRIC,
        "value": job_value(world, ms),
        "unit": "graphs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded 3d random walk; no public dataset in the reference)",
        "config": bench_config(args.workload, world),
        "solve_ms": sum(t.solve_ms for t in tims) / len(tims),
        "pcm_ms": sum(t.pcm_ms for t in tims) / len(tims),
        "pair_checks": last.pair_checks,
        "pair_checks_per_s": last.pair_checks / (pair_ms * 1e-3) if pair_ms > 0 else None,
        "gnc_iterations": last.gnc_iterations,
        "lm_iterations": last.lm_iterations,
        "linear_solves": last.linear_solves,
        "cg_iterations": last.cg_iterations,
        "chol_levels": last.chol_levels,
        "chol_tail": last.chol_tail,
        "gpu_launches": sum(t.kernel_launches for t in tims),
        "e2e": {"value": job_value(world, e2e_ms), "unit": "graphs/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": arm.h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"kernel": kname,
                     "bound": "latency (FP64 issue along the elimination tree and grid barriers); frac is against "
                              "HBM bandwidth",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "launch_ms": launch_ms,
                     "bytes_per_launch": launch_bytes, "launches_per_step": (n_chol or n_pcg) / len(tims),
                     "fp64_gflops": fp64, "fp64_peak_nominal_gflops": FP64_NOMINAL_GFLOPS},
        "clocks": clocks.summary(),
    }
    extras = world == 1 and not args.no_extras
    warm = None
    if extras:
        warm = warm_start_leg(args, arm, g_last, ms, flush)
        line["warm_start"] = {k: ({a: b for a, b in v.items() if not a.startswith("_")} if isinstance(v, dict) else v)
                              for k, v in warm.items()}
        if args.workload != "walk3d_5000":
            line["walk3d_5000"], c2 = small_graph_leg(flush)
        else:
            c2 = None
        line["batched"] = batched_leg(params)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the GPU line is printed whatever happens in the CPU leg
        try:
            cb, par = cpu_leg(args, s, params, g_last, warm, c2 if extras else None)
            line["cpu_baseline"] = cb
            line["parity"] = par
        except Exception as e:  # noqa: BLE001
            line["cpu_leg_error"] = f"{type(e).__name__}: {e}"[:500]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def warm_start_leg(args, arm, g_ref, plain_ms, flush):
    """The same graph through the learned GNC warm start (the shipped closure
    network), HBM-resident inputs, timed like `value`, in both warm modes:
    RPGO_WARM_ON (predicted inlier set, mu from warm_mu, certified TLS fixed
    point, plain schedule on a failed certificate) and
    RPGO_WARM_CONTINUATION (plain GNC's mu continuation, first weights from
    the prediction, LM from the previous estimate); the inlier decisions
    compared with the plain schedule's (g_ref, the last plain step)."""
    import copy

    import numpy as np

    from rpgo_gb300 import synth, warmstart
    from rpgo_gb300.params import WARM_CONTINUATION, WARM_ON

    model = warmstart.load_model()
    out = {"note": "opt-in (gnc_warm_start); `value` above is the plain schedule"}
    for name, mode in (("certified_fixed_point", WARM_ON), ("continuation", WARM_CONTINUATION)):
        p = copy.copy(arm.params)
        p.setGncWarmStart(mode)
        for _ in range(min(args.warmup, 3)):
            arm.step_dev(p, model)
        steps = max(3, min(args.steps, 8))
        times, g = timed_steps(lambda: arm.step_dev(p, model), steps, flush)
        ms = sum(times) / len(times)
        t = g.timing()
        c = g.counts()
        nk = c.num_odom + c.num_special
        wp, ww = g_ref.gnc_weights()[nk:], g.gnc_weights()[nk:]
        diff = int(np.sum(np.round(wp) != np.round(ww))) if len(wp) == len(ww) else None
        out[name] = {"value": 1000.0 / ms, "unit": "graphs/s", "ms_per_step": ms, "steps": steps,
                     "speedup_vs_plain": plain_ms / ms, "solve_ms": t.solve_ms, "gnc_iterations": t.gnc_iterations,
                     "linear_solves": t.linear_solves, "certified": t.warm_fallbacks == 0,
                     "closures_in_gnc": len(ww), "differing_decisions_vs_plain": diff,
                     "identical_inlier_set": diff == 0,
                     "ate_vs_plain_m": synth.ate(g.estimate()[1], g_ref.estimate()[1], 3), "_solver": g}
    return out


def small_graph_leg(flush):
    """The 5,000-pose graph (1,000 + 333 closures), timed like `value`; the
    solver of its last step comes back for the CPU leg's check."""
    s, params = make_workload("walk3d_5000")
    arm = Arm(s, params)
    for _ in range(3):
        arm.step_dev()
    times, g = timed_steps(arm.step_dev, 10, flush)
    e2e, _ = timed_steps(lambda: arm.step_e2e()[0], 10, flush)
    ms, ems = sum(times) / len(times), sum(e2e) / len(e2e)
    t = g.timing()
    return ({"workload": WORKLOADS["walk3d_5000"][0], "value": 1000.0 / ms, "unit": "graphs/s", "ms_per_step": ms,
             "e2e_value": 1000.0 / ems, "pcm_ms": t.pcm_ms, "solve_ms": t.solve_ms, "linear_solves": t.linear_solves,
             "steps": 10}, (s, params, g))


def _c4_graph(args):
    from rpgo_gb300 import synth

    n, ni, no, s = args
    return synth.walk3d(n, ni, no, seed=s).graph


def batched_leg(params, n_graphs=64, workers=8):
    """rpgo_solve_batch on the first n_graphs graphs of the batched workload
    (512 graphs of 200-8000 poses, closures 10-30 % of the poses, outlier
    rate U[0, 0.5]), against the same graphs solved one at a time."""
    import concurrent.futures as cf
    import multiprocessing

    import numpy as np

    from rpgo_gb300 import capi, synth

    sizes = synth.config_c4_sizes(512)[:n_graphs]
    with cf.ProcessPoolExecutor(8, mp_context=multiprocessing.get_context("spawn")) as ex:
        graphs = list(ex.map(_c4_graph, sizes, chunksize=2))
    # the graphs as the C ABI's host arrays (rpgo_factor_batch), built before the timing
    graphs = [capi.Batch(g) for g in graphs]
    capi.solve_batch(params, graphs[:workers], workers=workers)
    t0 = time.perf_counter()
    res = capi.solve_batch(params, graphs, workers=workers)
    tb = time.perf_counter() - t0
    assert all(r[0] == 0 for r in res)
    # the lock-step form: one launch per stage over all graphs
    capi.solve_batch(params, graphs[:workers], joint=True)
    t0 = time.perf_counter()
    rj = capi.solve_batch(params, graphs, joint=True)
    tj = time.perf_counter() - t0
    assert all(r[0] == 0 for r in rj)
    same = sum(int(np.array_equal(np.round(a[3]), np.round(b[3]))) for a, b in zip(res, rj))
    t0 = time.perf_counter()
    for gr in graphs:
        assert capi.RobustSolver(params).update(gr) == 0
    ts = time.perf_counter() - t0
    return {"value": n_graphs / tb, "unit": "graphs/s", "graphs": n_graphs, "workers": workers,
            "poses": int(sum(x[0] for x in sizes)), "seconds": tb, "one_at_a_time_graphs_per_s": n_graphs / ts,
            "speedup_vs_one_at_a_time": ts / tb,
            "joint": {"value": n_graphs / tj, "seconds": tj, "rounds_solve_ms": float(rj[0][4].solve_ms),
                      "linear_solves_max": int(max(r[4].linear_solves for r in rj)),
                      "linear_solves_sum": int(sum(r[4].linear_solves for r in rj)),
                      "graphs_with_worker_inlier_set": same},
            "workload": "first 64 graphs of the 512-graph batch (seed 4): 3d random walks of 200-8000 poses, "
                        "closures 10-30 % of the poses, outlier rate U[0, 0.5]; wall clock, host to host from the "
                        "C ABI's host arrays"}


# ------------------------------------------------------------------ CPU leg (oracle: timing sample + checks)
def _clique_scan_seconds(A, n, O, budget_s=1.5):
    """Seconds the reference's linear-search clique would take on the n x n
    matrix A: its inner-iteration count (estimated on bit rows, each kept
    element's position to its 64-bit word) times the time per iteration of
    the linear search itself, measured on the largest leading sub-matrix
    whose predicted run time (from its own exact iteration count) stays
    within budget_s."""
    import numpy as np

    def sub(m):
        w = (m + 31) // 32
        x = np.ascontiguousarray(A[:m, :w])
        if m % 32:
            x[:, -1] &= np.uint32((1 << (m % 32)) - 1)
        return x

    ops = O.clique_scan_ops(A, n, exact=False)
    before = O.set_clique_impl(0)
    try:
        m = min(n, 128)
        x = sub(m)
        sub_ops = O.clique_scan_ops(x, m)
        t0 = time.perf_counter()
        O.max_clique_heu(x, m)
        dt = time.perf_counter() - t0
        per_op = dt / sub_ops if sub_ops > 0 else 0.0
        while m < n and per_op > 0:
            m2 = min(n, 2 * m)
            x2 = sub(m2)
            ops2 = O.clique_scan_ops(x2, m2)
            if ops2 * per_op > budget_s:
                break
            t0 = time.perf_counter()
            O.max_clique_heu(x2, m2)
            dt = time.perf_counter() - t0
            m, sub_ops = m2, ops2
            per_op = dt / sub_ops if sub_ops > 0 else per_op
    finally:
        O.set_clique_impl(before)
    return ops * per_op, {"ops": ops, "ns_per_op": 1e9 * per_op, "timed_on_closures": m, "timed_s": dt,
                          "timed_ops": sub_ops}


def cpu_leg(args, s, params, gpu, warm, c2):
    """The CPU FP64 restatement of the reference path (oracle/), as the
    checker and as the CPU baseline.

    cpu_baseline (1 thread, kind "port"): a bounded sample of the graph's
    work, each part priced by its exact unit count: (a) pair tests of 16
    whole rows of the consistency matrix, scaled to all L(L-1)/2 pairs; (b)
    the reference's linear-search greedy clique: its inner-iteration count on
    this run's matrix times the time per iteration measured on a leading
    sub-matrix; (c) damped LM solves (linearise, factor, solve, retract,
    cost) on this run's filtered graph, one LM iteration, scaled to the
    linear-solve count of the GNC schedule (equal to the oracle's when the
    parity check passes). parity: oracle/parity.py on this run's result
    (all host threads)."""
    import numpy as np

    from oracle import parity
    from oracle import rpgo_oracle as O

    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    # ---- checks (all host threads)
    rows = None if args.workload == "walk3d_5000" else 256
    rep = parity.check(s.graph, params, gpu, rows=rows, seed=3, keep=True)
    par = {"workload": WORKLOADS[args.workload][0], "passed": parity.passed(rep)}
    par.update({k: v for k, v in rep.items() if not k.startswith("_")})
    if warm is not None and "_oracle" in rep:
        from rpgo_gb300 import synth

        o = rep["_oracle"]
        ko, po = o.estimate()
        par["warm_start"] = {}
        for name, leg in warm.items():
            if not isinstance(leg, dict) or "_solver" not in leg:
                continue
            g = leg["_solver"]
            nk = int(g.counts().num_odom + g.counts().num_special)
            wo, ww = o.gnc_weights()[nk:], g.gnc_weights()[nk:]
            same = len(wo) == len(ww)
            par["warm_start"][name] = {
                "identical_inlier_set_vs_oracle": bool(same and np.array_equal(np.round(wo), np.round(ww))),
                "differing_decisions_vs_oracle": int(np.sum(np.round(wo) != np.round(ww))) if same else None,
                "ate_vs_oracle_m": synth.ate(g.estimate()[1], po, 3)}
    if c2 is not None:
        s2, p2, g2 = c2
        r2 = parity.check(s2.graph, p2, g2, rows=None)
        par["walk3d_5000"] = {"passed": parity.passed(r2)}
        par["walk3d_5000"].update({k: v for k, v in r2.items() if not k.startswith("_")})
    # ---- CPU baseline sample (one thread; the pricing of the reference's
    # linear-search clique runs on all threads first, its timed sample is
    # sequential anyway)
    A = gpu.adjacency(0)
    n_all = 0 if A is None else A.shape[0]
    t_scan, cinfo = _clique_scan_seconds(A, n_all, O) if n_all else (0.0, {"ops": 0, "ns_per_op": 0.0})
    before = O.set_threads(1)
    try:
        # the greedy clique of this run's matrix, bit-row form, one thread
        old_impl = O.set_clique_impl(2)
        try:
            t0 = time.perf_counter()
            if n_all:
                O.max_clique_heu(A, n_all)
            t_clique = time.perf_counter() - t0
        finally:
            O.set_clique_impl(old_impl)
        n, _, _ = O.OracleSolver(params).pcm_rows(s.graph, [])
        sel = np.sort(np.random.default_rng(5).choice(n, min(16, n), replace=False)).astype(np.int32)
        t0 = time.perf_counter()
        O.OracleSolver(params).pcm_rows(s.graph, sel)
        t_rows = time.perf_counter() - t0
        pairs_per_s = len(sel) * (n - 1) / t_rows
        t_pairs = n * (n - 1) / 2 / pairs_per_s
        kind, k1, k2, _ = gpu.factors()
        c = gpu.counts()
        fg = O.filtered_graph(s.graph, kind, k1, k2)
        lm_params = type(params)()
        lm_params.__dict__.update(params.__dict__)
        lm_params.use_gnc = 0
        old_cap = O.set_lm_max_iterations(1)
        try:
            o = O.OracleSolver(lm_params)
            t0 = time.perf_counter()
            assert o.solve_graph(fg, int(c.num_odom + c.num_special)) == 0
            t_lm = time.perf_counter() - t0
            st = o.stats()
        finally:
            O.set_lm_max_iterations(old_cap)
        per_solve = t_lm / max(1, st["linear_solves"])
        n_solves = int(gpu.timing().linear_solves)
        t_solve = per_solve * n_solves
    finally:
        O.set_threads(before)
    full = t_pairs + t_clique + t_solve
    cb = {"value": 1.0 / full, "unit": "graphs/s", "cores": 1, "kind": "port",
          "sample": (f"CPU FP64 restatement of the reference path, 1 thread: pair tests of {len(sel)} whole rows of "
                     f"the {n}-closure consistency matrix ({t_rows:.2f} s, {pairs_per_s:.3g} pairs/s, scaled to "
                     f"{n * (n - 1) // 2} pairs: {t_pairs:.0f} s); the greedy clique of this run's matrix in the "
                     f"bit-row form (same decisions as the reference's linear search, {t_clique:.1f} s); one LM "
                     f"iteration on the filtered graph ({st['linear_solves']} damped solves, {per_solve:.3f} s "
                     f"each) x {n_solves} solves of the GNC schedule ({t_solve:.0f} s)"),
          "seconds_per_graph": full, "pairs_s": t_pairs, "clique_s": t_clique, "solve_s": t_solve,
          "reference_linear_search_clique": {
              "seconds": t_scan, **cinfo,
              "note": "the reference's own clique search (linear scans of neighbour lists) priced by its inner "
                      "iteration count, not run and not in `value`"}}
    return cb, par


# ------------------------------------------------------------------ reference arm
def run_reference(args):
    """The CPU FP64 restatement on every host thread, the same graph once,
    cut into K timed slices: slices 1..K-2 the pair tests (row blocks of the
    consistency matrix, each pair once, as the reference's incremental
    fill), slice K-1 the greedy clique (the bit-row form, whose
    decisions equal the reference's linear search), slice K the GNC-TLS / LM
    solve. value = 1 graph / the summed slice times. The warm-up steps are
    samples of 8 rows each."""
    import numpy as np

    dist_rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if dist_rank != 0:
        return
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    from oracle import rpgo_oracle as O

    threads = O.set_threads(os.cpu_count() or 1)
    s, params = make_workload(args.workload)
    graph = s.graph
    K = max(3, args.steps)
    n, src, _ = O.OracleSolver(params).pcm_rows(graph, [])
    words = (n + 31) // 32
    rng = np.random.default_rng(1)
    for _ in range(args.warmup):
        O.OracleSolver(params).pcm_rows(graph, rng.choice(n, min(8, n), replace=False).astype(np.int32))
    # row blocks with equal pair counts (row r adds r pairs)
    n_pair_slices = K - 2
    cuts = [int(round(n * np.sqrt(k / n_pair_slices))) for k in range(n_pair_slices + 1)]
    A = np.zeros((n, words), dtype=np.uint32)
    times = []
    for k in range(n_pair_slices):
        rows = np.arange(cuts[k], cuts[k + 1], dtype=np.int32)
        t0 = time.perf_counter()
        _, _, bits = O.OracleSolver(params).pcm_rows(graph, rows, lower_only=True)
        times.append(time.perf_counter() - t0)
        A[rows] = bits
    # mirror the lower triangle (not timed: the reference sets both bits in the same loop)
    Ab = np.unpackbits(A.view(np.uint8), axis=1, bitorder="little")[:, :n]
    Ab |= Ab.T
    A = np.packbits(np.pad(Ab, ((0, 0), (0, words * 32 - n))), axis=1, bitorder="little").view(np.uint32)
    del Ab
    before = O.set_clique_impl(2)
    try:
        t0 = time.perf_counter()
        size, idx = O.max_clique_heu(A, n)
        times.append(time.perf_counter() - t0)
    finally:
        O.set_clique_impl(before)
    kept = [int(src[i]) for i in idx[:size] if i < n]
    n_known = s.n_odom + 1
    from rpgo_gb300.graph import Graph

    fg = Graph(3)
    for j in list(range(n_known)) + kept:
        fg.kind.append(graph.kind[j])
        fg.key1.append(graph.key1[j])
        fg.key2.append(graph.key2[j])
        fg.measured.append(graph.measured[j])
        fg.cov.append(graph.cov[j])
        fg.sqrt_info.append(graph.sqrt_info[j])
    fg.value_keys, fg.value_poses = list(graph.value_keys), list(graph.value_poses)
    o = O.OracleSolver(params)
    t0 = time.perf_counter()
    assert o.solve_graph(fg, n_known) == 0
    times.append(time.perf_counter() - t0)
    st = o.stats()
    total = sum(times)
    v = 1.0 / total
    scan_s, cinfo = _clique_scan_seconds(A, n, O)
    sample = (f"CPU FP64 restatement of the reference path (the reference needs GTSAM, absent here) on {threads} "
              f"threads, the whole graph once in {K} slices: pair tests {sum(times[:-2]):.1f} s "
              f"({n * (n - 1) // 2} pairs), greedy clique {times[-2]:.1f} s (bit-row form, same decisions "
              f"as the reference's linear search), GNC-TLS solve {times[-1]:.1f} s ({st['gnc_iterations']} outer "
              f"iterations, {st['linear_solves']} damped solves)")
    line = {
        "metric": METRIC, "value": v, "unit": "graphs/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": 1000.0 * total / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded 3d random walk; no public dataset in the "
                                                   "reference)",
        "config": bench_config(args.workload, world),
        "impl": "reference",
        "graphs_per_step": 1.0 / K,
        "slice_seconds": [round(t, 3) for t in times],
        "cpu_baseline": {"value": v, "unit": "graphs/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "graphs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_clique": {"value_with_linear_search": 1.0 / (total - times[-2] + scan_s),
                             "linear_search_s": scan_s, **cinfo,
                             "note": "the reference's linear-search clique priced by its exact inner-iteration count "
                                     "(not run); `value` uses the bit-row form's measured time instead"},
    }
    print(json.dumps(line), flush=True)


def run_batch512(args):
    """The batched workload: 512 graphs (seed 4: 3d random walks of 200-8000
    poses, closures 10-30 % of the poses, outlier rate U[0, 0.5]) through
    rpgo_solve_batch; one step = 64 consecutive graphs of the 512 (steps 8
    cover them all), timed host to host. Every step's graphs are new to the
    device (their measurements arrive from host memory), so no L2 flush is
    needed."""
    import concurrent.futures as cf
    import multiprocessing

    import torch

    from rpgo_gb300 import build, capi, synth
    from rpgo_gb300.params import QUIET, RobustSolverParams

    build()
    capi.load()
    params = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    sizes = synth.config_c4_sizes(512)
    with cf.ProcessPoolExecutor(8, mp_context=multiprocessing.get_context("spawn")) as ex:
        graphs = list(ex.map(_c4_graph, sizes, chunksize=4))
    # the graphs as the C ABI's host arrays (rpgo_factor_batch), built before the timing
    graphs = [capi.Batch(g) for g in graphs]
    per = 64
    chunks = [graphs[i:i + per] for i in range(0, 512, per)]
    tuned = None
    if args.workers > 0:
        cfg = {"workers": args.workers, "coop_ctas": args.coop_ctas}
    else:
        # autotune the form (worker threads or lock-step groups) and its sizes
        # on 24 graphs drawn from across the batch
        cfg, tuned = capi.autotune_batch(params, graphs[::21][:24])
    for w in range(args.warmup):
        capi.solve_batch(params, chunks[w % len(chunks)][:16], **cfg)
    times, n = [], 0
    with ClockSampler(0) as clocks:
        for k in range(args.steps):
            chunk = chunks[k % len(chunks)]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = capi.solve_batch(params, chunk, **cfg)
            times.append(time.perf_counter() - t0)
            assert all(r[0] == 0 for r in res)
            n += len(chunk)
    sec = sum(times)
    line = {"metric": METRIC, "value": n / sec, "unit": "graphs/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * sec / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded 3d random walks)",
            "config": {"workload": "batch of 512 independent graphs (200-8000 poses, closures 10-30 %, outlier rate "
                                   "U[0, 0.5]); a step = 64 graphs through rpgo_solve_batch or rpgo_solve_batch_joint",
                       "graphs_timed": n, "poses_timed": int(sum(sz[0] for sz in sizes[:n])) if n <= 512 else None,
                       "batch_form": cfg,
                       "autotune_s": {k: round(t, 3) for k, t in tuned.items()} if tuned else None,
                       "l2": "not flushed: every step's graphs arrive from host memory",
                       "parallelism": "single GPU, concurrent graphs"},
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU leg (baseline sample and checks)")
    ap.add_argument("--no-extras", action="store_true", help="skip the warm-start, 5,000-pose and batched legs")
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=["walk3d_50000", "walk3d_5000", "batch512"],
                    help="walk3d_50000: the benchmark graph (default); the others are separate measurements")
    ap.add_argument("--workers", type=int, default=0,
                    help="host threads of the batch512 workload (0: autotuned with the CTA budget)")
    ap.add_argument("--coop-ctas", dest="coop_ctas", type=int, default=0, help="batch512: CTAs per direct solve")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        if args.workload == "batch512":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm runs the single-graph "
                                                                  "workloads"}), flush=True)
            return
        run_reference(args)
    elif args.workload == "batch512":
        run_batch512(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()

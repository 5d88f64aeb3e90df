"""Train the GNC warm-start network and evaluate it against plain GNC.

    python -m rpgo_gb300.train_warmstart [--closures 1000000] [--c3-graphs 6]
        [--epochs 30] [--out warmstart_model.npy] [--eval 2] [--json result.json]

Training data: closures labelled by plain GNC (the RECORD mode of the
solver: its features at the initial values, plain GNC's final weight as the
label) on graphs of the two benchmark generators, with seeds disjoint from
every evaluation graph: `--c3-graphs` 3D random walks of 50,000 poses with
20,000 closures (30 % outliers), then graphs with the batched workload's
size distribution (200-8000 poses, closures 10-30 % of the poses, outlier
rate U[0, 0.5]; every second one also with clustered outliers) until
`--closures` closures are collected. Most graphs are solved with PCM then
GNC; one in ten of those with at most 3,000 poses with the PCM checks
disabled (GNC alone sees every closure, outliers included).

Evaluation: held-out 20,000-pose graphs with 40 % outliers, half uniform and
half clustered (synth.config_c5), PCM then GNC: plain GNC against both warm
modes (the certified fixed point, RPGO_WARM_ON, and the mu-continuation
schedule, RPGO_WARM_CONTINUATION): time, linear solves, GNC iterations,
certificate fallbacks, closures whose inlier decision differs, ATE between
the estimates and against ground truth.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import multiprocessing
import time

import numpy as np

from . import capi, synth, warmstart
from .params import QUIET, WARM_ON, RobustSolverParams


def _params(pcm: bool) -> RobustSolverParams:
    p = RobustSolverParams()
    if pcm:
        p.setPcm3DParams(10.0, 5.0, QUIET)
    else:
        p.setPcm3DParams(-1.0, -1.0, QUIET)
    return p.setGncInlierCostThresholdsAtProbability(0.9)


def _make(args):
    g, (n, ni, no, s) = args
    clu = (no // 2) // 10 * 10 if g % 2 else 0
    pcm = not (g % 10 == 5 and n <= 3000)
    return pcm, synth.walk3d(n, ni, no - clu, seed=s, clustered_outliers=clu)


def _make_c3(seed):
    return True, synth.walk3d(50000, 14000, 6000, seed=seed)


def training_graphs(n_graphs: int, seed: int = 1000, procs: int = 8, start: int = 0):
    sizes = list(enumerate(synth.config_c4_sizes(start + n_graphs, seed)))[start:]
    with cf.ProcessPoolExecutor(procs, mp_context=multiprocessing.get_context("spawn")) as ex:
        return list(ex.map(_make, sizes, chunksize=4))


def collect(graphs, workers: int = 8):
    def one(item):
        pcm, s = item
        return warmstart.collect([s.graph], _params(pcm))

    with cf.ThreadPoolExecutor(workers) as ex:
        parts = list(ex.map(one, graphs))
    X = [p[0] for p in parts if len(p[0])]
    Y = [p[1] for p in parts if len(p[1])]
    if not X:
        return np.zeros((0, capi.MLP_FEATURES), np.float32), np.zeros(0, np.float32)
    return np.concatenate(X), np.concatenate(Y)


def collect_target(closures: int, c3_graphs: int, log=print):
    """Labelled closures from the 50,000-pose generator (seeds 3001+) and the
    batched workload's generator (seeds 1000+), until `closures`."""
    Xs, Ys, n, graphs = [], [], 0, 0
    with cf.ProcessPoolExecutor(min(4, max(1, c3_graphs)), mp_context=multiprocessing.get_context("spawn")) as ex:
        big = list(ex.map(_make_c3, [3001 + k for k in range(c3_graphs)]))
    X, Y = collect(big, workers=2)
    Xs.append(X)
    Ys.append(Y)
    n += len(X)
    graphs += len(big)
    log(f"{graphs} graphs of 50,000 poses: {n} closures")
    start = 0
    while n < closures:
        chunk = training_graphs(200, start=start)
        start += 200
        X, Y = collect(chunk)
        Xs.append(X)
        Ys.append(Y)
        n += len(X)
        graphs += len(chunk)
        log(f"{graphs} graphs: {n} closures")
    return np.concatenate(Xs)[:closures], np.concatenate(Ys)[:closures], graphs


def _solve(s, pcm: bool, model=None, mode=WARM_ON):
    p = _params(pcm)
    if model is not None:
        p.setGncWarmStart(mode)
    g = capi.RobustSolver(p)
    if model is not None:
        g.set_warm_start_model(model)
    t0 = time.perf_counter()
    rc = g.update(s.graph)
    dt = time.perf_counter() - t0
    t = g.timing()
    c = g.counts()
    nk = c.num_odom + c.num_special
    return dict(rc=rc, seconds=dt, solve_ms=t.solve_ms, pcm_ms=t.pcm_ms, linear_solves=t.linear_solves,
                gnc_iterations=t.gnc_iterations, warm_runs=t.warm_runs, warm_fallbacks=t.warm_fallbacks,
                weights=g.gnc_weights()[nk:], poses=g.estimate()[1])


def evaluate(model, n_eval: int = 2, seed: int = 5):
    from .params import WARM_CONTINUATION

    rows = []
    for e in range(n_eval):
        s = synth.config_c5(seed=seed + 100 * e)
        plain = _solve(s, True)
        for mode_name, mode in (("certified_fixed_point", WARM_ON), ("continuation", WARM_CONTINUATION)):
            warm = _solve(s, True, model, mode)
            same = len(plain["weights"]) == len(warm["weights"])
            diff = int(np.sum(np.round(plain["weights"]) != np.round(warm["weights"]))) if same else -1
            rows.append(dict(
                graph=e, mode="pcm+gnc", warm_mode=mode_name, closures=int(s.n_lc),
                plain_s=plain["seconds"], warm_s=warm["seconds"], speedup=plain["seconds"] / warm["seconds"],
                plain_solves=plain["linear_solves"], warm_solves=warm["linear_solves"],
                plain_gnc_iterations=plain["gnc_iterations"], warm_gnc_iterations=warm["gnc_iterations"],
                warm_fallbacks=warm["warm_fallbacks"], differing_decisions=diff,
                identical_inlier_set=diff == 0,
                ate_warm_vs_plain=synth.ate(warm["poses"], plain["poses"], 3),
                ate_plain_vs_truth=synth.ate(plain["poses"], s.gt, 3),
                ate_warm_vs_truth=synth.ate(warm["poses"], s.gt, 3)))
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--closures", type=int, default=1_000_000)
    ap.add_argument("--c3-graphs", dest="c3_graphs", type=int, default=6)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", default=warmstart.MODEL_PATH)
    ap.add_argument("--eval", type=int, default=2)
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    t0 = time.time()
    X, Y, n_graphs = collect_target(a.closures, a.c3_graphs, log=lambda m: print(m, flush=True))
    print(f"collected {len(X)} closures from {n_graphs} graphs ({Y.mean():.3f} kept by plain GNC) in "
          f"{time.time() - t0:.1f} s", flush=True)
    t0 = time.time()
    params = warmstart.train(X, Y, epochs=a.epochs, batch=a.batch, lr=a.lr, log=lambda m: print(m, flush=True))
    prob = warmstart.predict(params, X)
    acc = float(np.mean((prob >= 0.5) == (Y > 0.5)))
    print(f"trained in {time.time() - t0:.1f} s, training accuracy {acc:.4f}", flush=True)
    warmstart.save_model(params, a.out)
    res = dict(train_closures=int(len(X)), train_graphs=n_graphs, train_accuracy=acc,
               kept_fraction=float(Y.mean()), epochs=a.epochs, train_seconds=time.time() - t0)
    if a.eval:
        res["eval"] = evaluate(params, a.eval)
        for r in res["eval"]:
            print(json.dumps(r), flush=True)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()

"""Train the GNC warm-start network and evaluate it against plain GNC.

    python -m rpgo_gb300.train_warmstart [--graphs 400] [--epochs 30]
        [--out warmstart_model.npy] [--eval 2] [--json result.json]

Training data: 3D random-walk graphs with the batched workload's size
distribution (200-8000 poses, closures 10-30 % of the poses, outlier rate
U[0, 0.5]; half of the graphs also get clustered outliers), seeds disjoint
from every evaluation graph; every second graph is solved with PCM then GNC,
the others with the PCM checks disabled (GNC alone sees every closure).
Labels are plain GNC's final weights (the RECORD mode of the solver).

Evaluation: held-out 20,000-pose graphs with 40 % outliers, half uniform and
half clustered (synth.config_c5), plain vs warm-started GNC in both modes:
time, linear solves, GNC iterations, certificate fallbacks, closures whose
inlier decision differs, ATE between the two estimates and against ground
truth.
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
    return g % 2 == 0, synth.walk3d(n, ni, no - clu, seed=s, clustered_outliers=clu)


def training_graphs(n_graphs: int, seed: int = 1000, procs: int = 8):
    sizes = list(enumerate(synth.config_c4_sizes(n_graphs, seed)))
    with cf.ProcessPoolExecutor(procs, mp_context=multiprocessing.get_context("spawn")) as ex:
        return list(ex.map(_make, sizes, chunksize=4))


def collect(graphs, workers: int = 8):
    def one(item):
        pcm, s = item
        return warmstart.collect([s.graph], _params(pcm))

    with cf.ThreadPoolExecutor(workers) as ex:
        parts = list(ex.map(one, graphs))
    X = np.concatenate([p[0] for p in parts if len(p[0])])
    Y = np.concatenate([p[1] for p in parts if len(p[1])])
    return X, Y


def _solve(s, pcm: bool, model=None):
    p = _params(pcm)
    if model is not None:
        p.setGncWarmStart(WARM_ON)
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
    rows = []
    for e in range(n_eval):
        s = synth.config_c5(seed=seed + 100 * e)
        for pcm in (True, False):
            plain = _solve(s, pcm)
            warm = _solve(s, pcm, model)
            same = len(plain["weights"]) == len(warm["weights"])
            diff = int(np.sum(np.round(plain["weights"]) != np.round(warm["weights"]))) if same else -1
            rows.append(dict(
                graph=e, mode="pcm+gnc" if pcm else "gnc", closures=int(s.n_lc),
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
    ap.add_argument("--graphs", type=int, default=400)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", default=warmstart.MODEL_PATH)
    ap.add_argument("--eval", type=int, default=2)
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    t0 = time.time()
    graphs = training_graphs(a.graphs)
    print(f"generated {len(graphs)} graphs in {time.time() - t0:.1f} s", flush=True)
    t0 = time.time()
    X, Y = collect(graphs)
    print(f"collected {len(X)} closures ({Y.mean():.3f} kept by plain GNC) in {time.time() - t0:.1f} s", flush=True)
    t0 = time.time()
    params = warmstart.train(X, Y, epochs=a.epochs, batch=a.batch, lr=a.lr, log=lambda m: print(m, flush=True))
    prob = warmstart.predict(params, X)
    acc = float(np.mean((prob >= 0.5) == (Y > 0.5)))
    print(f"trained in {time.time() - t0:.1f} s, training accuracy {acc:.4f}", flush=True)
    warmstart.save_model(params, a.out)
    res = dict(train_closures=int(len(X)), train_graphs=len(graphs), train_accuracy=acc,
               kept_fraction=float(Y.mean()), epochs=a.epochs)
    if a.eval:
        res["eval"] = evaluate(params, a.eval)
        for r in res["eval"]:
            print(json.dumps(r), flush=True)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()

"""Batched solve of independent graphs (rpgo_solve_batch) through the C ABI.

Each graph of the batch must give what its own RobustSolver.update gives:
the same GNC inlier set and the same poses (the batch runs the same kernels,
concurrently, with the cooperative direct solve on fewer CTAs), and the
oracle's result for a graph checked against the CPU FP64 oracle.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import rpgo_oracle as O
from rpgo_gb300 import capi, synth
from rpgo_gb300.params import GN, LINEAR_PCG, QUIET, RobustSolverParams

ATE_TOL = 1e-4
SIZES = [(200, 30, 10, 41), (350, 60, 20, 42), (500, 80, 30, 43), (300, 40, 0, 44), (450, 70, 35, 45),
         (250, 30, 25, 46), (600, 90, 10, 47)]


def _params():
    return RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)


def test_batch_argument_checks_need_no_gpu():
    lib = capi.load()
    p = capi.params_struct(_params())
    assert lib.rpgo_solve_batch(C.byref(p), 0, None, None, 0, 0, None) == 0
    assert lib.rpgo_solve_batch(C.byref(p), -1, None, None, 0, 0, None) != 0
    assert lib.rpgo_solve_batch(C.byref(p), 2, None, None, 0, 0, None) != 0
    assert lib.rpgo_solve_batch_joint(C.byref(p), 0, None, None, 0, 0, None) == 0
    assert lib.rpgo_solve_batch_joint(C.byref(p), -1, None, None, 0, 0, None) != 0
    assert lib.rpgo_solve_batch_joint(C.byref(p), 2, None, None, 0, 0, None) != 0


@pytest.mark.gpu
@pytest.mark.parametrize("workers,ctas", [(3, 0), (7, 8), (1, 0)])
def test_batch_equals_individual_solves(workers, ctas):
    from rpgo_gb300 import build

    build()
    graphs = [synth.walk3d(n, ni, no, seed=s) for n, ni, no, s in SIZES]
    res = capi.solve_batch(_params(), [s.graph for s in graphs], workers=workers, coop_ctas=ctas)
    assert len(res) == len(graphs)
    for s, (status, keys, poses, w, t) in zip(graphs, res):
        assert status == 0
        g = capi.RobustSolver(_params())
        assert g.update(s.graph) == 0
        k1, p1 = g.estimate()
        assert np.array_equal(keys, k1)
        assert np.array_equal(np.round(w), np.round(g.gnc_weights()))
        assert synth.ate(poses, p1, 3) <= ATE_TOL
        np.testing.assert_allclose(poses, p1, rtol=1e-6, atol=1e-9)
        assert t.gnc_iterations > 0 and t.kernel_launches > 0


def _check_against_oracle(params, graphs, res, dim=3):
    for s, (status, keys, poses, w, t) in zip(graphs, res):
        assert status == 0
        o = O.OracleSolver(params)
        assert o.update(s.graph) == 0
        ko, po = o.estimate()
        assert np.array_equal(keys, ko)
        assert np.array_equal(np.round(w), np.round(o.gnc_weights()))
        assert synth.ate(poses, po, dim) <= ATE_TOL


@pytest.mark.gpu
def test_batch_graph_matches_oracle():
    from rpgo_gb300 import build

    build()
    graphs = [synth.walk3d(n, ni, no, seed=s) for n, ni, no, s in [(400, 60, 20, 48), (300, 50, 30, 49),
                                                                 (550, 90, 20, 50)]]
    res = capi.solve_batch(_params(), [s.graph for s in graphs], workers=2, coop_ctas=16)
    _check_against_oracle(_params(), graphs, res)


@pytest.mark.gpu
@pytest.mark.parametrize("group,streams", [(0, 1), (3, 0), (2, 3)])
def test_joint_batch_matches_oracle_and_individual_solves(group, streams):
    # lock-step solves (one launch per stage over all graphs of a group): each
    # graph's inlier set equals the oracle's and its own update's, poses
    # within the oracle tolerance and close to its own update's (the error
    # sums and the dense-tail-free plan round differently)
    from rpgo_gb300 import build

    build()
    graphs = [synth.walk3d(n, ni, no, seed=s) for n, ni, no, s in SIZES]
    res = capi.solve_batch(_params(), [s.graph for s in graphs], joint=True, group=group, streams=streams)
    _check_against_oracle(_params(), graphs, res)
    for s, (status, keys, poses, w, t) in zip(graphs, res):
        g = capi.RobustSolver(_params())
        assert g.update(s.graph) == 0
        k1, p1 = g.estimate()
        assert np.array_equal(keys, k1)
        assert np.array_equal(np.round(w), np.round(g.gnc_weights()))
        assert synth.ate(poses, p1, 3) <= ATE_TOL
        assert t.gnc_iterations == g.timing().gnc_iterations
        assert t.linear_solves > 0 and t.solve_ms > 0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["gn", "lm_only", "bias_odom", "no_closures", "pcg"])
def test_joint_batch_modes_match_oracle(mode):
    # Gauss-Newton under GNC, plain LM without GNC, GNC with odometry-biased
    # first weights, graphs whose closures PCM rejects entirely, and the PCG
    # solver (each graph then solved on its solver's own path)
    from rpgo_gb300 import build

    build()
    p = _params()
    sizes = SIZES[:4]
    if mode == "gn":
        p.setSolver(GN)
    elif mode == "lm_only":
        p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET)
    elif mode == "bias_odom":
        p.gnc_bias_odom = 1
    elif mode == "pcg":
        p.setLinearSolver(LINEAR_PCG)
    else:
        p = RobustSolverParams().setPcm3DParams(0.0, 0.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    graphs = [synth.walk3d(n, ni, no, seed=s) for n, ni, no, s in sizes]
    res = capi.solve_batch(p, [s.graph for s in graphs], joint=True)
    _check_against_oracle(p, graphs, res)


@pytest.mark.gpu
def test_joint_batch_graph_replay_equals_stage_launches():
    # the rounds replayed from one captured CUDA graph run the same kernels
    # on the same data as stage-by-stage launches: identical results
    from rpgo_gb300 import build

    build()
    lib = capi.load()
    graphs = [synth.walk3d(n, ni, no, seed=s) for n, ni, no, s in SIZES[:4]]
    r0 = lib.rpgo_joint_graph_rounds()
    res_g = capi.solve_batch(_params(), [s.graph for s in graphs], joint=True, streams=1)
    replayed = lib.rpgo_joint_graph_rounds() - r0
    old = lib.rpgo_set_joint_graphs(0)
    try:
        res_s = capi.solve_batch(_params(), [s.graph for s in graphs], joint=True, streams=1)
    finally:
        lib.rpgo_set_joint_graphs(old)
    assert replayed > 0
    for a, b in zip(res_g, res_s):
        assert a[0] == 0 and b[0] == 0
        assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])
        assert a[4].linear_solves == b[4].linear_solves


@pytest.mark.gpu
def test_joint_batch_2d_matches_oracle():
    # SE(2) graphs (PCM2D, 3x3 blocks) through the lock-step batch
    from rpgo_gb300 import build

    build()
    p = RobustSolverParams().setPcm2DParams(3.0, 3.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    graphs = [synth.grid2d(n, ni, no, seed=s) for n, ni, no, s in [(300, 60, 12, 61), (500, 100, 20, 62),
                                                                 (200, 30, 6, 63)]]
    res = capi.solve_batch(p, [s.graph for s in graphs], joint=True, streams=2)
    _check_against_oracle(p, graphs, res, dim=2)

"""The benchmark configurations on the GPU against the CPU FP64 oracle.

  * 2D grid walk, 500 poses, 100 inlier + 20 outlier closures, PCM2D(1.0,
    1.0), LM: the oracle's whole update, compared end to end;
  * 3D random walk, 5,000 poses, 1,000 + 333 closures, PCM3D(10, 5) then
    GNC-TLS at probability 0.9: the oracle's whole update, end to end, and
    the stage-by-stage check (whole consistency matrix);
  * 3D random walk, 50,000 poses, 14,000 + 6,000 closures (2e8 pair checks),
    same solver: stage by stage (256 seeded whole rows of the consistency
    matrix, the oracle's clique of the GPU's matrix, the oracle's GNC-TLS /
    LM over the GPU's filtered graph).

Bit-exact: adjacency bits, clique index lists (factor lists), inlier sets;
poses within ATE 1e-4 m and 1e-6 relative per entry.
"""
import numpy as np
import pytest

from oracle import parity
from oracle import rpgo_oracle as O
from rpgo_gb300 import capi, synth
from rpgo_gb300.params import QUIET, RobustSolverParams

pytestmark = pytest.mark.gpu

ATE_TOL = 1e-4
POSE_RTOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from rpgo_gb300 import build

    build()
    capi.load()


def _pcm_gnc_3d():
    return RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)


def _end_to_end(params, graph, dim):
    before = O.set_clique_impl(1)
    try:
        o = O.OracleSolver(params)
        assert o.update(graph) == 0
    finally:
        O.set_clique_impl(before)
    g = capi.RobustSolver(params)
    assert g.update(graph) == 0
    ao, ag = o.adjacency(0), g.adjacency(0)
    assert ao is not None and ag is not None and np.array_equal(ao, ag), "consistency matrix differs"
    for x, y in zip(o.factors()[:3], g.factors()[:3]):
        assert np.array_equal(x, y), "factor list (clique order) differs"
    co, cg = o.counts(), g.counts()
    assert (co.num_lc, co.num_lc_inliers, co.num_factors) == (cg.num_lc, cg.num_lc_inliers, cg.num_factors)
    assert np.array_equal(np.round(o.gnc_weights()), np.round(g.gnc_weights()))
    ko, po = o.estimate()
    kg, pg = g.estimate()
    assert np.array_equal(ko, kg)
    assert synth.ate(pg, po, dim) <= ATE_TOL
    assert np.max(np.abs(pg - po) / np.maximum(1.0, np.abs(po))) <= POSE_RTOL
    return o, g


def test_config_2d_grid_500_pcm_1_1_lm():
    s = synth.config_c1()
    p = RobustSolverParams().setPcm2DParams(1.0, 1.0, QUIET)
    o, g = _end_to_end(p, s.graph, 2)
    # the odometry check at 1.0 already drops most of the 120 closures; the
    # rest reach the pairwise check
    assert 0 < g.counts().num_lc <= 120 and g.counts().num_lc_inliers > 0
    assert g.counts().num_lc == o.counts().num_lc


def test_config_3d_walk_5000_pcm_gnc():
    s = synth.config_c2()
    o, g = _end_to_end(_pcm_gnc_3d(), s.graph, 3)
    # the closures that pass the odometry check (1,003 of 1,333) form the group
    assert 0 < g.counts().num_lc <= 1333 and g.counts().num_lc == o.counts().num_lc
    t = g.timing()
    assert t.gnc_iterations == o.stats()["gnc_iterations"]
    rep = parity.check(s.graph, _pcm_gnc_3d(), g, rows=None)
    assert parity.passed(rep, ATE_TOL, POSE_RTOL), rep
    assert rep["adjacency_rows_checked"] == rep["closures_checked"]


def test_config_3d_walk_50000_stagewise():
    s = synth.config_c3()
    p = _pcm_gnc_3d()
    g = capi.RobustSolver(p)
    assert g.update(s.graph) == 0
    assert 0 < g.counts().num_lc <= 20000
    rep = parity.check(s.graph, p, g, rows=256, seed=3)
    assert rep["closures_checked"] > 10000
    assert parity.passed(rep, ATE_TOL, POSE_RTOL), rep

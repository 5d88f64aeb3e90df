"""Temporary factors and values (GenericSolver.h:46-65; merged into every
optimisation by RobustSolver::optimize, src/RobustSolver.cpp:117-121, their
GNC weights at 169 / 264 and all-ones at 208 / 295; their values updated by
GenericSolver::updateValues, src/GenericSolver.cpp:37-45), restated from the
reference's tests/testTemporary.cpp:24-97 (TemporaryFactors): robot_a with
PCM thresholds high enough to keep every closure and GNC at probability 0.01
rejecting the three closures; a temporary factor and value are added, the
graph is re-optimised, then they are cleared. The EXPECT lines are checked on
the CPU oracle (CPU suite) and on the CUDA library (GPU suite, which also
compares the estimate, the temporary values and weights with the oracle's).
"""
import numpy as np
import pytest

from oracle import rpgo_oracle as O
from rpgo_gb300.graph import Graph, isotropic_variance, pose3, symbol
from rpgo_gb300.params import QUIET, RobustSolverParams


def _params():
    return RobustSolverParams().setPcm3DParams(100.0, 100.0, QUIET).setGncInlierCostThresholdsAtProbability(0.01)


def _temp():
    g = Graph(3)
    g.insert(symbol("b", 0), pose3())
    g.add_between(symbol("a", 0), symbol("b", 0), pose3(), isotropic_variance(6, 0.01))
    return g


def scenario(s, force, robot_a, check=None):
    """Runs the reference test's steps on solver s; returns failed EXPECTs."""
    fails = []

    def expect(cond, what):
        if not cond:
            fails.append(what)

    def closures_rejected(tag):
        w = s.gnc_weights()
        expect(len(w) == 52, f"{tag}: weights {len(w)}")
        expect(w[49:52].sum() == 0, f"{tag}: closure weights {w[49:52]}")
        expect(w.sum() == 49, f"{tag}: weight sum {w.sum()}")

    assert s.update(robot_a) == 0
    c = s.counts()
    expect(c.num_factors == 52 and c.num_values == 50, f"update: sizes {c.num_factors}/{c.num_values}")
    closures_rejected("update")
    expect(c.num_lc_inliers == 0, f"update: lc inliers {c.num_lc_inliers}")
    if check:
        check("update")

    assert s.updateTempFactorsValues(_temp()) == 0
    assert force() == 0
    c = s.counts()
    expect(c.num_factors == 52 and c.num_values == 50, f"temp: sizes {c.num_factors}/{c.num_values}")
    expect(s.temp_sizes() == (1, 1), f"temp: temp sizes {s.temp_sizes()}")
    expect(len(s.gnc_weights()) == 52, "temp: weights")
    expect(len(s.getGncTempWeights()) == 1, "temp: temp weights")
    expect(c.num_lc_inliers == 0, f"temp: lc inliers {c.num_lc_inliers}")
    if check:
        check("temp")

    assert s.clearTempFactorsValues() == 0
    assert force() == 0
    c = s.counts()
    expect(c.num_factors == 52 and c.num_values == 50, f"cleared: sizes {c.num_factors}/{c.num_values}")
    expect(s.temp_sizes() == (0, 0), f"cleared: temp sizes {s.temp_sizes()}")
    closures_rejected("cleared")
    expect(c.num_lc_inliers == 0, f"cleared: lc inliers {c.num_lc_inliers}")
    if check:
        check("cleared")
    return fails


def test_oracle_temporary_factors(robot_a):
    s = O.OracleSolver(_params())
    fails = scenario(s, s.force_optimize, robot_a)
    assert not fails, fails


def test_oracle_temporary_key_rules(robot_a):
    s = O.OracleSolver(_params())
    assert s.update(robot_a) == 0
    g = Graph(3).insert(symbol("a", 0), pose3())  # a key of the graph's values
    assert s.updateTempFactorsValues(g) != 0
    assert s.updateTempFactorsValues(_temp()) == 0
    assert s.updateTempFactorsValues(Graph(3).insert(symbol("b", 0), pose3())) != 0  # already temporary
    assert s.replaceTempFactorsValues(_temp()) == 0  # replacing may reuse it
    assert s.temp_sizes() == (1, 1)
    # a new graph value may not take a temporary key
    assert s.update(Graph(3).insert(symbol("b", 0), pose3())) != 0


@pytest.mark.gpu
def test_gpu_temporary_factors_match_reference_and_oracle(robot_a):
    from rpgo_gb300 import build, capi

    build()
    o = O.OracleSolver(_params())
    assert not scenario(o, o.force_optimize, robot_a)
    g = capi.RobustSolver(_params())
    o2 = O.OracleSolver(_params())
    steps = iter([lambda: 0, lambda: (o2.updateTempFactorsValues(_temp()), o2.force_optimize())[1],
                  lambda: (o2.clearTempFactorsValues(), o2.force_optimize())[1]])
    assert o2.update(robot_a) == 0
    mism = []

    def check(tag):
        if tag != "update":
            assert next(steps)() == 0
        kg, pg = g.estimate()
        ko, po = o2.estimate()
        if not (np.array_equal(kg, ko) and np.allclose(pg, po, rtol=1e-6, atol=1e-8)):
            mism.append((tag, "estimate", float(np.max(np.abs(pg - po)))))
        if not np.array_equal(np.round(g.gnc_weights()), np.round(o2.gnc_weights())):
            mism.append((tag, "weights"))
        if not np.array_equal(np.round(g.getGncTempWeights()), np.round(o2.getGncTempWeights())):
            mism.append((tag, "temp weights", g.getGncTempWeights(), o2.getGncTempWeights()))
        tg, to = g.getTempValues(), o2.getTempValues()
        if not (np.array_equal(tg[0], to[0]) and np.allclose(tg[1], to[1], rtol=1e-6, atol=1e-8)):
            mism.append((tag, "temp values"))

    next(steps)
    fails = scenario(g, lambda: g.forceUpdate(Graph(3)), robot_a, check)
    assert not fails, fails
    assert not mism, mism


def test_oracle_temporary_2d_without_gnc():
    # 2D, PCM without GNC: temporary factors are optimised with the graph,
    # their weights are all ones (src/RobustSolver.cpp:208), the temporary
    # value moves with the solve and the graph's own counts do not change
    from rpgo_gb300 import synth
    from rpgo_gb300.graph import pose2, pose2_compose

    s = synth.grid2d(60, 10, 2, seed=3)
    o = O.OracleSolver(RobustSolverParams().setPcm2DParams(3.0, 3.0, QUIET))
    assert o.update(s.graph) == 0
    n0 = (o.counts().num_factors, o.counts().num_values)
    t = Graph(2)
    t.insert(symbol("z", 0), pose2(0.0, 0.0, 0.0))
    t.add_between(symbol("a", 5), symbol("z", 0), pose2(0.5, -0.25, 0.1), isotropic_variance(3, 0.01))
    assert o.updateTempFactorsValues(t) == 0
    assert o.force_optimize() == 0
    assert (o.counts().num_factors, o.counts().num_values) == n0
    assert np.array_equal(o.getGncTempWeights(), [1.0])
    keys, poses = o.getTempValues()
    assert list(keys) == [symbol("z", 0)]
    # the only factor on z0 is the temporary one: z0 = a5 (+) measurement
    k, est = o.estimate()
    a5 = est[list(k).index(symbol("a", 5))]
    np.testing.assert_allclose(poses[0], pose2_compose(a5, pose2(0.5, -0.25, 0.1)), atol=1e-6)
    assert o.clearTempFactorsValues() == 0 and o.temp_sizes() == (0, 0)

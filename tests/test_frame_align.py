"""Multi-robot frame alignment (Pcm.h:1011-1131, MultiRobotAlignMethod),
restated from the reference's tests/testMultirobotFrameAlign.cpp:21-112:
three robots, inter-robot closures a-b and a-c; after PCM (GNC alignment at
the default probability 0.99) every robot's initial values are expressed in
robot a's frame, to 1e-6. The same update runs on the CPU oracle (CPU suite)
and on the CUDA library (GPU suite, also against the oracle for L2 and GNC
alignment of a larger two-robot graph)."""
import numpy as np
import pytest

from oracle import rpgo_oracle as O
from rpgo_gb300 import synth
from rpgo_gb300.graph import Graph, isotropic_variance, pose3, symbol
from rpgo_gb300.params import ALIGN_GNC, ALIGN_L2, QUIET, RobustSolverParams

R180 = np.diag([-1.0, -1.0, 1.0])


def _params(method=ALIGN_GNC):
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET)
    p.odom_trans_threshold, p.odom_rot_threshold = -1.0, -1.0
    p.dist_trans_threshold, p.dist_rot_threshold = 0.3, 100.0
    return p.setMultiRobotAlignMethod(method)


def _graph():
    s = lambda c, i: symbol(c, i)  # noqa: E731
    noise = isotropic_variance(6, 0.01)
    g = Graph(3)
    g.insert(s("a", 0), pose3())
    g.add_between(s("a", 0), s("a", 1), pose3(), noise)
    g.insert(s("a", 1), pose3())
    g.insert(s("b", 0), pose3(t=(1, 0, 0)))
    g.add_between(s("b", 0), s("b", 1), pose3(t=(1, 0, 0)), noise)
    g.insert(s("b", 1), pose3(t=(2, 0, 0)))
    g.insert(s("c", 0), pose3(R180, (0, 0, 0)))
    g.add_between(s("c", 0), s("c", 1), pose3(t=(1, 0, 0)), noise)
    g.insert(s("c", 1), pose3(R180, (-1, 0, 0)))
    g.add_between(s("a", 0), s("b", 0), pose3(), noise)
    g.add_between(s("a", 1), s("b", 1), pose3(t=(1, 0, 0)), noise)
    g.add_between(s("a", 0), s("c", 0), pose3(), noise)
    g.add_between(s("a", 1), s("c", 1), pose3(t=(1, 0, 0)), noise)
    return g


EXPECTED = {("a", 0): (0, 0, 0), ("a", 1): (0, 0, 0), ("b", 0): (0, 0, 0), ("b", 1): (1, 0, 0),
            ("c", 0): (0, 0, 0), ("c", 1): (1, 0, 0)}


def _check(solver):
    keys, poses = solver.estimate()
    fails = []
    for (c, i), t in EXPECTED.items():
        p = poses[list(keys).index(symbol(c, i))]
        if not (np.allclose(p[:9], np.eye(3).reshape(9), atol=1e-6) and np.allclose(p[9:], t, atol=1e-6)):
            fails.append(f"{c}{i}: {p}")
    return fails


def test_oracle_multirobot_frame_align_reference_test():
    o = O.OracleSolver(_params())
    assert o.update(_graph(), optimize_graph=False) == 0
    assert not _check(o), _check(o)


def _two_robots(seed):
    """Two random walks; b starts 10 m away with an unknown offset in its
    initial values; inter-robot closures from the ground truth, a few wrong."""
    a = synth.walk3d(300, 0, 0, seed=seed, prefix="a")
    b = synth.walk3d(300, 0, 0, seed=seed + 1, prefix="b")
    rng = np.random.default_rng(seed)
    off = np.eye(4)
    off[:3, :3] = synth.so3_exp(rng.normal(0, 0.3, 3))
    off[:3, 3] = (10.0, -4.0, 1.0)
    g = a.graph.copy()
    g.extend(b.graph)
    noise = isotropic_variance(6, 1e-3)
    for _ in range(12):
        i, j = (int(x) for x in rng.integers(0, 300, 2))
        Ta, Tb = synth._T(a.gt[i]), off @ synth._T(b.gt[j])
        g.add_between(symbol("a", i), symbol("b", j), synth._p(np.linalg.inv(Ta) @ Tb), noise)
    for _ in range(3):
        i, j = (int(x) for x in rng.integers(0, 300, 2))
        g.add_between(symbol("a", i), symbol("b", j), synth._p(synth.se3_exp(rng.normal(0, 2, 6))), noise)
    return g


@pytest.mark.gpu
def test_gpu_multirobot_frame_align():
    from rpgo_gb300 import build, capi

    build()
    g = capi.RobustSolver(_params())
    assert g.update(_graph(), optimize_graph=False) == 0
    assert not _check(g), _check(g)
    for method in (ALIGN_GNC, ALIGN_L2):
        p = RobustSolverParams().setPcm3DParams(1e9, 1e9, QUIET).setMultiRobotAlignMethod(method)
        gg, oo = capi.RobustSolver(p), O.OracleSolver(p)
        graph = _two_robots(71)
        assert gg.update(graph, optimize_graph=False) == 0 and oo.update(graph, optimize_graph=False) == 0
        kg, pg = gg.estimate()
        ko, po = oo.estimate()
        assert np.array_equal(kg, ko)
        np.testing.assert_allclose(pg, po, rtol=1e-6, atol=1e-9)

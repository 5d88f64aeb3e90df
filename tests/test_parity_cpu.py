"""The stage-by-stage checker (oracle/parity.py) on the CPU: an oracle update
checked against the oracle passes; planted differences in the matrix, the
factor list, the weights or the estimate are caught."""
import numpy as np

from oracle import parity
from oracle import rpgo_oracle as O
from rpgo_gb300 import synth
from rpgo_gb300.params import QUIET, RobustSolverParams


class _Planted:
    """An oracle solver whose getters can be altered (stands in for the GPU
    solver in the checker)."""

    def __init__(self, o):
        self.o = o
        self.adj = o.adjacency(0)
        self.fac = list(o.factors())
        self.w = o.gnc_weights()
        self.est = o.estimate()

    def adjacency(self, g=0):
        return self.adj

    def counts(self):
        return self.o.counts()

    def factors(self):
        return tuple(self.fac)

    def gnc_weights(self):
        return self.w

    def estimate(self):
        return self.est


def _setup():
    s = synth.walk3d(600, 150, 50, seed=37)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    o = O.OracleSolver(p)
    assert o.update(s.graph) == 0
    return s, p, o


def test_checker_accepts_the_oracle_itself():
    s, p, o = _setup()
    for rows in (None, 40):
        rep = parity.check(s.graph, p, _Planted(o), rows=rows)
        assert parity.passed(rep), rep
        assert rep["ate_vs_oracle_m"] == 0.0 and rep["max_rel_pose_err"] == 0.0


def test_checker_catches_planted_differences():
    s, p, o = _setup()
    # one flipped bit of the matrix (whole-matrix check)
    x = _Planted(o)
    x.adj = x.adj.copy()
    x.adj[3, 0] ^= np.uint32(1 << 5)
    assert not parity.check(s.graph, p, x, rows=None, solve=False)["adjacency_bit_exact"]
    # two kept closures swapped
    x = _Planted(o)
    n_known = int(o.counts().num_odom + o.counts().num_special)
    k1 = x.fac[1].copy()
    k1[[n_known, n_known + 1]] = k1[[n_known + 1, n_known]]
    x.fac[1] = k1
    assert not parity.check(s.graph, p, x, rows=10, solve=False)["clique_equal"]
    # one closure's weight flipped
    x = _Planted(o)
    x.w = x.w.copy()
    x.w[-1] = 1.0 - np.round(x.w[-1])
    assert not parity.check(s.graph, p, x, rows=10)["inlier_set_identical"]
    # an estimate moved by 1 mm at one pose
    x = _Planted(o)
    keys, poses = x.est
    poses = poses.copy()
    poses[100, 9] += 1e-3
    x.est = (keys, poses)
    rep = parity.check(s.graph, p, x, rows=10)
    assert rep["max_rel_pose_err"] > 1e-6 and not parity.passed(rep)

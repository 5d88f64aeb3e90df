"""Landmark PCM (Pcm.h:180-220 classification, 440-454 re-observations,
775-844 pairwise landmark consistency, 878-897 landmark cliques), restated
from the reference's tests/testLandmark.cpp:23-520 (LandmarkPcm,
LandmarkPcmSimple, LandmarkNoReject): the same update sequence and the
EXPECTed graph and value counts, on the CPU oracle (CPU suite) and on the
CUDA library (GPU suite, also checked against the oracle's estimate and
factor list after every step).

The landmark noise model is Diagonal::Precisions(0, 0, 0, 25, 25, 25): its
square-root information is diag(0, 0, 0, 5, 5, 5); its covariance, which PCM
reads, is the inverse of a singular information matrix, whose rotation block
is not a number — the case GeometryUtils.h:103-113 detects (rotation_info
false, translation-only Mahalanobis distance).
"""
import numpy as np
import pytest

from oracle import rpgo_oracle as O
from rpgo_gb300.graph import Graph, isotropic_variance, pose3, rot3_rz, symbol
from rpgo_gb300.params import QUIET, RobustSolverParams

R90 = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
a = lambda i: symbol("a", i)  # noqa: E731
l = lambda i: symbol("l", i)  # noqa: E731,E741


def _landmark_noise():
    cov = np.full((6, 6), np.nan)
    cov[3:, :] = 0.0
    cov[:, 3:] = 0.0
    cov[3:, 3:] = np.eye(3) / 25.0
    R = np.diag([0.0, 0.0, 0.0, 5.0, 5.0, 5.0])
    return cov, R


def _steps(no_reject):
    """(graph, expected num_factors, expected num_values) per update."""
    steps = [(Graph(3).insert(a(0), pose3()), None, None)]
    for i in range(2):
        g = Graph(3).insert(a(i + 1), pose3(t=(1, 0, 0)))
        g.add_between(a(i), a(i + 1), pose3(t=(1, 0, 0)), isotropic_variance(6, 0.1))
        steps.append((g, None, None))
    for i in range(2, 5):
        g = Graph(3).insert(a(i + 1), pose3(R90, (1, 0, 0)))
        g.add_between(a(i), a(i + 1), pose3(R90, (1, 0, 0)), isotropic_variance(6, 0.1))
        steps.append((g, None, None))
    noise = isotropic_variance(6, 0.1)
    lc = Graph(3)
    lc.add_between(a(3), a(2), pose3(rot3_rz(-1.57), (0, 0.9, 0)), noise)
    lc.add_between(a(4), a(1), pose3(rot3_rz(3.14), (2.1, 1.1, 2.5)), noise)
    steps.append((lc, 7 if no_reject else 6, 6))
    ln = _landmark_noise()
    g = Graph(3).add_between(a(1), l(0), pose3(t=(0, 1, 0)), ln)
    g.insert(l(0), pose3(t=(1, 1, 0)))
    steps.append((g, 8 if no_reject else 7, 7))
    if no_reject:
        steps.append((Graph(3).add_between(a(5), l(0), pose3(R90, (0, -1, 0)), ln), 9, 7))
        steps.append((Graph(3).add_between(a(4), l(0), pose3(t=(2, 0, 0)), ln), 10, 7))
    else:
        steps.append((Graph(3).add_between(a(5), l(0), pose3(t=(0, -1, 0)), ln), 8, 7))
        steps.append((Graph(3).add_between(a(4), l(0), pose3(t=(1, 0, 0)), ln), 8, 7))
    g = Graph(3).add_between(a(2), l(1), pose3(t=(0, -1, 0)), ln)
    g.insert(l(1), pose3(t=(1, 1, 0)))
    steps.append((g, 11 if no_reject else 9, 8))
    if no_reject:
        steps.append((Graph(3).add_between(a(5), l(1), pose3(R90, (2, 0, 0)), ln), 12, 8))
    else:
        steps.append((Graph(3).add_between(a(5), l(1), pose3(t=(2, 0, 0)), ln), 10, 8))
    return steps


def _params(kind):
    p = RobustSolverParams()
    if kind == "pcm":
        p.setPcm3DParams(5.0, 2.5, QUIET)
    elif kind == "simple":
        p.setPcmSimple3DParams(0.3, 0.05, QUIET)
    else:
        p.setNoRejection(QUIET)
    p.specialSymbols = ["l"]
    return p


def run(make, kind, check=None):
    s = make(_params(kind))
    fails = []
    for k, (g, nf, nv) in enumerate(_steps(kind == "none")):
        rc = s.update(g)
        if rc != 0:
            fails.append(f"step {k}: status {rc}")
        c = s.counts()
        if nf is not None and (c.num_factors != nf or c.num_values != nv):
            fails.append(f"step {k}: sizes {c.num_factors}/{c.num_values}, expected {nf}/{nv}")
        if check:
            check(k, s)
    return fails, s


@pytest.mark.parametrize("kind", ["pcm", "simple", "none"])
def test_oracle_landmark_reference_tests(kind):
    fails, _ = run(O.OracleSolver, kind)
    assert not fails, fails


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["pcm", "simple", "none"])
def test_gpu_landmark_reference_tests(kind):
    from rpgo_gb300 import build, capi

    build()
    o = O.OracleSolver(_params(kind))
    steps = _steps(kind == "none")
    results = []

    def check(k, s):
        assert o.update(steps[k][0]) == 0
        _, k1, k2, _ = s.factors()
        _, o1, o2, _ = o.factors()
        pg, po = s.estimate()[1], o.estimate()[1]
        # without rejection the graph keeps the conflicting closures and
        # landmark observations; LM then stops (relative decrease < 1e-5) at
        # points that differ by ~1e-6 between the two linear solvers'
        # rounding, hence 1e-5 here instead of the 1e-6 of consistent graphs
        tol = 1e-5 if kind == "none" else 1e-6
        results.append((k, np.array_equal(k1, o1) and np.array_equal(k2, o2),
                        np.allclose(pg, po, rtol=tol, atol=tol), float(np.max(np.abs(pg - po)))))

    fails, _ = run(capi.RobustSolver, kind, check)
    assert not fails, fails
    assert all(r[1] for r in results), [r for r in results if not r[1]]
    assert all(r[2] for r in results), [r for r in results if not r[2]]

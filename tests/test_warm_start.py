"""GNC warm start (no counterpart in the reference).

The warm-started schedule takes predicted inlier probabilities, solves with
the predicted inlier set, then iterates TLS weight updates from mu = warm_mu
(LM from the previous estimate each time) until the weights reproduce
themselves (a fixed point of the TLS rule). It is certified only when that
fixed point keeps >= 75 % of the predicted inliers; otherwise the plain
GncOptimizer schedule runs from the start.

CPU (oracle) tests pin the schedule's semantics; GPU tests check the CUDA
schedule against the oracle's on the same probabilities, through the C ABI.
"""
import numpy as np
import pytest

from oracle import rpgo_oracle as O
from rpgo_gb300 import synth
from rpgo_gb300.params import QUIET, WARM_ON, RobustSolverParams

ATE_TOL = 1e-4


def _params(warm=False, pcm_off=True):
    p = RobustSolverParams()
    if pcm_off:
        p.setPcm3DParams(-1.0, -1.0, QUIET)  # PCM checks disabled: GNC sees every closure
    else:
        p.setPcm3DParams(10.0, 5.0, QUIET)
    p.setGncInlierCostThresholdsAtProbability(0.9)
    if warm:
        p.setGncWarmStart(WARM_ON, 100.0)
    return p


def _graph():
    return synth.walk3d(400, 80, 40, seed=21)


def _plain_oracle(s, pcm_off=True):
    o = O.OracleSolver(_params(pcm_off=pcm_off))
    assert o.update(s.graph) == 0
    c = o.counts()
    return o, c.num_odom + c.num_special


def _warm_oracle(s, probs, pcm_off=True):
    o = O.OracleSolver(_params(True, pcm_off))
    assert o.update(s.graph, optimize_graph=False) == 0
    o.set_warm_probs(probs)
    assert o.force_optimize() == 0
    return o


def test_oracle_warm_with_plain_labels_reproduces_plain():
    s = _graph()
    plain, nk = _plain_oracle(s)
    w = plain.gnc_weights()
    assert (w[nk:] < 0.5).sum() >= 40  # every outlier reached GNC and was rejected
    warm = _warm_oracle(s, w)
    st, sp = warm.stats(), plain.stats()
    assert st["warm_runs"] == 1 and st["warm_fallbacks"] == 0
    assert np.array_equal(np.round(warm.gnc_weights()), np.round(w))
    assert synth.ate(warm.estimate()[1], plain.estimate()[1], 3) <= ATE_TOL
    assert st["linear_solves"] * 5 < sp["linear_solves"]


def test_oracle_warm_falls_back_on_contradicted_prediction():
    s = _graph()
    plain, nk = _plain_oracle(s)
    w = plain.gnc_weights()
    bad = np.ones_like(w)  # every closure predicted inlier, outliers included
    warm = _warm_oracle(s, bad)
    st = warm.stats()
    assert st["warm_runs"] == 1 and st["warm_fallbacks"] == 1
    # the plain schedule reran from the start: identical to plain
    assert np.array_equal(warm.gnc_weights(), w)
    assert synth.ate(warm.estimate()[1], plain.estimate()[1], 3) == 0.0


def test_oracle_warm_probs_of_wrong_size_run_plain():
    s = _graph()
    plain, nk = _plain_oracle(s)
    warm = _warm_oracle(s, np.ones(3))
    assert warm.stats()["warm_runs"] == 0
    assert np.array_equal(warm.gnc_weights(), plain.gnc_weights())


# ------------------------------------------------------------------ GPU schedule vs the oracle's
@pytest.mark.gpu
def test_gpu_warm_schedule_matches_oracle():
    from rpgo_gb300 import build, capi

    build()
    s = _graph()
    plain, nk = _plain_oracle(s)
    w = plain.gnc_weights()
    rng = np.random.default_rng(3)
    for probs in (w, np.where(rng.random(w.size) < 0.05, 1.0 - w, w), np.ones_like(w)):
        g = capi.RobustSolver(_params(True))
        assert g.update(s.graph, optimize_graph=False) == 0
        kind, k1, k2, _ = g.factors()
        ok, ok1, ok2, _ = plain.factors()
        assert np.array_equal(k1, ok1) and np.array_equal(k2, ok2)
        assert g.set_warm_start_probs(probs) == 0
        assert g.forceUpdate(_empty()) == 0
        o = _warm_oracle(s, probs)
        t, so = g.timing(), o.stats()
        assert t.warm_runs == 1
        assert t.warm_fallbacks == so["warm_fallbacks"]
        assert np.array_equal(np.round(g.gnc_weights()), np.round(o.gnc_weights()))
        assert synth.ate(g.estimate()[1], o.estimate()[1], 3) <= ATE_TOL


def _empty():
    from rpgo_gb300.graph import Graph

    return Graph(3)


# ------------------------------------------------------------------ continuation-preserving schedule
def _cont_params(pcm_off=True):
    from rpgo_gb300.params import WARM_CONTINUATION

    p = _params(pcm_off=pcm_off)
    p.setGncWarmStart(WARM_CONTINUATION)
    return p


def _cont_oracle(s, probs, pcm_off=True):
    o = O.OracleSolver(_cont_params(pcm_off))
    assert o.update(s.graph, optimize_graph=False) == 0
    if probs is not None:
        o.set_warm_probs(probs)
    assert o.force_optimize() == 0
    return o


def test_oracle_continuation_schedule_keeps_mu_path():
    # same mu continuation and weight rule as plain GNC: with all closures
    # predicted inliers the first solve is plain GNC's, and fewer damped
    # solves follow (LM from the previous estimate)
    s = _graph()
    plain, nk = _plain_oracle(s)
    ones = np.ones(plain.counts().num_factors)
    cont = _cont_oracle(s, ones)
    sp, sc = plain.stats(), cont.stats()
    assert sc["warm_runs"] == 1 and sc["gnc_iterations"] >= 1
    assert sc["linear_solves"] < sp["linear_solves"]
    # probabilities of the wrong size are ignored (first weights all ones)
    again = _cont_oracle(s, np.ones(3))
    assert np.array_equal(again.gnc_weights(), cont.gnc_weights())
    # a predicted outlier set changes the first solve
    zeros = ones.copy()
    zeros[nk:] = 0.0
    other = _cont_oracle(s, zeros)
    assert other.stats()["linear_solves"] != sc["linear_solves"]


@pytest.mark.gpu
def test_gpu_continuation_schedule_matches_oracle():
    from rpgo_gb300 import build, capi

    build()
    s = _graph()
    plain, nk = _plain_oracle(s)
    w = plain.gnc_weights()
    for probs in (w, np.ones_like(w)):
        g = capi.RobustSolver(_cont_params())
        assert g.update(s.graph, optimize_graph=False) == 0
        assert g.set_warm_start_probs(probs) == 0
        assert g.forceUpdate(_empty()) == 0
        o = _cont_oracle(s, probs)
        t, so = g.timing(), o.stats()
        assert t.warm_runs == 1 and t.gnc_iterations == so["gnc_iterations"]
        assert np.array_equal(np.round(g.gnc_weights()), np.round(o.gnc_weights()))
        assert synth.ate(g.estimate()[1], o.estimate()[1], 3) <= ATE_TOL


# ------------------------------------------------------------------ the trained network
@pytest.mark.gpu
@pytest.mark.parametrize("pcm_off", [False, True])
def test_trained_network_gain(pcm_off):
    """The shipped network against the method without it, on a held-out
    graph (seed outside the training and evaluation seeds): plain GNC, and
    the warm schedule started from 'every closure is an inlier'."""
    from rpgo_gb300 import build, capi, warmstart

    build()
    model = warmstart.load_model()
    s = synth.walk3d(800, 120, 40, seed=77, clustered_outliers=40)
    plain = capi.RobustSolver(_params(False, pcm_off))
    assert plain.update(s.graph) == 0
    wp, tp = plain.gnc_weights(), plain.timing()
    warm = capi.RobustSolver(_params(True, pcm_off))
    assert warm.set_warm_start_model(model) == 0
    assert warm.update(s.graph) == 0
    ww, tw = warm.gnc_weights(), warm.timing()
    c = plain.counts()
    nk = c.num_odom + c.num_special
    agree = float(np.mean(np.round(ww[nk:]) == np.round(wp[nk:])))
    print(f"pcm_off={pcm_off}: plain {tp.linear_solves} solves / {tp.gnc_iterations} GNC iterations, "
          f"warm {tw.linear_solves} / {tw.gnc_iterations}, fallbacks {tw.warm_fallbacks}, agreement {agree:.4f}")
    assert tw.warm_runs == 1 and tw.warm_fallbacks == 0
    assert tw.linear_solves * 3 < tp.linear_solves
    assert agree >= 0.85
    # every closure that plain GNC keeps is kept or rejected near the threshold; no closure that
    # plain GNC rejects as a gross outlier (true outlier) is kept by the warm start
    truth = _truth(s, plain)
    assert not np.any((np.round(ww[nk:]) == 1) & truth[nk:] & (np.round(wp[nk:]) == 0))
    # without the network: the same schedule from all-ones probabilities
    ones = capi.RobustSolver(_params(True, pcm_off))
    assert ones.update(s.graph, optimize_graph=False) == 0
    assert ones.set_warm_start_probs(np.ones(ones.counts().num_factors)) == 0
    assert ones.forceUpdate(_empty()) == 0
    to = ones.timing()
    print(f"  all-ones start: {to.linear_solves} solves, fallbacks {to.warm_fallbacks}")
    assert tw.linear_solves <= to.linear_solves


def _truth(s, solver):
    """Per factor of the solver's graph: True for a generated outlier."""
    a = s.graph.arrays()
    off = s.n_odom + 1
    bad = {(int(a["key1"][off + q]), int(a["key2"][off + q])): bool(s.is_outlier[q]) for q in range(s.n_lc)}
    _, k1, k2, _ = solver.factors()
    return np.array([bad.get((int(x), int(y)), False) for x, y in zip(k1, k2)])

"""Closure network of the GNC warm start: oracle self-checks (CPU) and the
CUDA kernels against the oracle through the C ABI (GPU).

Tolerances: the kernels accumulate in FP32 from BF16 weights; the oracle is
FP64 with the same BF16 rounding. Probabilities agree to 1e-5 absolute,
gradients to 1e-4 relative (norm), features to 1e-5 relative.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import mlp_oracle as M
from oracle import rpgo_oracle as O
from rpgo_gb300 import capi, synth
from rpgo_gb300.params import QUIET, WARM_RECORD, RobustSolverParams


def _rand_params(rng, scale=1.0):
    p = np.zeros(M.N_PARAMS, dtype=np.float32)
    p[M.OFF_MU:M.OFF_MU + 16] = rng.normal(0, 1, 16)
    p[M.OFF_ISD:M.OFF_ISD + 16] = rng.uniform(0.5, 2.0, 16)
    p[M.OFF_W1:] = rng.normal(0, 0.3 * scale, M.N_PARAMS - M.OFF_W1)
    return p


def test_layout_matches_library():
    assert M.N_PARAMS == capi.MLP_PARAMS == 5345
    assert capi.MLP_FEATURES == M.FEAT


def test_bf16_rounding_known_answers():
    x = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, -2.5, 3.14159265, 1e-20], dtype=np.float32)
    r = M.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1 + 2 ** -6) and r[3] == -2.5
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    y = rng.normal(0, 10, 10000).astype(np.float32)
    ref = torch.from_numpy(y).to(torch.bfloat16).float().numpy()
    assert np.array_equal(M.bf16_round(y), ref)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = _rand_params(rng).astype(np.float64)
    X = rng.normal(0, 1, (64, 16))
    y = (rng.random(64) < 0.6).astype(np.float64)
    loss, g = M.loss_and_grad(p, X, y, bf16=False)
    idx = np.concatenate([rng.choice(np.arange(M.OFF_W1, M.N_PARAMS), 40, replace=False), [M.OFF_B3]])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (M.loss_and_grad(pp, X, y, bf16=False)[0] - M.loss_and_grad(pm, X, y, bf16=False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(fd)


@pytest.mark.gpu
def test_gpu_forward_and_training_step_match_oracle():
    torch = pytest.importorskip("torch")
    from rpgo_gb300 import build

    build()
    lib = capi.load()
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(2)
    p = _rand_params(rng)
    X = rng.normal(0, 1, (3000, 16)).astype(np.float32)
    y = (rng.random(3000) < 0.7).astype(np.float32)
    P, Xd, Yd = (torch.from_numpy(a).to(dev) for a in (p, X, y))
    prob = torch.zeros(3000, device=dev)
    st = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    assert lib.rpgo_mlp_forward_dev(P.data_ptr(), 3000, Xd.data_ptr(), prob.data_ptr(), st) == 0
    po, _ = M.forward(p, X)
    np.testing.assert_allclose(prob.cpu().numpy(), po, atol=1e-5)
    # gradient only (lr = 0)
    m = torch.zeros_like(P)
    v = torch.zeros_like(P)
    g = torch.zeros_like(P)
    loss = C.c_double()
    assert lib.rpgo_mlp_train_step_dev(P.data_ptr(), m.data_ptr(), v.data_ptr(), 0, 0.0, 3000, Xd.data_ptr(),
                                       Yd.data_ptr(), g.data_ptr(), C.byref(loss), st) == 0
    lo, go = M.loss_and_grad(p, X, y)
    assert abs(loss.value - lo) <= 1e-5 * abs(lo)
    gg = g.cpu().numpy().astype(np.float64)
    assert np.all(gg[:32] == 0.0)
    assert np.linalg.norm(gg - go) <= 1e-4 * np.linalg.norm(go)
    # two Adam steps against the oracle's
    mo, vo, pw = np.zeros(M.N_PARAMS), np.zeros(M.N_PARAMS), p.astype(np.float64)
    for step in (1, 2):
        assert lib.rpgo_mlp_train_step_dev(P.data_ptr(), m.data_ptr(), v.data_ptr(), step, 1e-3, 3000,
                                           Xd.data_ptr(), Yd.data_ptr(), g.data_ptr(), None, st) == 0
        _, go = M.loss_and_grad(pw.astype(np.float32), X, y)
        pw, mo, vo = M.adam_step(pw, mo, vo, go, step, 1e-3)
    np.testing.assert_allclose(P.cpu().numpy(), pw, atol=2e-6)


@pytest.mark.gpu
def test_gpu_closure_features_match_oracle():
    from rpgo_gb300 import build

    build()
    s = synth.walk3d(600, 90, 30, seed=31, clustered_outliers=20)
    par = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    par.setGncWarmStart(WARM_RECORD)
    g = capi.RobustSolver(par)
    assert g.update(s.graph) == 0
    feats = g.closure_features()
    c = g.counts()
    n_known = c.num_odom + c.num_special
    kind, k1, k2, meas = g.factors()
    assert len(feats) == len(kind) - n_known > 0
    a = s.graph.arrays()
    x0 = {int(k): p for k, p in zip(a["value_keys"], a["value_poses"])}
    # sqrt information of each optimised factor, matched by keys and measurement
    by_key = {}
    for i in range(len(a["kind"])):
        by_key.setdefault((int(a["key1"][i]), int(a["key2"][i])), []).append(i)
    sq = np.zeros((len(kind), 36))
    for f in range(len(kind)):
        for i in by_key[(int(k1[f]), int(k2[f]))]:
            if np.array_equal(a["measured"][i], meas[f]):
                sq[f] = a["sqrt_info"][i].reshape(-1)
    # PCM statistics from the adjacency (one group) and the consistent list
    adj = g.adjacency(0)
    stats = _pcm_stats(s, n_known, k1, k2, meas, adj)
    ref = M.closure_features(3, x0, (kind, k1, k2, meas, sq), n_known, stats)
    np.testing.assert_allclose(feats, ref, rtol=1e-5, atol=1e-5)


def _pcm_stats(s, n_known, k1, k2, meas, adj):
    """The group holds the closures that passed the odometry check, in
    arrival order (a closure's row is its position there); with the pairwise
    check disabled (negative threshold) the oracle's graph lists exactly
    them, in that order."""
    n = adj.shape[0]
    odom_ok = O.OracleSolver(RobustSolverParams().setPcm3DParams(10.0, -1.0, QUIET))
    odom_ok.update(s.graph, optimize_graph=False)
    _, gk1, gk2, gm = odom_ok.factors()
    rows = {}
    r = 0
    for f in range(len(gk1)):
        if f < n_known:
            continue
        rows.setdefault((int(gk1[f]), int(gk2[f]), gm[f].tobytes()), []).append(r)
        r += 1
    assert r == n
    consistent = [rows[(int(k1[f]), int(k2[f]), meas[f].tobytes())][0] for f in range(n_known, len(k1))]
    return M.pcm_stats(np.ascontiguousarray(adj), n, consistent)

"""CUDA path against the CPU FP64 oracle, through the C ABI.

Bit-exact where the reference's decision is integer-valued (adjacency bits,
clique index lists, inlier sets, factor order); within tolerance for poses
(ATE <= 1e-4 m, elementwise 1e-6 relative on the pose entries).
"""
import math

import numpy as np
import pytest

from oracle import rpgo_oracle as O
from rpgo_gb300 import capi, synth
from rpgo_gb300.graph import Graph, diagonal_sigmas, isotropic_variance, pose2, pose3, symbol
from rpgo_gb300.params import LINEAR_CHOLESKY, LINEAR_PCG, QUIET, RobustSolverParams
from scenarios import PCM_SCENARIOS, load_graph_scenarios, run_scenario

pytestmark = pytest.mark.gpu

POSE_RTOL = 1e-6
ATE_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from rpgo_gb300 import build

    build()
    capi.load()


# ------------------------------------------------------------------ stage: pairwise adjacency (bit exact)
def _rand_rot(rng):
    return synth.uniform_rotation(rng)


def _rand_spd(rng, d, scale):
    A = rng.normal(size=(d, d))
    return scale * (A @ A.T + 0.1 * np.eye(d))


def _random_stage_inputs(rng, dim, mode, n_slots, n_lc):
    st, d = (12, 6) if dim == 3 else (4, 3)
    # half the slots from an odometry chain (nested covariances: LLT passes),
    # half independent (LLT fallback exercised)
    tp = np.zeros((n_slots, st))
    tc = np.zeros((n_slots, d, d))
    cur_p = pose3() if dim == 3 else pose2()
    cur_c = np.zeros((d, d))
    half = n_slots // 2
    for s in range(n_slots):
        if s < half:
            if dim == 3:
                R = synth.so3_exp(rng.normal(0, 0.2, 3))
                step = pose3(R, rng.normal(0, 1.0, 3))
            else:
                th = rng.normal(0, 0.3)
                step = pose2(th, *rng.normal(0, 1.0, 2))
            cur_p, cur_c, _ = O.pwc_op(dim, 0, cur_p, cur_c, 1, step, _rand_spd(rng, d, 0.01), 1)
            tp[s], tc[s] = cur_p, cur_c
        else:
            tp[s] = pose3(_rand_rot(rng), rng.normal(0, 5, 3)) if dim == 3 else pose2(rng.uniform(-3, 3),
                                                                                        *rng.normal(0, 5, 2))
            tc[s] = _rand_spd(rng, d, rng.uniform(0.01, 1.0))
    tn = rng.integers(0, 50, n_slots).astype(np.int32)
    tr = (rng.random(n_slots) > 0.05).astype(np.uint8)
    sa = rng.integers(0, n_slots, n_lc).astype(np.int32)
    sb = rng.integers(0, n_slots, n_lc).astype(np.int32)
    flip = (rng.random(n_lc) < 0.3).astype(np.uint8)
    zp = np.zeros((n_lc, st))
    zc = np.zeros((n_lc, d, d))
    for k in range(n_lc):
        # mostly near-consistent measurements so that both verdicts occur
        if rng.random() < 0.7:
            b, _, _ = O.pwc_op(dim, 1, tp[sa[k]], tc[sa[k]], 1, tp[sb[k]], tc[sb[k]], 1)
            zp[k] = b
        else:
            zp[k] = pose3(_rand_rot(rng), rng.normal(0, 3, 3)) if dim == 3 else pose2(rng.uniform(-3, 3),
                                                                                        *rng.normal(0, 3, 2))
        zc[k] = _rand_spd(rng, d, rng.uniform(0.001, 0.5))
        if rng.random() < 0.05:
            zc[k, 0, 0] = np.nan  # rotation information missing
    return sa, sb, flip, zp, zc, tp, tc, tn, tr


@pytest.mark.parametrize("dim,mode", [(3, 0), (3, 1), (2, 0), (2, 1)])
@pytest.mark.parametrize("seed", [0, 1])
def test_pairwise_stage_bit_exact(dim, mode, seed):
    rng = np.random.default_rng(100 + seed)
    sa, sb, flip, zp, zc, tp, tc, tn, tr = _random_stage_inputs(rng, dim, mode, 160, 150)
    th = [(5.0, 0.0), (1.0, 0.0)] if mode == 0 else [(0.5, 0.2), (2.0, 0.5)]
    for th0, th1 in th:
        ref = O.pairwise_adjacency(dim, mode, sa, sb, flip, zp, zc, tp, tc, tn, tr, th0, th1)
        got = capi.pairwise_adjacency(dim, mode, sa, sb, flip, zp, zc, tp, tc, tn, tr, th0, th1)
        assert np.array_equal(ref, got), (dim, mode, th0, int(np.sum(ref != got)))
        bits = int(sum(bin(int(x)).count("1") for x in ref.ravel()))
        assert 0 < bits < 150 * 149, bits  # both verdicts present


def test_pairwise_stage_edge_sizes():
    rng = np.random.default_rng(7)
    for n in (0, 1, 2, 31, 32, 33, 64, 65):
        sa, sb, flip, zp, zc, tp, tc, tn, tr = _random_stage_inputs(rng, 3, 0, 40, max(n, 1))
        sa, sb, flip, zp, zc = sa[:n], sb[:n], flip[:n], zp[:n], zc[:n]
        ref = O.pairwise_adjacency(3, 0, sa, sb, flip, zp, zc, tp, tc, tn, tr, 5.0, 0.0)
        got = capi.pairwise_adjacency(3, 0, sa, sb, flip, zp, zc, tp, tc, tn, tr, 5.0, 0.0)
        assert np.array_equal(ref.reshape(-1), got.reshape(-1)), n


# ------------------------------------------------------------------ stage: max clique (exact)
def _bits(n, edges):
    w = (n + 31) // 32
    adj = np.zeros((max(n, 1), max(w, 1)), dtype=np.uint32)
    for i, j in edges:
        adj[i, j >> 5] |= np.uint32(1 << (j & 31))
        adj[j, i >> 5] |= np.uint32(1 << (i & 31))
    return adj[:n, :w]


@pytest.mark.parametrize("seed", range(10))
def test_clique_stage_exact(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 400))
    p = rng.uniform(0.02, 0.98)
    iu = np.triu_indices(n, 1)
    m = rng.random(len(iu[0])) < p
    edges = list(zip(iu[0][m], iu[1][m]))
    adj = _bits(n, edges)
    rs, rc = O.max_clique_heu(adj, n)
    gs, gc = capi.max_clique_heu(adj, n)
    assert rs == gs and np.array_equal(rc, gc)
    first, seed_sz = n // 3, max(1, rs // 2)
    rs2, rc2 = O.max_clique_heu(adj, n, first, seed_sz)
    gs2, gc2 = capi.max_clique_heu(adj, n, first, seed_sz)
    assert rs2 == gs2 and np.array_equal(rc2, gc2)


def test_clique_planted_dense_clique():
    # a planted clique of 300 among 1000 vertices with sparse noise
    rng = np.random.default_rng(3)
    n = 1000
    members = rng.choice(n, 300, replace=False)
    edges = set()
    for a in range(len(members)):
        for b in range(a + 1, len(members)):
            edges.add((min(members[a], members[b]), max(members[a], members[b])))
    for _ in range(20000):
        i, j = rng.integers(0, n, 2)
        if i != j:
            edges.add((min(i, j), max(i, j)))
    adj = _bits(n, sorted(edges))
    rs, rc = O.max_clique_heu(adj, n)
    gs, gc = capi.max_clique_heu(adj, n)
    assert rs == gs >= 300 and np.array_equal(rc, gc)


# ------------------------------------------------------------------ the reference's tests through the GPU path
@pytest.mark.parametrize("name", sorted(PCM_SCENARIOS))
def test_pcm_scenarios_gpu(name):
    params, steps = PCM_SCENARIOS[name]()
    fails, _ = run_scenario(capi.RobustSolver, params, steps)
    assert not fails, fails


def test_load_graph_and_gnc_scenarios_gpu(robot_a, robot_b):
    sc = load_graph_scenarios(robot_a, robot_b)
    bad = {}
    for name, (params, steps) in sc.items():
        fails, _ = run_scenario(capi.RobustSolver, params, steps)
        if fails:
            bad[name] = fails
    assert not bad, bad


# ------------------------------------------------------------------ synthetic graphs: PCM bit exact, solve in tolerance
def _compare_pcm(params, graph, groups=1):
    o = O.OracleSolver(params)
    g = capi.RobustSolver(params)
    assert o.update(graph, False) == 0
    assert g.update(graph, False) == 0
    co, cg = o.counts(), g.counts()
    assert (co.num_factors, co.num_lc, co.num_lc_inliers) == (cg.num_factors, cg.num_lc, cg.num_lc_inliers)
    for gi in range(groups):
        ao, ag = o.adjacency(gi), g.adjacency(gi)
        assert ao is not None and ag is not None
        assert np.array_equal(ao, ag), int(np.sum(ao != ag))
    ko, k1o, k2o, _ = o.factors()
    kg, k1g, k2g, _ = g.factors()
    assert np.array_equal(ko, kg) and np.array_equal(k1o, k1g) and np.array_equal(k2o, k2g)
    return o, g


@pytest.mark.parametrize("seed", [11, 12])
def test_synthetic_3d_pcm_bit_exact(seed):
    s = synth.walk3d(600, 150, 50, seed=seed)
    _compare_pcm(RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET), s.graph)


def test_synthetic_2d_pcm_bit_exact():
    s = synth.grid2d(500, 100, 20, seed=1)
    _compare_pcm(RobustSolverParams().setPcm2DParams(3.0, 3.0, QUIET), s.graph)


@pytest.mark.parametrize("dim", [2, 3])
def test_synthetic_pcm_simple_bit_exact(dim):
    if dim == 3:
        s = synth.walk3d(500, 120, 40, seed=21)
        p = RobustSolverParams().setPcmSimple3DParams(0.05, 0.01, QUIET)
    else:
        s = synth.grid2d(400, 80, 20, seed=22)
        p = RobustSolverParams().setPcmSimple2DParams(0.1, 0.05, QUIET)
    _compare_pcm(p, s.graph)


def test_incremental_mode_matches_oracle():
    s = synth.walk3d(300, 60, 20, seed=31)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setIncremental()
    o, g = O.OracleSolver(p), capi.RobustSolver(p)
    g0 = s.graph.copy()
    n_base = s.n_odom + 1
    base = Graph(3)
    base.kind, base.key1, base.key2 = g0.kind[:n_base], g0.key1[:n_base], g0.key2[:n_base]
    base.measured, base.cov, base.sqrt_info = g0.measured[:n_base], g0.cov[:n_base], g0.sqrt_info[:n_base]
    base.value_keys, base.value_poses = g0.value_keys, g0.value_poses
    assert o.update(base, False) == 0 and g.update(base, False) == 0
    for k in range(n_base, g0.num_factors, 3):
        b = Graph(3)
        b.kind, b.key1, b.key2 = g0.kind[k:k + 3], g0.key1[k:k + 3], g0.key2[k:k + 3]
        b.measured, b.cov, b.sqrt_info = g0.measured[k:k + 3], g0.cov[k:k + 3], g0.sqrt_info[k:k + 3]
        assert o.update(b, False) == 0 and g.update(b, False) == 0
        assert o.counts().num_lc_inliers == g.counts().num_lc_inliers
    assert np.array_equal(o.adjacency(0), g.adjacency(0))
    assert np.array_equal(o.factors()[1], g.factors()[1])


def test_multi_robot_inter_group_bit_exact():
    a = synth.walk3d(200, 40, 10, seed=41, prefix="a")
    b = synth.walk3d(200, 40, 10, seed=42, prefix="b")
    p = RobustSolverParams().setPcm3DParams(10.0, 50.0, QUIET)
    o, g = O.OracleSolver(p), capi.RobustSolver(p)
    assert o.update(a.graph, False) == 0 and g.update(a.graph, False) == 0
    assert o.update(b.graph, False) == 0 and g.update(b.graph, False) == 0
    rng = np.random.default_rng(5)
    inter = Graph(3)
    for _ in range(60):
        i, j = rng.integers(0, 200, 2)
        ka, kb = symbol("a", int(i)), symbol("b", int(j))
        z = pose3(synth.so3_exp(rng.normal(0, 0.3, 3)), rng.normal(0, 2, 3))
        if rng.random() < 0.5:
            inter.add_between(ka, kb, z, isotropic_variance(6, 0.5))
        else:
            inter.add_between(kb, ka, z, isotropic_variance(6, 0.5))
    assert o.update(inter, False) == 0 and g.update(inter, False) == 0
    for gi in range(3):
        ao, ag = o.adjacency(gi), g.adjacency(gi)
        assert np.array_equal(ao, ag), gi
    assert np.array_equal(o.factors()[1], g.factors()[1]) and np.array_equal(o.factors()[2], g.factors()[2])


def _pose_close(po, pg, dim):
    assert synth.ate(pg, po, dim) <= ATE_TOL
    scale = np.maximum(1.0, np.abs(po))
    assert np.max(np.abs(pg - po) / scale) <= POSE_RTOL, float(np.max(np.abs(pg - po) / scale))


LINEAR = [LINEAR_CHOLESKY, LINEAR_PCG]


def _check_linear_path(g, linear):
    t = g.timing()
    if linear == LINEAR_CHOLESKY:
        assert t.chol_kernel_launches > 0 and t.pcg_kernel_launches == 0
    else:
        assert t.pcg_kernel_launches > 0 and t.chol_kernel_launches == 0


@pytest.mark.parametrize("linear", LINEAR)
@pytest.mark.parametrize("gnc", [False, True])
def test_solver_3d_matches_oracle(gnc, linear):
    s = synth.walk3d(400, 80, 25, seed=51)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setLinearSolver(linear)
    if gnc:
        p.setGncInlierCostThresholdsAtProbability(0.9)
    o, g = O.OracleSolver(p), capi.RobustSolver(p)
    assert o.update(s.graph) == 0 and g.update(s.graph) == 0
    ko, po = o.estimate()
    kg, pg = g.estimate()
    assert np.array_equal(ko, kg)
    _pose_close(po, pg, 3)
    _check_linear_path(g, linear)
    if gnc:
        wo, wg = o.gnc_weights(), g.gnc_weights()
        assert np.array_equal(np.round(wo), np.round(wg))
        assert o.counts().num_lc_inliers == g.counts().num_lc_inliers


@pytest.mark.parametrize("linear", LINEAR)
def test_solver_2d_matches_oracle(linear):
    s = synth.grid2d(300, 60, 15, seed=61)
    p = RobustSolverParams().setPcm2DParams(3.0, 3.0, QUIET).setLinearSolver(linear)
    o, g = O.OracleSolver(p), capi.RobustSolver(p)
    assert o.update(s.graph) == 0 and g.update(s.graph) == 0
    _pose_close(o.estimate()[1], g.estimate()[1], 2)
    _check_linear_path(g, linear)


@pytest.mark.parametrize("linear", LINEAR)
def test_gauss_newton_matches_oracle(linear):
    s = synth.walk3d(300, 50, 0, seed=71)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setLinearSolver(linear)
    p.solver = 1
    o, g = O.OracleSolver(p), capi.RobustSolver(p)
    assert o.update(s.graph) == 0 and g.update(s.graph) == 0
    _pose_close(o.estimate()[1], g.estimate()[1], 3)
    _check_linear_path(g, linear)


def test_direct_solve_larger_graph_matches_oracle():
    # 2,000 poses with many closures: a dense trailing block of several tiles
    s = synth.walk3d(2000, 500, 100, seed=53)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    o, g = O.OracleSolver(p), capi.RobustSolver(p)
    assert o.update(s.graph) == 0 and g.update(s.graph) == 0
    _pose_close(o.estimate()[1], g.estimate()[1], 3)
    assert np.array_equal(np.round(o.gnc_weights()), np.round(g.gnc_weights()))
    _check_linear_path(g, LINEAR_CHOLESKY)


def test_kernels_actually_launch():
    before = capi.kernel_launch_count()
    s = synth.walk3d(200, 40, 10, seed=81)
    g = capi.RobustSolver(RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET))
    assert g.update(s.graph) == 0
    assert capi.kernel_launch_count() > before
    t = g.timing()
    assert t.kernel_launches > 0 and t.pair_checks > 0


def test_update_dev_matches_host_update():
    # HBM-resident inputs (rpgo_update_dev) give the same result as host inputs
    s = synth.walk3d(300, 60, 20, seed=91)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    a, b = capi.RobustSolver(p), capi.RobustSolver(p)
    assert a.update(s.graph) == 0
    db = capi.DeviceBatch(s.graph)
    assert b.update_dev(db) == 0
    assert np.array_equal(a.adjacency(0), b.adjacency(0))
    assert np.array_equal(a.gnc_weights(), b.gnc_weights())
    ka, pa = a.estimate()
    kb, pb = b.estimate()
    assert np.array_equal(ka, kb) and np.array_equal(pa, pb)


@pytest.mark.parametrize("prefer", [1, 2])
def test_fill_in_guard_branches_match_oracle(prefer):
    # GNC alone on uniform outliers: every outlier joins distant poses and the
    # factor fills in. A zero guard makes every plan race the two solvers on
    # its first damped system; both branches (direct kept / PCG kept for the
    # rest of the schedule) equal the oracle.
    s = synth.walk3d(800, 160, 120, seed=57)
    p = RobustSolverParams().setPcm3DParams(-1.0, -1.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    old = capi.set_direct_solve_guard(0.0, prefer)
    try:
        o, g = O.OracleSolver(p), capi.RobustSolver(p)
        assert o.update(s.graph) == 0 and g.update(s.graph) == 0
    finally:
        capi.set_direct_solve_guard(old, 0)
    t = g.timing()
    if prefer == 1:
        assert t.pcg_kernel_launches == 1 and t.chol_kernel_launches == t.linear_solves
    else:
        assert t.chol_kernel_launches == 1 and t.pcg_kernel_launches == t.linear_solves
    assert np.array_equal(np.round(o.gnc_weights()), np.round(g.gnc_weights()))
    _pose_close(o.estimate()[1], g.estimate()[1], 3)


def test_fill_in_guard_off_below_threshold():
    # the benchmark-sized plans stay far below the default guard: no race
    s = synth.walk3d(600, 150, 50, seed=58)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    g = capi.RobustSolver(p)
    assert g.update(s.graph) == 0
    assert g.timing().pcg_kernel_launches == 0

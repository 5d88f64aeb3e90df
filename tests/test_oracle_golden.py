"""Pins the CPU oracle against the reference's own known answers.

Golden values come from the reference's tests (GeometryUtils, Trajectory,
Pcm, PcmSimple, PcmDoOptimize, LoadGraph, Gnc, MultiRobot) and from the
fixture files tests/data/robot_a.g2o / robot_b.g2o (copied by
tests/golden/make_golden.py). CPU only.
"""
import math

import numpy as np
import pytest

from oracle import rpgo_oracle as O
from rpgo_gb300.graph import pose3, rot3_quaternion
from scenarios import PCM_SCENARIOS, load_graph_scenarios, run_scenario

I6 = np.eye(6)


def pose_eq(a, b, tol=1e-9):
    return np.allclose(np.asarray(a), np.asarray(b), atol=tol)


# ---------------------------------------------------------------- testPoseWithCovariance.cpp
def test_pose_with_covariance_inverse():
    p = pose3()
    po, co, _ = O.pwc_op(3, 2, p, I6)
    assert pose_eq(po, pose3())
    assert np.array_equal(co, I6)


def test_pose_with_covariance_compose_golden():
    # testPoseWithCovariance.cpp:51-147
    A = (pose3(None, (1, 1, 1)), 0.1 * I6)
    AB = (pose3(None, (1, 1, 1)), 0.1 * I6)
    Bp, Bc, _ = O.pwc_op(3, 0, A[0], A[1], 1, AB[0], AB[1], 1)
    B_cov = 0.1 * np.array([[2, 0, 0, 0, -1, 1], [0, 2, 0, 1, 0, -1], [0, 0, 2, -1, 1, 0],
                            [0, 1, -1, 4, -1, -1], [-1, 0, 1, -1, 4, -1], [1, -1, 0, -1, -1, 4]], dtype=float)
    assert pose_eq(Bp, pose3(None, (2, 2, 2)))
    assert np.allclose(Bc, B_cov, atol=1e-9)
    BCc = 0.1 * I6
    BCc[3:, 3:] = 0.01 * np.eye(3)
    BC = (pose3(rot3_quaternion(0, 0, 0, 1), (0, 0, 0)), BCc)
    Cp, Cc, _ = O.pwc_op(3, 0, Bp, Bc, 1, BC[0], BC[1], 1)
    C_cov = np.array([[0.3, 0, 0, 0, -0.1, -0.1], [0, 0.3, 0, 0.1, 0, 0.1], [0, 0, 0.3, 0.1, -0.1, 0],
                      [0, 0.1, 0.1, 0.41, -0.1, 0.1], [-0.1, 0, -0.1, -0.1, 0.41, 0.1],
                      [-0.1, 0.1, 0, 0.1, 0.1, 0.41]])
    assert np.allclose(Cc, C_cov, atol=1e-9)
    CD = (pose3(rot3_quaternion(0, 0, 1, 0), (1, 0, 0)), 0.1 * I6)
    Dp, Dc, _ = O.pwc_op(3, 0, Cp, Cc, 1, CD[0], CD[1], 1)
    D_cov = np.array([[0.4, 0, 0, 0, 0.1, -0.1], [0, 0.4, 0, -0.1, 0, 0.2], [0, 0, 0.4, 0.1, -0.2, 0],
                      [0, -0.1, 0.1, 0.51, 0, 0], [0.1, 0, -0.2, 0, 0.61, -0.1], [-0.1, 0.2, 0, 0, -0.1, 0.61]])
    assert np.allclose(Dc, D_cov, atol=1e-9)


def test_pose_with_covariance_between_golden():
    # testPoseWithCovariance.cpp:168-200
    A_cov = np.array([[0.3, 0, 0, 0, -0.1, -0.1], [0, 0.3, 0, 0.1, 0, 0.1], [0, 0, 0.3, 0.1, -0.1, 0],
                      [0, 0.1, 0.1, 0.41, -0.1, 0.1], [-0.1, 0, -0.1, -0.1, 0.41, 0.1],
                      [-0.1, 0.1, 0, 0.1, 0.1, 0.41]])
    C_cov = np.array([[0.4, 0, 0, 0, 0.1, -0.1], [0, 0.4, 0, -0.1, 0, 0.2], [0, 0, 0.4, 0.1, -0.2, 0],
                      [0, -0.1, 0.1, 0.51, 0, 0], [0.1, 0, -0.2, 0, 0.61, -0.1], [-0.1, 0.2, 0, 0, -0.1, 0.61]])
    Cp = pose3(rot3_quaternion(0, 0, 1, 0), (1, 0, 0))
    Bp, Bc, _ = O.pwc_op(3, 1, pose3(), A_cov, 1, Cp, C_cov, 1)
    assert pose_eq(Bp, Cp)
    assert np.allclose(Bc, 0.1 * I6, atol=1e-9)


# ---------------------------------------------------------------- testPoseWithNode.cpp
def test_pose_with_node_norms():
    # testPoseWithNode.cpp:82-99
    t, r = O.pwn_norms(3, pose3(), 1)
    assert t == 0 and r == 0
    t, r = O.pwn_norms(3, pose3(rot3_quaternion(1, 0, 0, 0), (1, 0, 0)), 5)
    assert t == 0.2
    t, r = O.pwn_norms(3, pose3(rot3_quaternion(0, 0, 1, 0), (0, 0, 0)), 5)
    assert abs(r - 3.1415927 / 5) < 1e-6


def test_logmap_at_pi_axes():
    for q in [(0, 1, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1)]:
        xi = O.logmap(3, pose3(rot3_quaternion(*q), (0, 0, 0)))
        assert abs(np.linalg.norm(xi[:3]) - math.pi) < 1e-12


def test_logmap_against_scipy_style_reference():
    rng = np.random.default_rng(5)
    for _ in range(300):
        w = rng.normal(size=3)
        w *= rng.uniform(0, 3.1) / np.linalg.norm(w)
        th = np.linalg.norm(w)
        K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
        R = np.eye(3) + math.sin(th) / th * K + (1 - math.cos(th)) / th ** 2 * K @ K
        xi = O.logmap(3, pose3(R, (0.3, -1.0, 2.0)))
        assert np.allclose(xi[:3], w, atol=1e-12)


# ---------------------------------------------------------------- testTrajectory.cpp
def test_trajectory_between_matches_restitched_chain():
    # testTrajectory.cpp:35-107: getBetween(2, 99) equals composing the
    # 97 odometry steps from identity
    odom = (pose3(rot3_quaternion(1, 0, 0, 0), (1, 1, 0)), 0.0001 * I6)
    poses = {}
    cur = (pose3(), np.zeros((6, 6)))
    for i in range(100):
        p, c, _ = O.pwc_op(3, 0, cur[0], cur[1], 1, odom[0], odom[1], 1)
        cur = (p, c)
        poses[i] = cur
    bp, bc, _ = O.pwc_op(3, 1, poses[2][0], poses[2][1], 1, poses[99][0], poses[99][1], 1)
    reb = (pose3(), np.zeros((6, 6)))
    for i in range(2, 99):
        p, c, _ = O.pwc_op(3, 0, reb[0], reb[1], 1, odom[0], odom[1], 1)
        reb = (p, c)
    assert pose_eq(bp, reb[0])
    assert np.allclose(bc, reb[1], atol=1e-9)


# ---------------------------------------------------------------- own math
def test_atan2_within_two_ulp_of_libm():
    rng = np.random.default_rng(0)
    ys = np.concatenate([rng.normal(size=4000), [0.0, 1.0, -1.0, 1e-300, 3.0]])
    xs = np.concatenate([rng.normal(size=4000), [-1.0, 0.0, 0.0, 1.0, -3.0]])
    for y, x in zip(ys, xs):
        a, b = O.atan2(y, x), math.atan2(y, x)
        assert abs(a - b) <= 2 * np.spacing(max(abs(b), 1e-300)), (y, x, a, b)


@pytest.mark.parametrize("alpha,k,ref", [(0.9, 6, 10.644640675668), (0.99, 6, 16.811893829770),
                                         (0.01, 6, 0.872090330), (0.9, 3, 6.251388631170),
                                         (0.5, 1, 0.454936423119)])
def test_chi2inv(alpha, k, ref):
    assert abs(O.chi2inv(alpha, k) - ref) < 1e-7 * max(1.0, ref)


# ---------------------------------------------------------------- max clique heuristic
def _bits(n, edges):
    w = (n + 31) // 32
    adj = np.zeros((n, w), dtype=np.uint32)
    for i, j in edges:
        adj[i, j >> 5] |= np.uint32(1 << (j & 31))
        adj[j, i >> 5] |= np.uint32(1 << (i & 31))
    return adj


def fmc_reference_python(n, edges, first=0, seed=-1):
    """Line-by-line restatement of findCliqueHeu.cpp:32-117 in Python (small
    cases), independent of the C oracle."""
    nb = [[] for _ in range(n)]
    es = set()
    for i, j in edges:
        if i != j and (i, j) not in es and (j, i) not in es:
            es.add((i, j))
    for j in range(n):
        for i in range(j + 1, n):
            if (i, j) in es or (j, i) in es:
                nb[i].append(j)
                nb[j].append(i)
    for v in range(n):
        nb[v].sort()
    deg = [len(x) for x in nb]
    maxdeg = max(deg) if n else -1
    S = [0] * (maxdeg + 1)
    best, maxclq = None, seed
    for v in range(first, n):
        if maxclq > deg[v]:
            continue
        pos = 0
        S[pos] = v
        pos += 1
        for u in nb[v]:
            if maxclq <= deg[u]:
                S[pos] = u
                pos += 1
        icc = 0
        while pos > 0:
            icc += 1
            m = S[pos - 1]
            S1 = [S[a] for a in range(pos) if S[a] in nb[m] and maxclq <= deg[S[a]]]
            for a, x in enumerate(S1):
                S[a] = x
            pos = len(S1)
        if maxclq < icc:
            best = list(S)
            maxclq = icc
    return maxclq, (best[:maxclq] if best is not None else [])


def test_clique_stale_buffer_example():
    # candidate 0 with neighbours {1,2,3}, 3~1, 2 only adjacent to 0: the
    # greedy chain is {3,1,0} but the buffer slots read [0,1,2]
    adj = _bits(4, [(0, 1), (0, 2), (0, 3), (1, 3)])
    size, cl = O.max_clique_heu(adj, 4)
    assert size == 3 and list(cl) == [0, 1, 2]
    assert fmc_reference_python(4, [(0, 1), (0, 2), (0, 3), (1, 3)]) == (3, [0, 1, 2])


@pytest.mark.parametrize("seed", range(12))
def test_clique_oracle_matches_python_restatement(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 70))
    p = rng.uniform(0.05, 0.95)
    edges = [(i, j) for j in range(n) for i in range(j) if rng.random() < p]
    adj = _bits(n, edges)
    size, cl = O.max_clique_heu(adj, n)
    ps, pcl = fmc_reference_python(n, edges)
    assert size == ps and list(cl) == pcl
    # incremental form: seed with a previous size and scan only the tail
    first = n // 2
    prev = max(1, size // 2)
    size2, cl2 = O.max_clique_heu(adj, n, first, prev)
    ps2, pcl2 = fmc_reference_python(n, edges, first, prev)
    assert size2 == ps2 and list(cl2) == pcl2


def test_clique_empty_graph_keeps_first_closure():
    size, cl = O.max_clique_heu(np.zeros((5, 1), dtype=np.uint32), 5)
    assert size == 1 and list(cl) == [0]


# ---------------------------------------------------------------- PCM scenarios
@pytest.mark.parametrize("name", sorted(PCM_SCENARIOS))
def test_pcm_scenarios_oracle(name):
    params, steps = PCM_SCENARIOS[name]()
    fails, _ = run_scenario(O.OracleSolver, params, steps)
    assert not fails, fails


def test_load_graph_and_gnc_scenarios_oracle(robot_a, robot_b):
    sc = load_graph_scenarios(robot_a, robot_b)
    bad = {}
    for name, (params, steps) in sc.items():
        fails, _ = run_scenario(O.OracleSolver, params, steps)
        if fails:
            bad[name] = fails
    assert not bad, bad


def test_oracle_pair_tests_same_on_any_thread_count():
    # the oracle fills new rows of the consistency matrix on OpenMP threads;
    # the matrix (and so every later result) must not depend on their count
    from rpgo_gb300 import synth
    from rpgo_gb300.params import QUIET, RobustSolverParams

    s = synth.walk3d(600, 120, 40, seed=17)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET)
    before = O.set_threads(0)
    try:
        out = []
        for threads in (1, 4):
            O.set_threads(threads)
            o = O.OracleSolver(p)
            assert o.update(s.graph) == 0
            out.append((o.adjacency(0), o.factors()[1], o.estimate()[1]))
        assert np.array_equal(out[0][0], out[1][0])
        assert np.array_equal(out[0][1], out[1][1])
        assert np.array_equal(out[0][2], out[1][2])
    finally:
        O.set_threads(before)


# ---------------------------------------------------------------- oracle forms used for large checks
@pytest.mark.parametrize("seed", range(8))
def test_clique_stamp_form_matches_linear_scan(seed):
    # the membership-stamp form must reproduce the reference's linear-search
    # form exactly: size, index list (stale slots included), incremental form
    rng = np.random.default_rng(200 + seed)
    n = int(rng.integers(1, 300))
    p = rng.uniform(0.02, 0.98)
    iu = np.triu_indices(n, 1)
    m = rng.random(len(iu[0])) < p
    adj = _bits(n, list(zip(iu[0][m], iu[1][m])))
    before = O.set_clique_impl(0)
    try:
        ref = O.max_clique_heu(adj, n)
        ref2 = O.max_clique_heu(adj, n, n // 3, max(1, ref[0] // 2))
        for impl in (1, 2):
            O.set_clique_impl(impl)
            got = O.max_clique_heu(adj, n)
            got2 = O.max_clique_heu(adj, n, n // 3, max(1, ref[0] // 2))
            assert ref[0] == got[0] and np.array_equal(ref[1], got[1]), impl
            assert ref2[0] == got2[0] and np.array_equal(ref2[1], got2[1]), impl
    finally:
        O.set_clique_impl(before)


def _oracle_run(p, graph, impl):
    before = O.set_clique_impl(impl)
    try:
        o = O.OracleSolver(p)
        assert o.update(graph) == 0
        return o
    finally:
        O.set_clique_impl(before)


def test_oracle_stamp_clique_same_pcm_result():
    # whole PCM + solve on the 2D benchmark graph (thresholds 1.0 / 1.0) and a
    # 3D walk: same factor list and estimate with either clique form
    from rpgo_gb300 import synth
    from rpgo_gb300.params import QUIET, RobustSolverParams

    cases = [(synth.config_c1().graph, RobustSolverParams().setPcm2DParams(1.0, 1.0, QUIET)),
             (synth.walk3d(800, 200, 60, seed=19).graph,
              RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9))]
    for graph, p in cases:
        a = _oracle_run(p, graph, 0)
        for impl in (1, 2):
            b = _oracle_run(p, graph, impl)
            for x, y in zip(a.factors()[:3], b.factors()[:3]):
                assert np.array_equal(x, y)
            assert np.array_equal(a.estimate()[1], b.estimate()[1])
            assert np.array_equal(a.gnc_weights(), b.gnc_weights())


def test_pcm_rows_equal_full_matrix_rows():
    from rpgo_gb300 import synth
    from rpgo_gb300.params import QUIET, RobustSolverParams

    s = synth.walk3d(700, 160, 60, seed=23)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET)
    o = O.OracleSolver(p)
    assert o.update(s.graph, False) == 0
    full = o.adjacency(0)
    n, src, _ = O.OracleSolver(p).pcm_rows(s.graph, [])
    assert n == full.shape[0]
    rows = np.array([0, 1, n // 2, n - 1], dtype=np.int32)
    n2, src2, bits = O.OracleSolver(p).pcm_rows(s.graph, rows)
    assert n2 == n and np.array_equal(src, src2)
    assert np.array_equal(bits, full[rows])
    # src: group order = arrival order of the closures that passed the odometry check
    assert np.all(np.diff(src) > 0) and src[0] >= s.n_odom + 1


def test_solve_graph_equals_update_solve():
    # the solve stage alone on the factor list an update produced (known
    # inliers = odometry + priors) equals that update's solve
    from rpgo_gb300 import synth
    from rpgo_gb300.params import QUIET, RobustSolverParams

    s = synth.walk3d(500, 120, 40, seed=29)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    o = O.OracleSolver(p)
    assert o.update(s.graph) == 0
    c = o.counts()
    kind, k1, k2, _ = o.factors()
    fg = O.filtered_graph(s.graph, kind, k1, k2)
    o2 = O.OracleSolver(p)
    assert o2.solve_graph(fg, c.num_odom + c.num_special) == 0
    assert np.array_equal(o.estimate()[1], o2.estimate()[1])
    assert np.array_equal(o.gnc_weights(), o2.gnc_weights())
    assert o.stats()["linear_solves"] == o2.stats()["linear_solves"]


def test_oracle_solve_same_on_any_thread_count():
    # per-factor linearisation and error terms run on OpenMP threads and are
    # summed in factor order: the estimate must not depend on the count
    from rpgo_gb300 import synth
    from rpgo_gb300.params import QUIET, RobustSolverParams

    s = synth.walk3d(400, 100, 30, seed=31)
    p = RobustSolverParams().setPcm3DParams(10.0, 5.0, QUIET).setGncInlierCostThresholdsAtProbability(0.9)
    before = O.set_threads(0)
    try:
        out = []
        for threads in (1, 5):
            O.set_threads(threads)
            o = O.OracleSolver(p)
            assert o.update(s.graph) == 0
            out.append((o.estimate()[1], o.gnc_weights()))
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    finally:
        O.set_threads(before)


def _scan_ops_python(n, adj):
    """findCliqueHeu.cpp:32-117 with a counter on the inner linear search."""
    nb = [[j for j in range(n) if j != i and (adj[i, j >> 5] >> np.uint32(j & 31)) & 1] for i in range(n)]
    deg = [len(x) for x in nb]
    S = [0] * ((max(deg) if n else 0) + 1)
    maxclq, ops = -1, 0
    for v in range(n):
        if maxclq > deg[v]:
            continue
        pos = 0
        S[pos] = v
        pos += 1
        for u in nb[v]:
            if maxclq <= deg[u]:
                S[pos] = u
                pos += 1
        icc = 0
        while pos > 0:
            icc += 1
            m = S[pos - 1]
            S1 = []
            for a in range(pos):
                for e, u in enumerate(nb[m]):
                    ops += 1
                    if S[a] == u and maxclq <= deg[u]:
                        S1.append(S[a])
                        break
            for a, x in enumerate(S1):
                S[a] = x
            pos = len(S1)
        if maxclq < icc:
            maxclq = icc
    return ops


@pytest.mark.parametrize("seed", range(4))
def test_clique_scan_op_count(seed):
    rng = np.random.default_rng(300 + seed)
    n = int(rng.integers(2, 60))
    iu = np.triu_indices(n, 1)
    m = rng.random(len(iu[0])) < rng.uniform(0.2, 0.9)
    adj = _bits(n, list(zip(iu[0][m], iu[1][m])))
    assert O.clique_scan_ops(adj, n) == _scan_ops_python(n, adj)


def test_clique_bit_rows_on_dense_planted_graphs():
    # dense graphs (the regime of the 50,000-pose benchmark matrix): the
    # bit-row form equals the linear search, size and index list
    rng = np.random.default_rng(43)
    for n, p in ((400, 0.8), (700, 0.95)):
        dense = np.triu(rng.random((n, n)) < p, 1)
        members = rng.choice(n, n // 2, replace=False)
        dense[np.ix_(members, members)] = True
        iu = np.nonzero(np.triu(dense, 1))
        adj = _bits(n, list(zip(iu[0], iu[1])))
        before = O.set_clique_impl(0)
        try:
            ref = O.max_clique_heu(adj, n)
            O.set_clique_impl(2)
            got = O.max_clique_heu(adj, n)
        finally:
            O.set_clique_impl(before)
        assert ref[0] == got[0] and np.array_equal(ref[1], got[1])


def test_clique_scan_op_estimate_near_count():
    # the bit-row estimate (positions in N(m) to the 64-bit word) against
    # the exact count on dense random graphs with a planted clique
    rng = np.random.default_rng(41)
    for n, p in ((300, 0.6), (500, 0.9)):
        dense = np.triu(rng.random((n, n)) < p, 1)
        members = rng.choice(n, n // 3, replace=False)
        dense[np.ix_(members, members)] = True
        iu = np.nonzero(np.triu(dense, 1))
        adj = _bits(n, list(zip(iu[0], iu[1])))
        exact, est = O.clique_scan_ops(adj, n), O.clique_scan_ops(adj, n, exact=False)
        assert abs(est - exact) <= 0.02 * exact, (n, exact, est)

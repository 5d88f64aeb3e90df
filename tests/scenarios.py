"""The reference's own unit and integration tests, restated as data.

Each scenario is (params, steps); a step is (graph, optimize_graph,
expectations). The same scenarios run against the CPU oracle (CPU suite)
and against the CUDA library through its C ABI (GPU suite). Expected values
are the reference's EXPECT lines:
  tests/testPcm.cpp:17-192          Pcm3D odometry / pairwise checks
  tests/testPcmSimple.cpp:18-390    PcmSimple3D checks
  tests/testPcmDoOptimize.cpp:20-140
  tests/testLoadGraph.cpp:25-580    robot_a / robot_b integration
  tests/testGnc.cpp:25-259          GNC weights
  tests/testMultiRobot.cpp:22-188   inter-robot groups
The reference calls Pcm::removeOutliers directly in the unit tests; here the
same factor sequence goes through RobustSolver::update with
optimize_graph=False, which runs removeOutliers and nothing else.
"""
import math

import numpy as np

from rpgo_gb300.graph import Graph, isotropic_variance, pose3, rot3_rz, symbol
from rpgo_gb300.params import QUIET, RobustSolverParams

R90 = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
RM90 = np.array([[0.0, 1.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
R180 = np.array([[-1.0, 0.0, 0.0], [0.0, -1.0, 0.0], [0.0, 0.0, 1.0]])


def _prior_step(noise_var=0.01):
    g = Graph(3)
    g.insert(0, pose3())
    g.add_prior(0, pose3(), isotropic_variance(6, noise_var))
    return g


def _odom(i, R, t, var=0.1):
    g = Graph(3)
    g.insert(i + 1, pose3(R, t))
    g.add_between(i, i + 1, pose3(R, t), isotropic_variance(6, var))
    return g


def _lc(a, b, R, t, var=0.1):
    return Graph(3).add_between(a, b, pose3(R, t), isotropic_variance(6, var))


def pcm_odometry_check():
    p = RobustSolverParams().setPcm3DParams(0.3, -1.0, QUIET)
    steps = [(_prior_step(), False, {})]
    for i in range(3):
        steps.append((_odom(i, R90, (1, 0, 0)), False, {}))
    steps[-1] = (steps[-1][0], False, dict(num_factors=4, num_values=4))
    steps.append((_lc(3, 0, rot3_rz(1.51), (0.8, 0, 0), 0.1), False,
                  dict(num_factors=5, num_values=4, do_optimize=1)))
    steps.append((_lc(3, 0, rot3_rz(1.51), (0.8, 0, 0), 0.05), False,
                  dict(num_factors=5, num_values=4, do_optimize=1)))
    return p, steps


def _consistency_base():
    steps = [(_prior_step(), False, {})]
    for i in range(2):
        steps.append((_odom(i, R90, (1, 0, 0)), False, {}))
    for i in range(2, 6):
        steps.append((_odom(i, None, (1, 0, 0)), False, {}))
    steps[-1] = (steps[-1][0], False, dict(num_factors=7, num_values=7))
    return steps


def pcm_consistency_check():
    p = RobustSolverParams().setPcm3DParams(-1.0, 0.5, QUIET)
    steps = _consistency_base()
    steps.append((_lc(3, 0, rot3_rz(3.1416), (0, 0.9, 0)), False, {}))
    steps.append((_lc(4, 0, rot3_rz(3.1416), (-1, 0.8, 0)), False, dict(num_factors=9, do_optimize=1)))
    steps.append((_lc(5, 0, rot3_rz(0.99 * 3.1416), (-1.8, 0.8, 0)), False, dict(num_factors=10, do_optimize=1)))
    steps.append((_lc(6, 0, rot3_rz(0.98 * 3.1416), (-2.6, 0.6, 0)), False, dict(num_factors=10, do_optimize=1)))
    return p, steps


def pcm_simple_odom_trans():
    p = RobustSolverParams().setPcmSimple3DParams(0.051, 100.0, -1.0, -1.0, QUIET)
    steps = [(_prior_step(), False, {})]
    for i in range(3):
        steps.append((_odom(i, R90, (1, 0, 0)), False, {}))
    steps[-1] = (steps[-1][0], False, dict(num_factors=4, num_values=4))
    steps.append((_lc(3, 0, R90, (0.8, 0, 0), 0.1), False, dict(num_factors=5, do_optimize=1)))
    steps.append((_lc(3, 0, R90, (0.792, 0, 0), 0.05), False, dict(num_factors=5, do_optimize=1)))
    return p, steps


def pcm_simple_odom_rot():
    p = RobustSolverParams().setPcmSimple3DParams(100.0, 0.005, -1.0, -1.0, QUIET)
    steps = [(_prior_step(), False, {})]
    for i in range(3):
        steps.append((_odom(i, R90, (1, 0, 0)), False, {}))
    steps.append((_lc(3, 0, rot3_rz(1.551), (1.0, 0, 0)), False, dict(num_factors=5, do_optimize=1)))
    steps.append((_lc(3, 0, rot3_rz(1.55), (1.0, 0, 0)), False, dict(num_factors=5, do_optimize=1)))
    return p, steps


def pcm_simple_consistency_trans():
    p = RobustSolverParams().setPcmSimple3DParams(-1.0, -1.0, 0.05, 100.0, QUIET)
    steps = _consistency_base()
    steps.append((_lc(3, 0, R180, (0, 0.9, 0)), False, {}))
    steps.append((_lc(4, 0, rot3_rz(3.1416), (-0.9, 0.9, 0)), False, dict(num_factors=9, do_optimize=1)))
    steps.append((_lc(5, 0, rot3_rz(3.1416), (-1.9, 0.8, 0)), False, dict(num_factors=10, do_optimize=1)))
    steps.append((_lc(6, 0, rot3_rz(3.1416), (-2.8, 0.75, 0)), False, dict(num_factors=10, do_optimize=1)))
    return p, steps


def pcm_simple_consistency_rot():
    p = RobustSolverParams().setPcmSimple3DParams(-1.0, -1.0, 100.0, 0.005, QUIET)
    steps = _consistency_base()
    steps.append((_lc(3, 0, R180, (0, 1.0, 0)), False, {}))
    steps.append((_lc(4, 0, rot3_rz(3.141), (-1.0, 1.0, 0)), False, dict(num_factors=9, do_optimize=1)))
    steps.append((_lc(5, 0, rot3_rz(3.13), (-2.0, 1.0, 0)), False, dict(num_factors=10, do_optimize=1)))
    steps.append((_lc(6, 0, rot3_rz(3.12), (-3.0, 1.0, 0)), False, dict(num_factors=10, do_optimize=1)))
    return p, steps


def do_optimize_odometry():
    p = RobustSolverParams().setPcm3DParams(-1.0, 1.0, QUIET)
    noise = isotropic_variance(6, 0.01)
    s1 = Graph(3).insert(0, pose3()).add_prior(0, pose3(), noise)
    s2 = Graph(3).insert(1, pose3(None, (1, 0, 0))).add_between(0, 1, pose3(None, (1, 0, 0)), noise)
    return p, [(s1, False, dict(num_factors=1, num_values=1)),
               (s2, False, dict(num_factors=2, num_values=2, do_optimize=0))]


def do_optimize_odometry_no_prior():
    p = RobustSolverParams().setPcm3DParams(-1.0, 1.0, QUIET)
    noise = isotropic_variance(6, 0.01)
    s1 = Graph(3).insert(0, pose3())
    s2 = Graph(3).insert(1, pose3(None, (1, 0, 0))).add_between(0, 1, pose3(None, (1, 0, 0)), noise)
    return p, [(s1, False, dict(num_factors=0, num_values=1)),
               (s2, False, dict(num_factors=1, num_values=2, do_optimize=0))]


def do_optimize_loop_closure():
    p = RobustSolverParams().setPcm3DParams(-1.0, 1.0, QUIET)
    noise = isotropic_variance(6, 0.01)
    odom = pose3(None, (1, 0, 0))
    s1 = Graph(3).insert(0, pose3())
    s2 = Graph(3).insert(1, odom).add_between(0, 1, odom, noise)
    s3 = Graph(3).insert(2, pose3(None, (0, 0, 0))).add_between(1, 2, pose3(None, (-1, 0, 0)), noise)
    s4 = Graph(3).add_between(2, 0, pose3(), noise)
    return p, [(s1, False, {}), (s2, False, {}), (s3, False, dict(num_factors=2, num_values=3)),
               (s4, False, dict(num_factors=3, num_values=3, do_optimize=1))]


# ------------------------------------------------------------------ robot_a / robot_b
def _with_prior(g):
    g = g.copy()
    k = symbol("a", 0)
    g.add_prior(k, g.value(k), isotropic_variance(6, 0.01))
    return g


def _inter(pairs, noise_var=0.01):
    g = Graph(3)
    for a, b in pairs:
        g.add_between(symbol("a", a), symbol("b", b), pose3(), isotropic_variance(6, noise_var))
    return g


def load_graph_scenarios(robot_a, robot_b):
    """name -> (params, steps) for testLoadGraph.cpp and testGnc.cpp."""
    out = {}
    P = RobustSolverParams
    out["Load1"] = (P().setPcm3DParams(0.0, 10.0, QUIET), [(_with_prior(robot_a), True, dict(num_factors=50,
                                                                                                 num_values=50))])
    out["Add1"] = (P().setPcm3DParams(0.0, 0.0, QUIET), [
        (_with_prior(robot_a), True, {}),
        (robot_b, True, dict(num_factors=91, num_values=92)),
        (_inter([(1, 1), (2, 2)]), True, dict(num_factors=92, num_values=92))])
    out["Load2"] = (P().setPcm3DParams(100.0, 100.0, QUIET), [(_with_prior(robot_a), True,
                                                                dict(num_factors=53, num_values=50))])
    out["Add2"] = (P().setPcm3DParams(100.0, 100.0, QUIET), [
        (_with_prior(robot_a), True, {}),
        (robot_b, True, dict(num_factors=96, num_values=92)),
        (_inter([(1, 1)]), True, dict(num_factors=97, num_values=92))])
    out["Load1NoPrior"] = (P().setPcm3DParams(0.0, 10.0, QUIET), [(robot_a, True, dict(num_factors=49,
                                                                                         num_values=50))])
    out["NoRejectLoad"] = (P().setNoRejection(QUIET), [(_with_prior(robot_a), True, dict(num_factors=53,
                                                                                           num_values=50))])
    out["NoRejectAdd"] = (P().setNoRejection(QUIET), [
        (_with_prior(robot_a), True, {}),
        (robot_b, True, dict(num_factors=96, num_values=92)),
        (_inter([(1, 1)]), True, dict(num_factors=97, num_values=92))])
    out["Load1PcmSimple"] = (P().setPcmSimple3DParams(0.001, 0.0001, QUIET), [
        (_with_prior(robot_a), True, dict(num_factors=50, num_values=50))])
    out["Add1PcmSimple"] = (P().setPcmSimple3DParams(0.0, 0.0, QUIET), [
        (_with_prior(robot_a), True, {}),
        (robot_b, True, dict(num_factors=91, num_values=92)),
        (_inter([(1, 1), (2, 2)]), True, dict(num_factors=92, num_values=92))])
    out["Load2PcmSimple"] = (P().setPcmSimple3DParams(100.0, 100.0, QUIET), [
        (_with_prior(robot_a), True, dict(num_factors=53, num_values=50))])
    out["Add2PcmSimple"] = (P().setPcmSimple3DParams(100.0, 100.0, QUIET), [
        (_with_prior(robot_a), True, {}),
        (robot_b, True, dict(num_factors=96, num_values=92)),
        (_inter([(1, 1)]), True, dict(num_factors=97, num_values=92))])
    out["Load1NoPriorPcmSimple"] = (P().setPcmSimple3DParams(100.0, 100.0, QUIET), [
        (robot_a, True, dict(num_factors=52, num_values=50))])
    # testGnc.cpp
    out["GncDefault"] = (P().setPcm3DParams(100.0, 100.0, QUIET).setGncInlierCostThresholdsAtProbability(0.01), [
        (_with_prior(robot_a), True, dict(num_factors=53, num_values=50, num_weights=53,
                                          weights_segment=(50, 3, 0.0), weights_sum=50.0, num_lc_inliers=0))])
    out["GncHighThreshold"] = (P().setPcm3DParams(100.0, 100.0, QUIET).setGncInlierCostThresholdsAtProbability(0.99),
                               [(_with_prior(robot_a), True, dict(num_factors=53, num_values=50, num_weights=53,
                                                                  weights_segment=(50, 3, 3.0), weights_sum=53.0,
                                                                  num_lc_inliers=3))])
    out["GncMultirobotDefault"] = (P().setPcm3DParams(100.0, 100.0, QUIET).setGncInlierCostThresholds(1.0), [
        (_with_prior(robot_a), True, {}),
        (robot_b, True, dict(num_factors=96, num_values=92, num_weights=96, weights_segment=(91, 5, 0.0),
                             weights_sum=91.0, num_lc_inliers=0)),
        (_inter([(1, 1), (2, 2)]), True, dict(num_factors=98, num_values=92, num_weights=98,
                                              weights_segment=(91, 7, 2.0), weights_sum=93.0, num_lc_inliers=2))])
    out["GncMultirobotHighThreshold"] = (P().setPcm3DParams(100.0, 100.0, QUIET).setGncInlierCostThresholds(100.0), [
        (_with_prior(robot_a), True, {}),
        (robot_b, True, dict(num_factors=96, num_values=92, num_weights=96, weights_segment=(91, 5, 5.0),
                             weights_sum=96.0, num_lc_inliers=5)),
        (_inter([(1, 1), (2, 2)]), True, dict(num_factors=98, num_values=92, num_weights=98,
                                              weights_segment=(91, 7, 7.0), weights_sum=98.0, num_lc_inliers=7))])
    return out


def multi_robot_pcm():
    p = RobustSolverParams().setPcm3DParams(3.0, 0.05, QUIET)
    noise = isotropic_variance(6, 0.1)
    a, b = (lambda i: symbol("a", i)), (lambda i: symbol("b", i))
    steps = [(Graph(3).insert(a(0), pose3()).insert(b(0), pose3(None, (0, -1, 0))), True, {})]
    odom = pose3(None, (1, 0, 0))
    for i in range(3):
        g = Graph(3).insert(a(i + 1), odom).insert(b(i + 1), odom)
        g.add_between(a(i), a(i + 1), odom, noise).add_between(b(i), b(i + 1), odom, noise)
        steps.append((g, True, {}))
    for i in range(3, 5):
        o = pose3(R90, (1, 0, 0))
        steps.append((Graph(3).insert(a(i + 1), o).add_between(a(i), a(i + 1), o, noise), True, {}))
    for i in range(3, 5):
        o = pose3(RM90, (1, 0, 0))
        steps.append((Graph(3).insert(b(i + 1), o).add_between(b(i), b(i + 1), o, noise), True, {}))
    g = Graph(3).add_between(b(1), a(1), pose3(None, (0, 1, 0)), noise)
    g.add_between(b(4), a(4), pose3(R180, (-1, 0, 0)), noise)
    steps.append((g, True, dict(num_factors=12, num_values=12)))
    g = Graph(3).add_between(a(2), b(2), pose3(None, (0, -1, 0)), noise)
    g.add_between(b(5), a(5), pose3(None, (0, -3.3, 0)), noise)
    steps.append((g, True, dict(num_factors=12, num_values=12)))
    g = Graph(3).add_between(a(4), a(1), pose3(RM90, (0, 3, 0)), noise)
    g.add_between(a(4), a(2), pose3(rot3_rz(-1.54), (0, 2, 0)), noise)
    steps.append((g, True, dict(num_factors=13, num_values=12)))
    return p, steps


PCM_SCENARIOS = {
    "PcmOdometryCheck": pcm_odometry_check,
    "PcmConsistencyCheck": pcm_consistency_check,
    "PcmSimpleOdomTransCheck": pcm_simple_odom_trans,
    "PcmSimpleOdomRotCheck": pcm_simple_odom_rot,
    "PcmSimpleConsistencyTransCheck": pcm_simple_consistency_trans,
    "PcmSimpleConsistencyRotCheck": pcm_simple_consistency_rot,
    "DoOptimizeOdometry": do_optimize_odometry,
    "DoOptimizeOdometryNoPrior": do_optimize_odometry_no_prior,
    "DoOptimizeLoopClosure": do_optimize_loop_closure,
    "MultiRobotPcm": multi_robot_pcm,
}


def run_scenario(make_solver, params, steps):
    """Run steps; returns list of failures (empty when all expectations hold)."""
    s = make_solver(params)
    fails = []
    for idx, (g, opt, exp) in enumerate(steps):
        rc = s.update(g, opt)
        if rc != 0:
            fails.append(f"step {idx}: status {rc}")
            continue
        c = s.counts()
        for k, v in exp.items():
            if k == "num_factors" and c.num_factors != v:
                fails.append(f"step {idx}: num_factors {c.num_factors} != {v}")
            elif k == "num_values" and c.num_values != v:
                fails.append(f"step {idx}: num_values {c.num_values} != {v}")
            elif k == "do_optimize" and c.last_do_optimize != v:
                fails.append(f"step {idx}: do_optimize {c.last_do_optimize} != {v}")
            elif k == "num_lc_inliers" and c.num_lc_inliers != v:
                fails.append(f"step {idx}: num_lc_inliers {c.num_lc_inliers} != {v}")
            elif k == "num_weights" and c.num_gnc_weights != v:
                fails.append(f"step {idx}: num_weights {c.num_gnc_weights} != {v}")
            elif k == "weights_sum":
                w = s.gnc_weights()
                if abs(w.sum() - v) > 1e-9:
                    fails.append(f"step {idx}: weights sum {w.sum()} != {v}")
            elif k == "weights_segment":
                w = s.gnc_weights()
                a0, n, tot = v
                if abs(w[a0:a0 + n].sum() - tot) > 1e-9:
                    fails.append(f"step {idx}: weights[{a0}:{a0 + n}] sum {w[a0:a0 + n].sum()} != {tot}")
    return fails, s

"""Symbolic analysis of the direct solve's plan builder (chol_plan.cpp), no
GPU: the column structures that the elimination tree gives for a fixed order
equal the elimination game's (the neighbours of each variable when it is
eliminated) on random pose-graph-shaped and random graphs under random,
identity and reversed orders; and every level's tasks come in non-increasing
order of weight with every slot in one level (the kernel's lane groups take
consecutive tasks)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("plan") / "libplansym.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread",
                    os.path.join(ROOT, "tests", "native", "plan_symbolic.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    lib.plan_symbolic_check.restype = C.c_int
    lib.plan_task_order_check.restype = C.c_int
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _pose_graph(n, closures, radius, rng):
    # odometry chain plus local closures (|i - j| <= radius), as the benchmark graphs
    e = [(i, i + 1) for i in range(n - 1)]
    for _ in range(closures):
        i = int(rng.integers(0, n))
        j = int(np.clip(i + rng.integers(2, radius + 1) * rng.choice([-1, 1]), 0, n - 1))
        if i != j:
            e.append((i, j))
    return e


def _random_graph(n, m, rng):
    e = []
    for _ in range(m):
        i, j = (int(x) for x in rng.integers(0, n, 2))
        if i != j:
            e.append((i, j))
    return e


def _edges(e):
    a = np.array(e, dtype=np.int32).reshape(-1, 2)
    return np.ascontiguousarray(a[:, 0]), np.ascontiguousarray(a[:, 1])


@pytest.mark.parametrize("seed", range(6))
def test_elimination_tree_structure_equals_elimination_game(lib, seed):
    rng = np.random.default_rng(seed)
    graphs = [_pose_graph(int(rng.integers(20, 400)), int(rng.integers(0, 120)), 30, rng),
              _random_graph(int(rng.integers(10, 120)), int(rng.integers(5, 400)), rng),
              [(0, 1)], []]
    for e in graphs:
        n = 1 + max([max(i, j) for i, j in e], default=1)
        ei, ej = _edges(e) if e else (np.zeros(0, np.int32), np.zeros(0, np.int32))
        for order in (rng.permutation(n), np.arange(n), np.arange(n)[::-1]):
            order = np.ascontiguousarray(order, dtype=np.int32)
            assert lib.plan_symbolic_check(n, len(ei), _p(ei), _p(ej), _p(order)) == 0


@pytest.mark.parametrize("d", [3, 6])
def test_level_tasks_by_non_increasing_weight(lib, d):
    rng = np.random.default_rng(10 + d)
    for n, closures in [(300, 60), (2000, 500), (50, 0)]:
        ei, ej = _edges(_pose_graph(n, closures, 40, rng))
        levels = C.c_int(0)
        assert lib.plan_task_order_check(n, d, len(ei), _p(ei), _p(ej), C.byref(levels)) == 0
        assert levels.value >= 1

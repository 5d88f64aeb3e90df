"""Host logic of the direct solve: the symbolic plan (make_chol_plan) and the
phase order of the GPU kernel, run by a sequential CPU emulation of the same
items (tests/native/chol_emulate.cpp), against a dense numpy solve of
(H + lambda D) x = b on random pose-graph-shaped systems. No GPU."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "kimera-rpgo_gb300", "csrc")


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("chol") / "libcholemu.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CSRC,
                    os.path.join(ROOT, "tests", "native", "chol_emulate.cpp"), os.path.join(CSRC, "chol_plan.cpp"),
                    "-o", out], check=True)
    lib = C.CDLL(out)
    lib.chol_emulate.restype = C.c_int
    return lib


def _system(N, d, edges, priors, seed):
    rng = np.random.default_rng(seed)
    kind, vi, vj, fH = [], [], [], []
    Hd = np.zeros((N, d, d))
    for (i, j) in edges:
        # pose-graph-like Jacobians: -w Q (Q orthogonal) and w (I + small),
        # so that H behaves like a weighted graph Laplacian (well conditioned
        # enough for the dense reference solve)
        w = rng.uniform(0.5, 2.0)
        Q, _ = np.linalg.qr(rng.normal(size=(d, d)))
        Ji = -w * Q
        Jj = w * (np.eye(d) + 0.1 * rng.normal(size=(d, d)))
        kind.append(0), vi.append(i), vj.append(j)
        Hd[i] += Ji.T @ Ji
        Hd[j] += Jj.T @ Jj
        fH.append(Ji.T @ Jj)
    for v in priors:
        J = rng.normal(size=(d, d)) + 3 * np.eye(d)
        kind.append(1), vi.append(v), vj.append(v)
        Hd[v] += J.T @ J
        fH.append(np.zeros((d, d)))
    H = np.zeros((N * d, N * d))
    for v in range(N):
        H[v * d:(v + 1) * d, v * d:(v + 1) * d] += Hd[v]
    for f, (i, j) in enumerate(edges):
        H[i * d:(i + 1) * d, j * d:(j + 1) * d] += fH[f]
        H[j * d:(j + 1) * d, i * d:(i + 1) * d] += fH[f].T
    damp = np.abs(np.diagonal(H)).reshape(N, d).copy()
    rhs = rng.normal(size=N * d)
    return (np.array(kind, np.int32), np.array(vi, np.int32), np.array(vj, np.int32), Hd,
            np.ascontiguousarray(np.array(fH).reshape(-1, d, d)), H, damp, rhs)


def _run(lib, N, d, sysm, lam):
    kind, vi, vj, Hd, fH, H, damp, rhs = sysm
    x = np.zeros(N * d)
    info = np.zeros(5, np.int32)
    p = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)
    lib.chol_emulate(N, d, len(kind), p(kind), p(vi), p(vj), p(Hd), p(fH), p(rhs), C.c_double(lam), p(damp),
                     x.ctypes.data_as(C.c_void_p), info.ctypes.data_as(C.c_void_p))
    A = H + lam * np.diag(damp.reshape(-1))
    ref = np.linalg.solve(A, rhs)
    return x, ref, info


def _pose_graph(N, n_lc, seed):
    rng = np.random.default_rng(seed)
    edges = [(i, i + 1) for i in range(N - 1)]
    for _ in range(n_lc):
        i, j = sorted(rng.choice(N, 2, replace=False))
        edges.append((int(i), int(j)))
    return edges


@pytest.mark.parametrize("d", [6, 3])
@pytest.mark.parametrize("N,n_lc,seed", [(1, 0, 0), (2, 0, 1), (40, 0, 2), (300, 60, 3), (120, 400, 4), (900, 150, 5)])
def test_emulated_direct_solve_matches_dense(emu, d, N, n_lc, seed):
    edges = _pose_graph(N, n_lc, seed) if N > 1 else []
    sysm = _system(N, d, edges, [0], seed)
    for lam in (0.0, 1e-3):
        x, ref, info = _run(emu, N, d, sysm, lam)
        assert info[4] == 0
        assert info[0] + info[1] == N and info[1] >= 1
        assert np.allclose(x, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max()), np.abs(x - ref).max()


def test_emulated_direct_solve_forest_and_duplicate_edges(emu):
    # two components (each anchored by a prior) and repeated closures between
    # the same pair of variables (their Hessian blocks add)
    d = 6
    edges = [(i, i + 1) for i in range(49)] + [(i, i + 1) for i in range(50, 99)] + [(3, 40), (3, 40), (60, 90)]
    sysm = _system(100, d, edges, [0, 50], 9)
    x, ref, info = _run(emu, 100, d, sysm, 1e-4)
    assert info[4] == 0
    assert np.allclose(x, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())


def test_emulated_direct_solve_reports_indefinite_system(emu):
    # without a prior the pose-graph Hessian of a tree is singular only in
    # theory; a negative diagonal makes it indefinite for sure
    d = 3
    edges = _pose_graph(30, 5, 11)
    kind, vi, vj, Hd, fH, H, damp, rhs = _system(30, d, edges, [0], 11)
    Hd = Hd.copy()
    Hd[7] -= 1e6 * np.eye(d)
    H = H.copy()
    H[21:24, 21:24] -= 1e6 * np.eye(d)
    x, ref, info = _run(emu, 30, d, (kind, vi, vj, Hd, fH, H, damp, rhs), 0.0)
    assert info[4] == 1


def test_plan_is_deterministic(emu):
    # the plan's candidate orders are computed on several threads; the chosen
    # plan, and so the emulated solve, must not depend on their timing
    d = 6
    edges = _pose_graph(500, 150, 12)
    sysm = _system(500, d, edges, [0], 12)
    runs = [_run(emu, 500, d, sysm, 1e-3) for _ in range(4)]
    for x, _, info in runs[1:]:
        assert np.array_equal(x, runs[0][0])
        assert np.array_equal(info, runs[0][2])


def test_emulated_joint_batch_plan_matches_dense(emu):
    # the joint batch's merged plan: three graphs of different sizes and
    # levels, planned without dense tails and merged, each damped with its
    # own lambda; the emulated solve equals the dense solve of each graph
    emu.chol_emulate_joint.restype = C.c_int
    d = 6
    sizes = [(300, 60, 21), (40, 0, 22), (120, 200, 23)]
    lams = np.array([1e-3, 0.0, 10.0])
    parts = [_system(N, d, _pose_graph(N, n_lc, seed), [0], seed) for N, n_lc, seed in sizes]
    Ns = np.array([N for N, _, _ in sizes], np.int32)
    Fs = np.array([len(pt[0]) for pt in parts], np.int32)
    voff = np.concatenate([[0], np.cumsum(Ns)])
    kind = np.concatenate([pt[0] for pt in parts]).astype(np.int32)
    vi = np.concatenate([pt[1] + voff[g] for g, pt in enumerate(parts)]).astype(np.int32)
    vj = np.concatenate([pt[2] + voff[g] for g, pt in enumerate(parts)]).astype(np.int32)
    Hd = np.ascontiguousarray(np.concatenate([pt[3] for pt in parts]))
    fH = np.ascontiguousarray(np.concatenate([pt[4] for pt in parts]))
    damp = np.ascontiguousarray(np.concatenate([pt[6] for pt in parts]))
    rhs = np.ascontiguousarray(np.concatenate([pt[7] for pt in parts]))
    x = np.zeros(int(voff[-1]) * d)
    info = np.zeros(5, np.int32)
    p = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)
    emu.chol_emulate_joint(3, p(Ns), p(Fs), d, p(kind), p(vi), p(vj), p(Hd), p(fH), p(rhs), p(lams), p(damp),
                           x.ctypes.data_as(C.c_void_p), info.ctypes.data_as(C.c_void_p))
    assert info[4] == 0 and info[1] == 0 and info[0] == voff[-1]
    for g, pt in enumerate(parts):
        H, dmp, b = pt[5], pt[6], pt[7]
        ref = np.linalg.solve(H + lams[g] * np.diag(dmp.reshape(-1)), b)
        xg = x[voff[g] * d:voff[g + 1] * d]
        assert np.allclose(xg, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max()), (g, np.abs(xg - ref).max())

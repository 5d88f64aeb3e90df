"""Seeded synthetic pose graphs with inlier and outlier loop closures.

The reference measures on no public dataset; these generators produce the
workload shapes the benchmark names:
  * grid2d:   2D walk with 1 m forward steps and +-pi/2 yaw turns (p = 0.2 per
              step); odometry sigma_t 0.05 m, sigma_theta 0.01 rad; inlier
              closures between ground-truth poses within 2 m; outliers on
              random pose pairs with t ~ U[-10, 10]^2 and yaw ~ U[-pi, pi].
  * walk3d:   3D random walk with 0.5 m steps along body x and rotation
              increments Exp(w), w ~ N(0, 0.1^2 I); odometry sigma_t 0.02 m,
              sigma_R 0.005 rad; inlier closures within 3 m; outliers with t
              uniform in a 20 m cube and a uniformly random rotation (Shoemake).
Closures never join consecutive keys (|i - j| >= 2), so they are never
mistaken for odometry. Initial values are dead reckoning from the noisy
odometry; a prior anchors the first pose at its initial value.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
from scipy.spatial import cKDTree

from .graph import Graph, diagonal_sigmas, isotropic_variance, symbol


def _skew(w):
    return np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])


def so3_exp(w):
    th = np.linalg.norm(w)
    K = _skew(w)
    if th < 1e-12:
        return np.eye(3) + K
    return np.eye(3) + math.sin(th) / th * K + (1 - math.cos(th)) / th ** 2 * (K @ K)


def se3_exp(xi):
    w, v = xi[:3], xi[3:]
    R = so3_exp(w)
    th = np.linalg.norm(w)
    K = _skew(w)
    if th < 1e-12:
        V = np.eye(3) + 0.5 * K
    else:
        V = np.eye(3) + (1 - math.cos(th)) / th ** 2 * K + (th - math.sin(th)) / th ** 3 * (K @ K)
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = V @ v
    return T


def _skew_n(w):
    K = np.zeros(w.shape[:-1] + (3, 3))
    K[..., 0, 1], K[..., 0, 2], K[..., 1, 2] = -w[..., 2], w[..., 1], -w[..., 0]
    K[..., 1, 0], K[..., 2, 0], K[..., 2, 1] = w[..., 2], -w[..., 1], w[..., 0]
    return K


def se3_exp_n(xi):
    """Batched se3_exp: (..., 6) -> (..., 4, 4)."""
    w, v = xi[..., :3], xi[..., 3:]
    th = np.linalg.norm(w, axis=-1)[..., None, None]
    K = _skew_n(w)
    K2 = K @ K
    small = th < 1e-12
    ths = np.where(small, 1.0, th)
    A = np.where(small, 1.0, np.sin(ths) / ths)
    B = np.where(small, 0.0, (1 - np.cos(ths)) / ths ** 2)
    Bv = np.where(small, 0.5, B)
    C = np.where(small, 0.0, (ths - np.sin(ths)) / ths ** 3)
    I = np.eye(3)
    T = np.zeros(xi.shape[:-1] + (4, 4))
    T[..., :3, :3] = I + A * K + B * K2
    T[..., :3, 3] = ((I + Bv * K + C * K2) @ v[..., None])[..., 0]
    T[..., 3, 3] = 1.0
    return T


def uniform_rotation(rng):
    u1, u2, u3 = rng.random(3)
    q = (math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
         math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3))
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _T(p):  # 12-vector -> 4x4
    T = np.eye(4)
    T[:3, :3] = p[:9].reshape(3, 3)
    T[:3, 3] = p[9:]
    return T


def _p(T):
    return np.concatenate([T[:3, :3].reshape(9), T[:3, 3]])


def _M2(p):  # (c, s, x, y) -> 3x3
    c, s, x, y = p
    return np.array([[c, -s, x], [s, c, y], [0, 0, 1.0]])


def _p2(M):
    return np.array([M[0, 0], M[1, 0], M[0, 2], M[1, 2]])


def _se2_exp(v):
    x, y, th = v
    c, s = math.cos(th), math.sin(th)
    if abs(th) < 1e-12:
        A, B = 1.0, 0.0
    else:
        A, B = s / th, (1 - c) / th
    return np.array([[c, -s, A * x - B * y], [s, c, B * x + A * y], [0, 0, 1.0]])


@dataclass
class Synthetic:
    graph: Graph               # odometry, prior, then loop closures in arrival order
    gt: np.ndarray             # ground-truth poses (n x stride)
    is_outlier: np.ndarray     # per loop closure, arrival order
    n_odom: int
    n_lc: int


def _pick_pairs(rng, pos, radius, count, min_gap=2):
    tree = cKDTree(pos)
    pairs = np.array(sorted(tree.query_pairs(radius)), dtype=np.int64).reshape(-1, 2)
    if len(pairs):
        pairs = pairs[np.abs(pairs[:, 0] - pairs[:, 1]) >= min_gap]
    if len(pairs) > count:
        pairs = pairs[rng.choice(len(pairs), size=count, replace=False)]
    return pairs


def walk3d(n_poses=5000, n_inliers=1000, n_outliers=333, seed=2, step=0.5, rot_sigma=0.1, sigma_t=0.02,
           sigma_r=0.005, radius=3.0, prefix="a", prior_var=1e-4, clustered_outliers=0, cluster=10):
    """3D random walk. n_outliers closures join uniformly random pose pairs
    with a random measurement; clustered_outliers more come in groups of
    `cluster` that all claim the same wrong place: for a random pose pair
    (a0, b0) and a random rigid offset W, closure k joins a0 + k and b0 + k
    with the measurement of gt[b0 + k] moved by W (mutually consistent,
    inconsistent with the trajectory)."""
    rng = np.random.default_rng(seed)
    sig = np.array([sigma_r] * 3 + [sigma_t] * 3)
    noise = diagonal_sigmas(sig)
    gt = [np.eye(4)]
    est = [np.eye(4)]
    g = Graph(3)
    k = lambda i: symbol(prefix, i)
    g.insert(k(0), _p(est[0]))
    # per step: 3 rotation-increment draws then 6 noise draws (one stream)
    draws = rng.standard_normal((max(n_poses - 1, 0), 9))
    D = se3_exp_n(np.concatenate([draws[:, :3] * rot_sigma, np.zeros((len(draws), 3))], axis=1))
    D[:, :3, 3] = (step, 0, 0)
    Z = D @ se3_exp_n(draws[:, 3:] * sig)
    odom = list(Z)
    for i in range(1, n_poses):
        gt.append(gt[-1] @ D[i - 1])
        est.append(est[-1] @ Z[i - 1])
        g.insert(k(i), _p(est[-1]))
    for i, z in enumerate(odom):
        g.add_between(k(i), k(i + 1), _p(z), noise)
    g.add_prior(k(0), _p(est[0]), isotropic_variance(6, prior_var))
    pos = np.array([T[:3, 3] for T in gt])
    pairs = _pick_pairs(rng, pos, radius, n_inliers)
    lcs = []
    for i, j in pairs:
        a, b = (j, i) if rng.random() < 0.5 else (i, j)
        z = np.linalg.inv(gt[a]) @ gt[b] @ se3_exp(rng.normal(0, 1, 6) * sig)
        lcs.append((a, b, z, False))
    for _ in range(n_outliers):
        while True:
            a, b = rng.integers(0, n_poses, 2)
            if abs(int(a) - int(b)) >= 2:
                break
        z = np.eye(4)
        z[:3, :3] = uniform_rotation(rng)
        z[:3, 3] = rng.uniform(-10, 10, 3)
        lcs.append((int(a), int(b), z, True))
    for _ in range(0, clustered_outliers, cluster):
        while True:
            a0, b0 = (int(x) for x in rng.integers(0, max(n_poses - cluster, 1), 2))
            if abs(a0 - b0) >= cluster + 2:
                break
        W = np.eye(4)
        W[:3, :3] = uniform_rotation(rng)
        W[:3, 3] = rng.uniform(-10, 10, 3)
        made = len(lcs) - len(pairs) - n_outliers
        for c in range(min(cluster, clustered_outliers - made)):
            a, b = a0 + c, b0 + c
            z = np.linalg.inv(gt[a]) @ W @ gt[b] @ se3_exp(rng.normal(0, 1, 6) * sig)
            lcs.append((a, b, z, True))
    order = rng.permutation(len(lcs))
    out = []
    for o in order:
        a, b, z, bad = lcs[o]
        g.add_between(k(a), k(b), _p(z), noise)
        out.append(bad)
    return Synthetic(g, np.array([_p(T) for T in gt]), np.array(out, dtype=bool), len(odom), len(lcs))


def grid2d(n_poses=500, n_inliers=100, n_outliers=20, seed=1, sigma_t=0.05, sigma_th=0.01, radius=2.0,
           prefix="a", prior_var=1e-4):
    rng = np.random.default_rng(seed)
    sig = np.array([sigma_t, sigma_t, sigma_th])
    noise = diagonal_sigmas(sig)
    gt = [np.eye(3)]
    est = [np.eye(3)]
    g = Graph(2)
    k = lambda i: symbol(prefix, i)
    g.insert(k(0), _p2(est[0]))
    odom = []
    for i in range(1, n_poses):
        r = rng.random()
        yaw = math.pi / 2 if r < 0.1 else (-math.pi / 2 if r < 0.2 else 0.0)
        d = _se2_exp(np.array([0.0, 0.0, yaw])) @ np.array([[1, 0, 1.0], [0, 1, 0], [0, 0, 1]])
        gt.append(gt[-1] @ d)
        z = d @ _se2_exp(rng.normal(0, 1, 3) * sig)
        est.append(est[-1] @ z)
        odom.append(z)
        g.insert(k(i), _p2(est[-1]))
    for i, z in enumerate(odom):
        g.add_between(k(i), k(i + 1), _p2(z), noise)
    g.add_prior(k(0), _p2(est[0]), isotropic_variance(3, prior_var))
    pos = np.array([T[:2, 2] for T in gt])
    pairs = _pick_pairs(rng, pos, radius, n_inliers)
    lcs = []
    for i, j in pairs:
        a, b = (j, i) if rng.random() < 0.5 else (i, j)
        z = np.linalg.inv(gt[a]) @ gt[b] @ _se2_exp(rng.normal(0, 1, 3) * sig)
        lcs.append((a, b, z, False))
    for _ in range(n_outliers):
        while True:
            a, b = rng.integers(0, n_poses, 2)
            if abs(int(a) - int(b)) >= 2:
                break
        th = rng.uniform(-math.pi, math.pi)
        t = rng.uniform(-10, 10, 2)
        z = np.array([[math.cos(th), -math.sin(th), t[0]], [math.sin(th), math.cos(th), t[1]], [0, 0, 1.0]])
        lcs.append((int(a), int(b), z, True))
    order = rng.permutation(len(lcs))
    out = []
    for o in order:
        a, b, z, bad = lcs[o]
        g.add_between(k(a), k(b), _p2(z), noise)
        out.append(bad)
    return Synthetic(g, np.array([_p2(M) for M in gt]), np.array(out, dtype=bool), len(odom), len(lcs))


def config_c1():
    """2D grid walk: 500 poses, 100 inlier + 20 outlier closures (seed 1)."""
    return grid2d(500, 100, 20, seed=1)


def config_c2():
    """3D random walk: 5,000 poses, 1,000 inliers, 25% outliers of the closure set (333, seed 2)."""
    return walk3d(5000, 1000, 333, seed=2)


def config_c3():
    """3D random walk: 50,000 poses, 20,000 closures with 30% outliers (seed 3)."""
    return walk3d(50000, 14000, 6000, seed=3)


def config_c4_sizes(n_graphs=512, seed=4):
    """Sizes of the batched workload: per graph (poses, inlier closures,
    outlier closures, seed); poses ~ U[200, 8000], closures 10-30 % of the
    poses, outlier rate ~ U[0, 0.5] of the closures."""
    rng = np.random.default_rng(seed)
    out = []
    for g in range(n_graphs):
        n = int(rng.integers(200, 8001))
        lc = int(round(rng.uniform(0.10, 0.30) * n))
        no = int(round(rng.uniform(0.0, 0.5) * lc))
        out.append((n, lc - no, no, seed + g))
    return out


def config_c4(n_graphs=512, seed=4):
    """Batched workload: independent 3D random walks of the walk3d generator
    with the sizes of config_c4_sizes."""
    return [walk3d(n, ni, no, seed=s) for n, ni, no, s in config_c4_sizes(n_graphs, seed)]


def config_c5(seed=5, n_poses=20000, n_closures=8000, outlier_frac=0.4):
    """Warm-start evaluation graph: 3D random walk of 20,000 poses, 40 %
    outliers, half uniform and half in clusters of 10 mapping to the same
    wrong place."""
    n_out = int(round(outlier_frac * n_closures))
    n_clu = n_out // 2 // 10 * 10
    return walk3d(n_poses, n_closures - n_out, n_out - n_clu, seed=seed, clustered_outliers=n_clu)


def ate(est_poses: np.ndarray, ref_poses: np.ndarray, dim: int = 3) -> float:
    """RMS translation error between two pose arrays in the same gauge."""
    if dim == 3:
        d = est_poses[:, 9:12] - ref_poses[:, 9:12]
    else:
        d = est_poses[:, 2:4] - ref_poses[:, 2:4]
    return float(np.sqrt(np.mean(np.sum(d * d, axis=1))))

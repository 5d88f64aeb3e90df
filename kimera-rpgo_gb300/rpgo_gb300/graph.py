"""Factor-graph model of the robust back-end, in numpy.

This is the host-side mirror of the GTSAM types the reference's API takes
(``gtsam::NonlinearFactorGraph`` of ``BetweenFactor<Pose2|Pose3>`` /
``PriorFactor``, ``gtsam::Values``, ``gtsam::noiseModel``), reduced to what
the robust back-end reads: keys, measured poses, the covariance PCM reads
(``noiseModel()->covariance()``, include/KimeraRPGO/utils/GeometryUtils.h:93-96)
and the square-root information the solver whitens with.

Pose layouts (row-major doubles): Pose3 = R (9) + t (3); Pose2 = (cos, sin, x, y).
Keys are ``gtsam::Symbol`` values ``(chr << 56) | index``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

BETWEEN = 0
PRIOR = 1


# --------------------------------------------------------------------- keys
def symbol(c: str, index: int) -> int:
    return (ord(c) << 56) | int(index)


def symbol_chr(key: int) -> str:
    return chr((int(key) >> 56) & 0xFF)


def symbol_index(key: int) -> int:
    return int(key) & ((1 << 56) - 1)


# --------------------------------------------------------------------- poses
def rot3_quaternion(w: float, x: float, y: float, z: float, normalize: bool = False) -> np.ndarray:
    """Rotation matrix of a quaternion (gtsam::Rot3::Quaternion(w, x, y, z))."""
    if normalize:
        f = 1.0 / math.sqrt(w * w + x * x + y * y + z * z)
        w, x, y, z = f * w, f * x, f * y, f * z
    tx, ty, tz = 2.0 * x, 2.0 * y, 2.0 * z
    twx, twy, twz = tx * w, ty * w, tz * w
    txx, txy, txz = tx * x, ty * x, tz * x
    tyy, tyz, tzz = ty * y, tz * y, tz * z
    return np.array(
        [
            [1.0 - (tyy + tzz), txy - twz, txz + twy],
            [txy + twz, 1.0 - (txx + tzz), tyz - twx],
            [txz - twy, tyz + twx, 1.0 - (txx + tyy)],
        ]
    )


def rot3_rz(theta: float) -> np.ndarray:
    c, s = math.cos(theta), math.sin(theta)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def rot3_to_quaternion(R: np.ndarray) -> Tuple[float, float, float, float]:
    """(w, x, y, z) of a rotation matrix (Shepperd's method)."""
    tr = R[0, 0] + R[1, 1] + R[2, 2]
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2
        return 0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s
    if R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = math.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        return (R[2, 1] - R[1, 2]) / s, 0.25 * s, (R[0, 1] + R[1, 0]) / s, (R[0, 2] + R[2, 0]) / s
    if R[1, 1] > R[2, 2]:
        s = math.sqrt(1.0 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        return (R[0, 2] - R[2, 0]) / s, (R[0, 1] + R[1, 0]) / s, 0.25 * s, (R[1, 2] + R[2, 1]) / s
    s = math.sqrt(1.0 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
    return (R[1, 0] - R[0, 1]) / s, (R[0, 2] + R[2, 0]) / s, (R[1, 2] + R[2, 1]) / s, 0.25 * s


def pose3(R=None, t=(0.0, 0.0, 0.0)) -> np.ndarray:
    R = np.eye(3) if R is None else np.asarray(R, dtype=np.float64)
    return np.concatenate([R.reshape(9), np.asarray(t, dtype=np.float64)])


def pose2(theta: float = 0.0, x: float = 0.0, y: float = 0.0) -> np.ndarray:
    return np.array([math.cos(theta), math.sin(theta), x, y])


def pose3_matrix(p: np.ndarray) -> np.ndarray:
    T = np.eye(4)
    T[:3, :3] = np.asarray(p[:9]).reshape(3, 3)
    T[:3, 3] = p[9:12]
    return T


def pose3_from_matrix(T: np.ndarray) -> np.ndarray:
    return pose3(T[:3, :3], T[:3, 3])


def pose3_compose(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return pose3_from_matrix(pose3_matrix(a) @ pose3_matrix(b))


def pose2_matrix(p: np.ndarray) -> np.ndarray:
    c, s, x, y = p
    return np.array([[c, -s, x], [s, c, y], [0.0, 0.0, 1.0]])


def pose2_compose(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    M = pose2_matrix(a) @ pose2_matrix(b)
    return np.array([M[0, 0], M[1, 0], M[0, 2], M[1, 2]])


# --------------------------------------------------------------------- noise models
def _upper(R: np.ndarray) -> np.ndarray:
    return np.triu(R)


def isotropic_variance(dim: int, variance: float):
    """gtsam::noiseModel::Isotropic::Variance: sigma = sqrt(v), cov = sigma^2."""
    sigma = math.sqrt(variance)
    return isotropic_sigma(dim, sigma)


def isotropic_sigma(dim: int, sigma: float):
    cov = np.eye(dim) * (sigma * sigma)
    R = np.eye(dim) * (1.0 / sigma)
    return cov, R


def diagonal_sigmas(sigmas):
    s = np.asarray(sigmas, dtype=np.float64)
    return np.diag(s * s), np.diag(1.0 / s)


def diagonal_precisions(precisions):
    """gtsam::noiseModel::Diagonal::Precisions -> Variances(1/p) -> Sigmas(sqrt)."""
    p = np.asarray(precisions, dtype=np.float64)
    return diagonal_sigmas(np.sqrt(1.0 / p))


def gaussian_information(info: np.ndarray, smart: bool = True):
    """gtsam::noiseModel::Gaussian::Information (smart: diagonal -> Precisions)."""
    info = np.asarray(info, dtype=np.float64)
    if smart and np.count_nonzero(info - np.diag(np.diag(info))) == 0:
        return diagonal_precisions(np.diag(info))
    L = np.linalg.cholesky(info)
    return np.linalg.inv(info), _upper(L.T)


def gaussian_covariance(cov: np.ndarray, smart: bool = True):
    cov = np.asarray(cov, dtype=np.float64)
    if smart and np.count_nonzero(cov - np.diag(np.diag(cov))) == 0:
        return diagonal_sigmas(np.sqrt(np.diag(cov)))
    info = np.linalg.inv(cov)
    L = np.linalg.cholesky(info)
    return cov.copy(), _upper(L.T)


# --------------------------------------------------------------------- graph container
@dataclass
class Graph:
    """Factors (in order) and values of one update call."""

    dim: int  # 2 or 3
    kind: List[int] = field(default_factory=list)
    key1: List[int] = field(default_factory=list)
    key2: List[int] = field(default_factory=list)
    measured: List[np.ndarray] = field(default_factory=list)
    cov: List[np.ndarray] = field(default_factory=list)
    sqrt_info: List[np.ndarray] = field(default_factory=list)
    value_keys: List[int] = field(default_factory=list)
    value_poses: List[np.ndarray] = field(default_factory=list)

    @property
    def stride(self) -> int:
        return 12 if self.dim == 3 else 4

    @property
    def d(self) -> int:
        return 6 if self.dim == 3 else 3

    def add_between(self, k1: int, k2: int, measured, noise):
        cov, R = noise
        self.kind.append(BETWEEN)
        self.key1.append(int(k1))
        self.key2.append(int(k2))
        self.measured.append(np.asarray(measured, dtype=np.float64))
        self.cov.append(np.asarray(cov, dtype=np.float64))
        self.sqrt_info.append(np.asarray(R, dtype=np.float64))
        return self

    def add_prior(self, k: int, measured, noise):
        cov, R = noise
        self.kind.append(PRIOR)
        self.key1.append(int(k))
        self.key2.append(int(k))
        self.measured.append(np.asarray(measured, dtype=np.float64))
        self.cov.append(np.asarray(cov, dtype=np.float64))
        self.sqrt_info.append(np.asarray(R, dtype=np.float64))
        return self

    def insert(self, k: int, pose):
        self.value_keys.append(int(k))
        self.value_poses.append(np.asarray(pose, dtype=np.float64))
        return self

    def value(self, k: int) -> np.ndarray:
        return self.value_poses[self.value_keys.index(int(k))]

    @property
    def num_factors(self) -> int:
        return len(self.kind)

    def extend(self, other: "Graph") -> "Graph":
        assert other.dim == self.dim
        for name in ("kind", "key1", "key2", "measured", "cov", "sqrt_info", "value_keys", "value_poses"):
            getattr(self, name).extend(getattr(other, name))
        return self

    def copy(self) -> "Graph":
        g = Graph(self.dim)
        return g.extend(self)

    def factors_only(self) -> "Graph":
        g = self.copy()
        g.value_keys, g.value_poses = [], []
        return g

    def arrays(self):
        """Contiguous numpy arrays in C-ABI layout."""
        n, d, st = len(self.kind), self.d, self.stride
        out = dict(
            kind=np.asarray(self.kind, dtype=np.int32).reshape(n),
            key1=np.asarray(self.key1, dtype=np.uint64).reshape(n),
            key2=np.asarray(self.key2, dtype=np.uint64).reshape(n),
            measured=np.ascontiguousarray(np.asarray(self.measured, dtype=np.float64).reshape(n, st)),
            cov=np.ascontiguousarray(np.asarray(self.cov, dtype=np.float64).reshape(n, d, d)),
            sqrt_info=np.ascontiguousarray(np.asarray(self.sqrt_info, dtype=np.float64).reshape(n, d, d)),
            value_keys=np.asarray(self.value_keys, dtype=np.uint64).reshape(len(self.value_keys)),
            value_poses=np.ascontiguousarray(
                np.asarray(self.value_poses, dtype=np.float64).reshape(len(self.value_keys), st)
            ),
        )
        return out


# --------------------------------------------------------------------- g2o
_G2O_TR_SWAP = [3, 4, 5, 0, 1, 2]  # g2o [t; R] <-> GTSAM [R; t]


def _upper21_to_matrix(vals) -> np.ndarray:
    m = np.zeros((6, 6))
    k = 0
    for i in range(6):
        for j in range(i, 6):
            m[i, j] = vals[k]
            m[j, i] = vals[k]
            k += 1
    return m


def parse_g2o_3d(text: str) -> Graph:
    """VERTEX_SE3:QUAT / EDGE_SE3:QUAT as GTSAM load3D reads them: normalised
    quaternions, information reordered from [t; R] to [R; t], noise model
    Gaussian::Information (smart)."""
    g = Graph(3)
    for line in text.splitlines():
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "VERTEX_SE3:QUAT":
            key = int(tok[1])
            x, y, z, qx, qy, qz, qw = map(float, tok[2:9])
            g.insert(key, pose3(rot3_quaternion(qw, qx, qy, qz, normalize=True), (x, y, z)))
        elif tok[0] == "EDGE_SE3:QUAT":
            k1, k2 = int(tok[1]), int(tok[2])
            x, y, z, qx, qy, qz, qw = map(float, tok[3:10])
            info_g2o = _upper21_to_matrix(list(map(float, tok[10:31])))
            info = info_g2o[np.ix_(_G2O_TR_SWAP, _G2O_TR_SWAP)]
            g.add_between(k1, k2, pose3(rot3_quaternion(qw, qx, qy, qz, normalize=True), (x, y, z)),
                          gaussian_information(info))
    return g


def parse_g2o_2d(text: str) -> Graph:
    """VERTEX_SE2 / EDGE_SE2 (information upper triangle in (x, y, theta))."""
    g = Graph(2)
    for line in text.splitlines():
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "VERTEX_SE2":
            g.insert(int(tok[1]), pose2(float(tok[4]), float(tok[2]), float(tok[3])))
        elif tok[0] == "EDGE_SE2":
            k1, k2 = int(tok[1]), int(tok[2])
            x, y, th = map(float, tok[3:6])
            v = list(map(float, tok[6:12]))
            info = np.array([[v[0], v[1], v[2]], [v[1], v[3], v[4]], [v[2], v[4], v[5]]])
            g.add_between(k1, k2, pose2(th, x, y), gaussian_information(info))
    return g


def write_g2o(path: str, dim: int, keys, poses, kinds, key1, key2, measured, sqrt_info) -> None:
    """Kimera-RPGO writeG2o (src/Logger.cpp:64-164): vertices, then the
    between factors with their information R^T R (Pose3: block-swapped back
    to g2o's [t; R] order)."""
    lines = []
    for k, p in zip(keys, poses):
        if dim == 3:
            R = np.asarray(p[:9]).reshape(3, 3)
            w, x, y, z = rot3_to_quaternion(R)
            lines.append(f"VERTEX_SE3:QUAT {int(k)} {p[9]:g} {p[10]:g} {p[11]:g} {x:g} {y:g} {z:g} {w:g}")
        else:
            lines.append(f"VERTEX_SE2 {int(k)} {p[2]:g} {p[3]:g} {math.atan2(p[1], p[0]):g}")
    for kind, a, b, m, R in zip(kinds, key1, key2, measured, sqrt_info):
        if kind != BETWEEN:
            continue
        R = np.asarray(R)
        info = R.T @ R
        if dim == 3:
            Rm = np.asarray(m[:9]).reshape(3, 3)
            w, x, y, z = rot3_to_quaternion(Rm)
            # diagonal blocks swapped, off-diagonal blocks copied in place
            # (src/Logger.cpp:148-152)
            ig = np.empty((6, 6))
            ig[:3, :3] = info[3:, 3:]
            ig[3:, 3:] = info[:3, :3]
            ig[:3, 3:] = info[:3, 3:]
            ig[3:, :3] = info[3:, :3]
            tri = " ".join(f"{ig[i, j]:g}" for i in range(6) for j in range(i, 6))
            lines.append(f"EDGE_SE3:QUAT {int(a)} {int(b)} {m[9]:g} {m[10]:g} {m[11]:g} {x:g} {y:g} {z:g} {w:g} {tri}")
        else:
            tri = " ".join(f"{info[i, j]:g}" for i in range(3) for j in range(i, 3))
            lines.append(f"EDGE_SE2 {int(a)} {int(b)} {m[2]:g} {m[3]:g} {math.atan2(m[1], m[0]):g} {tri}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def graph_from_g2o_arrays(vertex_keys, vertex_vals, edge_keys, edge_vals) -> Graph:
    """Same graph as parse_g2o_3d, from the numbers of VERTEX_SE3:QUAT
    (x y z qx qy qz qw) and EDGE_SE3:QUAT (x y z qx qy qz qw + 21 information
    values) lines."""
    g = Graph(3)
    for k, v in zip(vertex_keys, vertex_vals):
        x, y, z, qx, qy, qz, qw = v[:7]
        g.insert(int(k), pose3(rot3_quaternion(qw, qx, qy, qz, normalize=True), (x, y, z)))
    for (k1, k2), v in zip(edge_keys, edge_vals):
        x, y, z, qx, qy, qz, qw = v[:7]
        info_g2o = _upper21_to_matrix(v[7:28])
        info = info_g2o[np.ix_(_G2O_TR_SWAP, _G2O_TR_SWAP)]
        g.add_between(int(k1), int(k2), pose3(rot3_quaternion(qw, qx, qy, qz, normalize=True), (x, y, z)),
                      gaussian_information(info))
    return g

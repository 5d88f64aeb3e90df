"""Closure-network oracle of the GNC warm start — TEST INFRASTRUCTURE ONLY.

The warm start has no counterpart in the reference; this is the FP64 numpy
statement of what the library's kernels compute, used by tests/ to check
them: the BF16 rounding of the weights (round to nearest even on the FP32
bit pattern), the forward pass, the mean binary cross-entropy and its
gradient by back-propagation, one Adam step, and the per-closure features
(from the graph arrays and the oracle's Logmap).
"""
from __future__ import annotations

import numpy as np

FEAT, HID = 16, 64
OFF_MU, OFF_ISD, OFF_W1 = 0, 16, 32
OFF_B1 = OFF_W1 + HID * FEAT
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID
N_PARAMS = OFF_B3 + 1


def bf16_round(x: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 (round to nearest, ties to even) -> FP32, finite inputs."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray, bf16: bool = True):
    """bf16=False keeps the weights unrounded (FP64), for finite-difference
    checks of the gradient formulas."""
    if bf16:
        p = np.asarray(params, dtype=np.float32)
        rnd = lambda w: bf16_round(w).astype(np.float64)
    else:
        p = np.asarray(params, dtype=np.float64)
        rnd = lambda w: w.astype(np.float64)
    mu = p[OFF_MU:OFF_MU + FEAT].astype(np.float64)
    isd = p[OFF_ISD:OFF_ISD + FEAT].astype(np.float64)
    W1 = rnd(p[OFF_W1:OFF_B1]).reshape(HID, FEAT)
    b1 = p[OFF_B1:OFF_W2].astype(np.float64)
    W2 = rnd(p[OFF_W2:OFF_B2]).reshape(HID, HID)
    b2 = p[OFF_B2:OFF_W3].astype(np.float64)
    W3 = rnd(p[OFF_W3:OFF_B3])
    b3 = float(p[OFF_B3])
    return mu, isd, W1, b1, W2, b2, W3, b3


def forward(params, X, bf16: bool = True):
    """Probabilities and the intermediate activations (FP64)."""
    mu, isd, W1, b1, W2, b2, W3, b3 = unpack(params, bf16)
    xn = (np.asarray(X, dtype=np.float64) - mu) * isd
    h1 = np.maximum(xn @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    logit = h2 @ W3 + b3
    return 1.0 / (1.0 + np.exp(-logit)), (xn, h1, h2, logit)


def loss_and_grad(params, X, y, bf16: bool = True):
    """Mean BCE-with-logits loss and its gradient (N_PARAMS entries; the
    normalisation slots are zero). Gradients flow to the FP32 master weights
    through the BF16 rounding unchanged (straight through)."""
    mu, isd, W1, b1, W2, b2, W3, b3 = unpack(params, bf16)
    p, (xn, h1, h2, logit) = forward(params, X, bf16)
    y = np.asarray(y, dtype=np.float64)
    n = len(y)
    loss = np.mean(np.maximum(logit, 0.0) - logit * y + np.log1p(np.exp(-np.abs(logit))))
    dl = (p - y) / n
    dh2 = np.where(h2 > 0, dl[:, None] * W3[None, :], 0.0)
    dh1 = np.where(h1 > 0, dh2 @ W2, 0.0)
    g = np.zeros(N_PARAMS)
    g[OFF_W1:OFF_B1] = (dh1.T @ xn).reshape(-1)
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    g[OFF_W2:OFF_B2] = (dh2.T @ h1).reshape(-1)
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    g[OFF_W3:OFF_B3] = dl @ h2
    g[OFF_B3] = dl.sum()
    return loss, g


def adam_step(params, m, v, grad, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    p, m, v = params.astype(np.float64).copy(), m.astype(np.float64).copy(), v.astype(np.float64).copy()
    s = slice(OFF_W1, N_PARAMS)
    m[s] = b1 * m[s] + (1 - b1) * grad[s]
    v[s] = b2 * v[s] + (1 - b2) * grad[s] ** 2
    p[s] -= lr * (m[s] / (1 - b1 ** step)) / (np.sqrt(v[s] / (1 - b2 ** step)) + eps)
    return p, m, v


def closure_features(dim, x0_by_key, factors, n_known, pcm_stats=None):
    """Features of factors[n_known:] (kind, key1, key2, measured, sqrt_info)
    at the initial values, in the library's layout."""
    from . import rpgo_oracle as O

    kind, k1, k2, meas, sqrt_info = factors
    d = 6 if dim == 3 else 3
    st = 12 if dim == 3 else 4
    out = []
    kmask = (1 << 56) - 1
    for q, f in enumerate(range(n_known, len(kind))):
        row = np.zeros(FEAT)
        if kind[f] != 0:
            out.append(row)
            continue
        a, b = int(k1[f]), int(k2[f])
        Xi, Xj, Z = x0_by_key[a], x0_by_key[b], meas[f]
        if dim == 3:
            Ti, Tj, Tz = _m3(Xi), _m3(Xj), _m3(Z)
        else:
            Ti, Tj, Tz = _m2(Xi), _m2(Xj), _m2(Z)
        rel = np.linalg.inv(Tz) @ (np.linalg.inv(Ti) @ Tj)
        e = O.logmap(dim, _p(rel, dim))
        ez = O.logmap(dim, np.asarray(Z, dtype=np.float64))
        r = np.asarray(sqrt_info[f]).reshape(d, d) @ e
        c = float(r @ r)
        row[:d] = np.log1p(np.abs(r))
        if dim == 3:
            rot, tr, zrot, ztr = np.linalg.norm(e[:3]), np.linalg.norm(e[3:]), np.linalg.norm(ez[:3]), \
                np.linalg.norm(Z[9:12])
        else:
            rot, tr, zrot, ztr = abs(e[2]), np.linalg.norm(e[:2]), abs(ez[2]), np.linalg.norm(Z[2:4])
        gap = abs((a & kmask) - (b & kmask)) if (a >> 56) == (b >> 56) else 0
        row[6] = np.log1p(c)
        row[7] = rot
        row[8] = np.log1p(tr)
        row[9] = np.log1p(gap)
        row[10] = np.log1p(c / max(1.0, gap))
        if pcm_stats is not None:
            row[11:14] = pcm_stats[q]
        row[14] = np.log1p(ztr)
        row[15] = zrot
        out.append(row)
    return np.array(out).reshape(-1, FEAT)


def _m3(p):
    T = np.eye(4)
    T[:3, :3] = np.asarray(p[:9]).reshape(3, 3)
    T[:3, 3] = p[9:12]
    return T


def _m2(p):
    c, s, x, y = p
    return np.array([[c, -s, x], [s, c, y], [0, 0, 1.0]])


def _p(T, dim):
    if dim == 3:
        return np.concatenate([T[:3, :3].reshape(9), T[:3, 3]])
    return np.array([T[0, 0], T[1, 0], T[0, 2], T[1, 2]])


def pcm_stats(adj_words: np.ndarray, n: int, consistent) -> np.ndarray:
    """Degree ratio, log1p(degree) and clique support of each entry of the
    consistent list (the library's closure_stats)."""
    bits = np.unpackbits(adj_words.view(np.uint8), bitorder="little").reshape(n, -1)[:, :n].astype(bool)
    members = np.zeros(n, dtype=bool)
    members[list(consistent)] = True
    out = []
    for i in consistent:
        deg = int(bits[i].sum())
        sup = int((bits[i] & members).sum())
        out.append([deg / max(1, n - 1), np.log1p(deg), sup / max(1, int(members.sum()) - 1)])
    return np.array(out, dtype=np.float64).reshape(-1, 3)

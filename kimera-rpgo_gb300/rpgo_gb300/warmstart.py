"""Learned GNC warm start: data collection, training and the model file.

The closure network (16 features -> 64 -> 64 -> 1, BF16 weights, FP32
accumulation) predicts, per loop closure, whether plain GNC keeps it. Its
labels are what plain GNC produces: a solver in RECORD mode runs the plain
schedule and records every closure's features; the final GNC weights are the
labels. Training runs on the GPU through the library's own kernels
(rpgo_mlp_train_step_dev: forward, back-propagation, Adam); torch only
provides the device buffers and the batch gather.

The trained parameters ship as warmstart_model.npy next to this file; a
solver uses them with params.setGncWarmStart(WARM_ON) after
RobustSolver.set_warm_start_model(load_model()).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import capi
from .params import WARM_RECORD

MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "warmstart_model.npy")
FEAT, HID = capi.MLP_FEATURES, 64
OFF_W1 = 32
OFF_B1 = OFF_W1 + HID * FEAT
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID


def collect(graphs, params):
    """Features and plain-GNC labels of every closure the GNC solve of each
    graph sees. `params` is a RobustSolverParams with GNC on; it is copied
    with the warm mode set to RECORD (plain schedule)."""
    import copy

    p = copy.copy(params)
    p.gnc_warm_start = WARM_RECORD
    X, Y = [], []
    for g in graphs:
        s = capi.RobustSolver(p)
        if s.update(g) != 0:
            continue
        f = s.closure_features()
        w = s.gnc_weights()
        if len(f) == 0:
            continue
        X.append(f)
        Y.append((w[len(w) - len(f):] > 0.5).astype(np.float32))
    if not X:
        return np.zeros((0, FEAT), np.float32), np.zeros(0, np.float32)
    return np.concatenate(X).astype(np.float32), np.concatenate(Y)


def init_params(features: np.ndarray, seed: int = 0) -> np.ndarray:
    """Normalisation from the data (mean, 1/std), He-initialised weights."""
    rng = np.random.default_rng(seed)
    p = np.zeros(capi.MLP_PARAMS, dtype=np.float32)
    mu = features.mean(0) if len(features) else np.zeros(FEAT)
    sd = features.std(0) if len(features) else np.ones(FEAT)
    p[0:FEAT] = mu
    p[FEAT:2 * FEAT] = 1.0 / np.maximum(sd, 1e-3)
    p[OFF_W1:OFF_B1] = rng.normal(0, np.sqrt(2.0 / FEAT), HID * FEAT)
    p[OFF_W2:OFF_B2] = rng.normal(0, np.sqrt(2.0 / HID), HID * HID)
    p[OFF_W3:OFF_B3] = rng.normal(0, np.sqrt(1.0 / HID), HID)
    return p


def train(features: np.ndarray, labels: np.ndarray, epochs: int = 20, batch: int = 8192, lr: float = 2e-3,
          seed: int = 0, log=None) -> np.ndarray:
    """Adam on the mean binary cross-entropy, minibatches of `batch`
    closures, on the GPU (library kernels). Returns the FP32 parameters."""
    import torch

    dev = torch.device("cuda:0")
    lib = capi.load()
    params = torch.from_numpy(init_params(features, seed)).to(dev)
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    grad = torch.zeros_like(params)
    X = torch.from_numpy(np.ascontiguousarray(features, dtype=np.float32)).to(dev)
    Y = torch.from_numpy(np.ascontiguousarray(labels, dtype=np.float32)).to(dev)
    n = X.shape[0]
    gen = torch.Generator(device="cpu").manual_seed(seed)
    stream = torch.cuda.current_stream(dev).cuda_stream
    step = 0
    loss = C.c_double(0.0)
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen).to(dev)
        total, count = 0.0, 0
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            xb = X.index_select(0, idx).contiguous()
            yb = Y.index_select(0, idx).contiguous()
            step += 1
            rc = lib.rpgo_mlp_train_step_dev(params.data_ptr(), m.data_ptr(), v.data_ptr(), step, float(lr),
                                             int(xb.shape[0]), xb.data_ptr(), yb.data_ptr(), grad.data_ptr(),
                                             C.byref(loss), C.c_void_p(stream))
            if rc:
                raise capi.RpgoError(f"rpgo_mlp_train_step_dev: {rc}")
            total += loss.value * xb.shape[0]
            count += xb.shape[0]
        if log:
            log(f"epoch {ep}: loss {total / max(count, 1):.5f}")
    torch.cuda.synchronize()
    return params.cpu().numpy()


def predict(params: np.ndarray, features: np.ndarray) -> np.ndarray:
    """Inlier probabilities from the library's forward kernel."""
    import torch

    dev = torch.device("cuda:0")
    P = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).to(dev)
    X = torch.from_numpy(np.ascontiguousarray(features, dtype=np.float32)).to(dev)
    out = torch.zeros(X.shape[0], dtype=torch.float32, device=dev)
    rc = capi.load().rpgo_mlp_forward_dev(P.data_ptr(), int(X.shape[0]), X.data_ptr(), out.data_ptr(),
                                          C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if rc:
        raise capi.RpgoError(f"rpgo_mlp_forward_dev: {rc}")
    return out.cpu().numpy()


def save_model(params: np.ndarray, path: str = MODEL_PATH) -> None:
    np.save(path, np.asarray(params, dtype=np.float32))


def load_model(path: str = MODEL_PATH) -> np.ndarray:
    p = np.load(path).astype(np.float32)
    if p.size != capi.MLP_PARAMS:
        raise ValueError(f"{path}: {p.size} parameters, expected {capi.MLP_PARAMS}")
    return p

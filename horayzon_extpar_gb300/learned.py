"""Learned warm start: training data, training loop and evaluation.

The MLP (32 -> 64 -> 64 -> 1, ReLU, BF16 weights, FP32 accumulation) maps 32
terrain features of a (cell, azimuth) -- elevation angles of the height field
at 8 distances x 4 azimuth offsets, seen from the ray origin -- to the
horizon in units of 8 degrees. The search starts each azimuth's bracket at
the proposal and refines it exactly as without the MLP.

Training data come from the plain method itself on other terrain seeds: the
device entry point returns the features and the unclipped horizon lattice
index of every (cell, azimuth) (hz_options.features / raw_index); the
targets are that index clipped below at -4 deg. Training
runs on the GPU with the library's own forward, backward and Adam kernels
(hz_mlp_train_step).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib
from .horizon_svf import horizon_svf_comp_device

N_IN = 32
N_HID = 64
N_PARAMS = N_IN * N_HID + N_HID + N_HID * N_HID + N_HID + N_HID + 1  # 6337
TARGET_MIN_J = -16  # -4 deg in quarter degrees


def save_params(path: str, params) -> None:
    """Writes trained parameters (FP32, packed as hz_mlp_train_step uses them;
    the kernels round the weights to BF16 when they load them)."""
    p = np.ascontiguousarray(params, dtype=np.float32).ravel()
    if p.size != N_PARAMS:
        raise ValueError("expected %d parameters, got %d" % (N_PARAMS, p.size))
    np.save(path, p)


def load_params(path: str) -> np.ndarray:
    p = np.load(path).astype(np.float32).ravel()
    if p.size != N_PARAMS:
        raise ValueError("expected %d parameters, got %d" % (N_PARAMS, p.size))
    return p


def num_params() -> int:
    return int(_lib.load().hz_mlp_num_params())


def init_params(seed: int = 0) -> np.ndarray:
    """He-initialised packed parameters (FP32)."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / N_IN), (N_IN, N_HID))
    W2 = rng.normal(0, np.sqrt(2.0 / N_HID), (N_HID, N_HID))
    W3 = rng.normal(0, np.sqrt(1.0 / N_HID), N_HID)
    p = np.concatenate([W1.ravel(), np.zeros(N_HID), W2.ravel(), np.zeros(N_HID), W3, [0.0]])
    assert p.size == num_params()
    return p.astype(np.float32)


def training_samples(domain, args, max_samples: int | None = None, seed: int = 0,
                     device: int = 0):
    """(features [n, 32], targets [n]) as CUDA tensors from the plain search."""
    import torch
    dev = torch.device("cuda", device)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in domain.inputs()]
    L = int(args[0]) * int(args[4])
    raw = torch.empty((L, domain.ncell), dtype=torch.int16, device=dev)
    feats = torch.empty((L, domain.ncell, N_IN), dtype=torch.float32, device=dev)
    horizon_svf_comp_device(*t, *args, raw_index=raw, features=feats)
    X = feats.reshape(-1, N_IN)
    # Horizons below -4 deg are clipped: the search reaches them by walking
    # down from any start near 0 deg, and the few -85 deg "void" directions at
    # the domain border would otherwise dominate the squared error.
    Y = raw.reshape(-1).to(torch.float32).clamp_(min=TARGET_MIN_J) / 32.0
    if max_samples is not None and X.shape[0] > max_samples:
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        idx = torch.randperm(X.shape[0], generator=g, device=dev)[:max_samples]
        X, Y = X[idx], Y[idx]
    return X.contiguous(), Y.contiguous()


def train_step(params, m, v, X, T, step, lr, loss, grads, stream=None):
    """One hz_mlp_train_step on CUDA tensors; returns the loss (float)."""
    import torch
    s = stream or torch.cuda.current_stream(X.device)
    rc = _lib.load().hz_mlp_train_step(params.data_ptr(), m.data_ptr(), v.data_ptr(),
                                       X.data_ptr(), T.data_ptr(), int(X.shape[0]), int(step),
                                       float(lr), loss.data_ptr(), grads.data_ptr(),
                                       C.c_void_p(s.cuda_stream))
    _lib.check(rc)
    return float(loss.item())


def gradients(params, X, T):
    """Loss and gradient (no update) for a batch, as numpy arrays."""
    import torch
    dev = X.device
    p = torch.as_tensor(params, dtype=torch.float32, device=dev).contiguous()
    grads = torch.empty(num_params(), dtype=torch.float32, device=dev)
    loss = torch.empty(1, dtype=torch.float32, device=dev)
    train_step(p, p, p, X, T, 1, 0.0, loss, grads)
    return float(loss.item()), grads.cpu().numpy()


def forward(params, X):
    import torch
    dev = X.device
    p = torch.as_tensor(params, dtype=torch.float32, device=dev).contiguous()
    Y = torch.empty(X.shape[0], dtype=torch.float32, device=dev)
    rc = _lib.load().hz_mlp_forward(p.data_ptr(), X.data_ptr(), int(X.shape[0]), Y.data_ptr(),
                                    C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    _lib.check(rc)
    return Y


def train(X, T, steps: int = 2000, batch: int = 32768, lr: float = 2e-3, seed: int = 0,
          params: np.ndarray | None = None, log_every: int = 0):
    """Adam on random mini-batches; returns (params as numpy FP32, loss history)."""
    import torch
    dev = X.device
    p = torch.as_tensor(init_params(seed) if params is None else params, dtype=torch.float32,
                        device=dev).contiguous()
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    grads = torch.empty_like(p)
    loss = torch.empty(1, dtype=torch.float32, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    n = X.shape[0]
    hist = []
    t0 = time.perf_counter()
    for step in range(1, steps + 1):
        idx = torch.randint(0, n, (min(batch, n),), generator=g, device=dev)
        lr_t = lr * 0.5 * (1.0 + np.cos(np.pi * (step - 1) / steps))  # cosine decay
        val = train_step(p, m, v, X[idx].contiguous(), T[idx].contiguous(), step, lr_t, loss,
                         grads)
        if log_every and step % log_every == 0:
            hist.append((step, val, time.perf_counter() - t0))
    return p.cpu().numpy(), hist

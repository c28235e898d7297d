"""TEST INFRASTRUCTURE ONLY: numpy restatement of the row-marking MLP
(16 -> 64 -> 64 -> 1, ReLU) with the device's BF16 rounding points, used to
check the CUDA forward and gradient kernels. Not part of the product path.

Parameter vector layout (FP32): W1[64][16], b1[64], W2[64][64], b2[64], w3[64], b3.

With bf16=True the forward rounds exactly where the device does (inputs and
weights to BF16, relu(a1) to BF16 before layer 2, bf16(da2) for the product
with W2 in the backward); with bf16=False everything is FP64, which the
finite-difference check uses to validate the gradient formulas themselves.
"""
from __future__ import annotations

import numpy as np

IN, H = 16, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
N_PARAMS = OFF_B3 + 1


def bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float32 values."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def _r(x, on):
    return bf16(x).astype(np.float64) if on else np.asarray(x, np.float64)


def forward(p, x, bf16_round=True):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = _r(x, bf16_round)
    a1 = X @ _r(W1, bf16_round).T + b1
    h1 = _r(np.maximum(a1, 0.0), bf16_round)
    a2 = h1 @ _r(W2, bf16_round).T + b2
    z = np.maximum(a2, 0.0) @ _r(w3, bf16_round) + b3
    return z, (X, a1, h1, a2)


def loss_and_grad(p, x, y, w, bf16_round=True):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    z, (X, a1, h1, a2) = forward(p, x, bf16_round)
    y = np.asarray(y, np.float64)
    w = np.asarray(w, np.float64)
    ws = w.sum()
    loss = float(np.sum(w * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))) / ws)
    pz = 1.0 / (1.0 + np.exp(-z))
    dz = w * (pz - y) / ws
    w3r = _r(w3, bf16_round)
    g = np.zeros(N_PARAMS)
    g[OFF_W3:OFF_B3] = dz @ np.maximum(a2, 0.0)
    g[OFF_B3] = dz.sum()
    da2 = dz[:, None] * w3r[None, :] * (a2 > 0)
    g[OFF_W2:OFF_B2] = (da2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = da2.sum(0)
    dh1 = _r(da2, bf16_round) @ _r(W2, bf16_round)
    da1 = dh1 * (a1 > 0)
    g[OFF_W1:OFF_B1] = (da1.T @ X).ravel()
    g[OFF_B1:OFF_W2] = da1.sum(0)
    return loss, g


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    p[OFF_W1:OFF_B1] = rng.uniform(-1, 1, H * IN) * np.sqrt(6 / IN)
    p[OFF_W2:OFF_B2] = rng.uniform(-1, 1, H * H) * np.sqrt(6 / H)
    p[OFF_W3:OFF_B3] = rng.uniform(-1, 1, H) * np.sqrt(6 / H)
    return p

"""CPU oracle of the cost-model MLP (test infrastructure only: the product path never imports it).

Restates, in numpy, what the GPU kernels of t-fsm_gb300/csrc/costmodel/mlp.cu compute: a 32-64-64-1
ReLU network, its mean-squared-error gradient and the parameter layout
  W1[32][64], b1[64], W2[64][64], b2[64], W3[64], b3        (6337 FP32 values)
with the kernels' BF16 rounding points (round to nearest even): X, W1, W2, W3, H1 = relu(Z1), dZ2
and dZ1 are BF16; all sums are FP32 on the GPU and float64 here.  `rounding=False` drops the BF16
rounding, which makes the gradient checkable against finite differences.

This model has no counterpart in the reference (T-FSM has no learned component); the oracle pins
the GPU kernels' arithmetic, not a reference behaviour.
"""
from __future__ import annotations

import numpy as np

IN, H = 32, 64
N_PARAMS = IN * H + H + H * H + H + H + 1


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to BF16 (nearest, ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray):
    p = np.asarray(p, dtype=np.float32)
    assert p.shape == (N_PARAMS,)
    o = 0
    w1 = p[o:o + IN * H].reshape(IN, H); o += IN * H
    b1 = p[o:o + H]; o += H
    w2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return w1, b1, w2, b2, w3, b3


def forward(p, x, rounding: bool = True):
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float32))
    w1, b1, w2, b2, w3, b3 = unpack(p)
    f = np.float64
    xb = r(x).astype(f)
    z1 = xb @ r(w1).astype(f) + b1.astype(f)
    h1b = r(np.maximum(z1, 0).astype(np.float32)).astype(f)
    z2 = h1b @ r(w2).astype(f) + b2.astype(f)
    h2 = np.maximum(z2, 0)
    y = h2 @ r(w3).astype(f) + f(b3)
    return y, (xb, z1, h1b, z2, h2)


def gradients(p, x, t, rounding: bool = True):
    """Gradient of mean((y - t)^2) in the parameter layout (float64)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float32))
    w1, b1, w2, b2, w3, b3 = unpack(p)
    f = np.float64
    y, (xb, z1, h1b, z2, h2) = forward(p, x, rounding)
    n = len(x)
    dy = 2.0 * (y - np.asarray(t, dtype=f)) / n
    dw3 = h2.T @ dy
    db3 = dy.sum()
    dz2 = (dy[:, None] * r(w3).astype(f)[None, :]) * (z2 > 0)
    db2 = dz2.sum(0)
    dz2b = r(dz2.astype(np.float32)).astype(f)
    dw2 = h1b.T @ dz2b
    dh1 = dz2b @ r(w2).astype(f).T
    dz1 = dh1 * (z1 > 0)
    db1 = dz1.sum(0)
    dw1 = xb.T @ r(dz1.astype(np.float32)).astype(f)
    return np.concatenate([dw1.ravel(), db1, dw2.ravel(), db2, dw3, [db3]])


def loss(p, x, t, rounding: bool = True) -> float:
    y, _ = forward(p, x, rounding)
    return float(np.mean((y - np.asarray(t, dtype=np.float64)) ** 2))

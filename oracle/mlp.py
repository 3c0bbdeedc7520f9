"""CPU oracle of the step-size proposer MLP -- TEST INFRASTRUCTURE ONLY.

Float64 restatement of the forward pass and the gradient of the MSE loss of the MLP
16 -> 64 -> 64 -> 1 with SiLU activations, evaluated with the weights rounded to
bfloat16 exactly as the GPU kernels use them (round to nearest even).  The flat
parameter layout is W1[64][16], b1[64], W2[64][64], b2[64], W3[64], b3 (include/simgb.h).
"""
from __future__ import annotations

import numpy as np

IN, H = 16, 64
NP = H * IN + H + H * H + H + H + 1


def bf16_round(w: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(w, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def unpack(w):
    w = np.asarray(w, np.float64)
    o = 0
    W1 = w[o:o + H * IN].reshape(H, IN); o += H * IN
    b1 = w[o:o + H]; o += H
    W2 = w[o:o + H * H].reshape(H, H); o += H * H
    b2 = w[o:o + H]; o += H
    W3 = w[o:o + H]; o += H
    b3 = w[o]
    return W1, b1, W2, b2, W3, b3


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(X, w, bf16=True):
    wb = bf16_round(w) if bf16 else np.asarray(w, np.float32)
    W1, b1, W2, b2, W3, b3 = unpack(wb)
    X = np.asarray(X, np.float64)
    z1 = X @ W1.T + b1
    h1 = silu(z1)
    z2 = h1 @ W2.T + b2
    h2 = silu(z2)
    return h2 @ W3 + b3


def loss_and_grad(X, Y, w, bf16=True):
    """MSE loss (1/n) sum (o - y)^2 and its gradient w.r.t. the flat weights."""
    wb = bf16_round(w) if bf16 else np.asarray(w, np.float32)
    W1, b1, W2, b2, W3, b3 = unpack(wb)
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    n = len(Y)
    z1 = X @ W1.T + b1
    h1 = silu(z1)
    z2 = h1 @ W2.T + b2
    h2 = silu(z2)
    o = h2 @ W3 + b3
    d = o - Y
    loss = float(np.mean(d * d))
    go = 2.0 * d / n
    gW3 = h2.T @ go
    gb3 = go.sum()
    gz2 = (go[:, None] * W3[None, :]) * silu_grad(z2)
    gW2 = gz2.T @ h1
    gb2 = gz2.sum(0)
    gz1 = (gz2 @ W2) * silu_grad(z1)
    gW1 = gz1.T @ X
    gb1 = gz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g

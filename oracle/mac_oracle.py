"""CPU oracle of the learned-MAC MLP (float64 numpy).

TEST INFRASTRUCTURE ONLY: checks the GPU forward pass, loss and gradients of
gbh_mac_loss_grad / gbh_mac_predict.  It mirrors the GPU arithmetic: the
inputs, weights and hidden activations that enter a tensor-core product are
rounded to BF16 (round to nearest even); sums are exact (float64 here, FP32
on the GPU); the backward pass is straight-through for those roundings and
uses the FP32 master weights and the unrounded activations.
Parameter layout: W1[32][12], b1[32], W2[32][32], b2[32], w3[32], b3.
"""
from __future__ import annotations

import numpy as np

F, H = 12, 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * F
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAMS = OFF_B3 + 1


def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(H, F)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(H, H)
    b2 = p[OFF_B2:OFF_W3]
    w3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    return W1, b1, W2, b2, w3, b3


def forward(p, x, round_bf16=True):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    r = bf16 if round_bf16 else (lambda v: np.asarray(v, np.float64))
    xb = r(x)
    z1 = xb @ r(W1).T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = r(h1) @ r(W2).T + b2
    h2 = np.maximum(z2, 0.0)
    y = r(h2) @ r(w3) + b3
    return y, (xb, h1, h2)


def loss(p, x, t, round_bf16=True):
    y, _ = forward(p, x, round_bf16)
    e = y - np.asarray(t, np.float64)
    return float(np.mean(e * e))


def loss_grad(p, x, t, round_bf16=True):
    """Mean squared error and its gradient (GPU conventions)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    y, (xb, h1, h2) = forward(p, x, round_bf16)
    B = len(t)
    e = y - np.asarray(t, np.float64)
    loss = float(np.mean(e * e))
    dy = 2.0 * e / B
    dz2 = dy[:, None] * w3[None, :] * (h2 > 0)
    dz1 = (dz2 @ W2) * (h1 > 0)
    g = np.zeros(NPARAMS)
    g[OFF_W1:OFF_B1] = (dz1.T @ xb).reshape(-1)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).reshape(-1)
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W3:OFF_B3] = dy @ h2
    g[OFF_B3] = dy.sum()
    return loss, g

"""CPU oracle of the plan scorer (TEST INFRASTRUCTURE ONLY): the same 3-layer
MLP, loss and gradients in float64 numpy, used to check the GPU training
kernels' gradients and the BF16 inference path."""
from __future__ import annotations

import numpy as np


def unpack(p: np.ndarray, in_dim: int, hid: int):
    p = p.astype(np.float64)
    o = 0
    W1 = p[o:o + hid * in_dim].reshape(hid, in_dim); o += hid * in_dim
    b1 = p[o:o + hid]; o += hid
    W2 = p[o:o + hid * hid].reshape(hid, hid); o += hid * hid
    b2 = p[o:o + hid]; o += hid
    w3 = p[o:o + hid]; o += hid
    b3 = p[o:o + 1]
    return W1, b1, W2, b2, w3, b3


def forward(p, x, in_dim, hid, bf16=False):
    W1, b1, W2, b2, w3, b3 = unpack(p, in_dim, hid)
    x = x.astype(np.float64)
    if bf16:
        q = bf16_round
        z1 = q(x) @ q(W1).T + b1
        a1 = q(np.maximum(z1, 0))
        z2 = a1 @ q(W2).T + b2
    else:
        z1 = x @ W1.T + b1
        a1 = np.maximum(z1, 0)
        z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0)
    return a2 @ w3 + b3[0]


def loss_grad(p, x, t, in_dim, hid):
    W1, b1, W2, b2, w3, b3 = unpack(p, in_dim, hid)
    x = x.astype(np.float64)
    t = t.astype(np.float64)
    B = x.shape[0]
    z1 = x @ W1.T + b1
    a1 = np.maximum(z1, 0)
    z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0)
    y = a2 @ w3 + b3[0]
    d = y - t
    loss = 0.5 * np.mean(d * d)
    dy = d / B
    gw3 = a2.T @ dy
    gb3 = np.array([dy.sum()])
    dz2 = np.outer(dy, w3) * (z2 > 0)
    gW2 = dz2.T @ a1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (z1 > 0)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, gb3])


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even to bfloat16, returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)

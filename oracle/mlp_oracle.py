"""CPU restatement of the learned proposal network (kodama_gb300/csrc/mlp.cu):
bfloat16 rounding of weights, inputs and activations as the device does it,
float64 arithmetic otherwise.

TEST INFRASTRUCTURE ONLY: checks the device forward pass and gradients in
tests/; the product never imports it."""

from __future__ import annotations

import numpy as np

IN, H = 8, 64
W1, B1 = 0, IN * H
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + H
PARAMS = B3 + 1


def bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).copy()
    keep = ~np.isfinite(a)
    out[keep] = a[keep]
    return out


def unpack(p, rounding=True):
    p = np.asarray(p, np.float32)
    rnd = bf16 if rounding else (lambda v: v)
    w1 = rnd(p[W1:B1]).reshape(IN, H).astype(np.float64)
    w2 = rnd(p[W2:B2]).reshape(H, H).astype(np.float64)
    w3 = rnd(p[W3:B3]).astype(np.float64)
    return w1, p[B1:W2].astype(np.float64), w2, p[B2:W3].astype(np.float64), w3, float(p[B3])


def forward(p, x, rounding=True):
    """Logits and activations of rows x (n x 8)."""
    rnd = bf16 if rounding else (lambda v: np.asarray(v, np.float64))
    w1, b1, w2, b2, w3, b3 = unpack(p, rounding)
    xb = np.asarray(rnd(np.asarray(x, np.float32)), np.float64)
    h1 = np.asarray(rnd(np.maximum(xb @ w1 + b1, 0.0).astype(np.float32 if rounding else np.float64)), np.float64)
    h2 = np.asarray(rnd(np.maximum(h1 @ w2 + b2, 0.0).astype(np.float32 if rounding else np.float64)), np.float64)
    return h2 @ w3 + b3, (xb, h1, h2)


def gradient(p, x, y, rounding=True):
    """Mean binary cross-entropy and its gradient (PARAMS floats) over rows x, targets y."""
    w1, b1, w2, b2, w3, b3 = unpack(p, rounding)
    z, (xb, h1, h2) = forward(p, x, rounding)
    y = np.asarray(y, np.float64)
    n = len(y)
    pr = 1.0 / (1.0 + np.exp(-z))
    loss = float(np.mean(np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z)))))
    dz = (pr - y) / n
    g = np.zeros(PARAMS)
    g[W3:B3] = h2.T @ dz
    g[B3] = dz.sum()
    d2 = np.where(h2 > 0, dz[:, None] * w3[None, :], 0.0)
    g[W2:B2] = (h1.T @ d2).ravel()
    g[B2:W3] = d2.sum(0)
    d1 = np.where(h1 > 0, d2 @ w2.T, 0.0)
    g[W1:B1] = (xb.T @ d1).ravel()
    g[B1:W2] = d1.sum(0)
    return g, loss

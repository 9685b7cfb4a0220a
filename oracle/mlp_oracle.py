"""CPU oracle of the selector network (test infrastructure only).

numpy restatement of cross-corr_gb300/csrc/mlp.cu: a 3-layer MLP
8 -> 64 -> ReLU -> 64 -> ReLU -> 7 with parameters packed as
W1[64][8], b1[64], W2[64][64], b2[64], W3[7][64], b3[7], the masked
mean-squared error and its analytic gradient, in float64.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 8, 64, 7
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (OUT, H)), ("b3", (OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def forward(p, x):
    w = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ w["W1"].T + w["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = np.maximum(z2, 0)
    y = h2 @ w["W3"].T + w["b3"]
    return y, (x, h1, h2)


def loss_and_grad(p, x, t, m):
    """loss = sum m (y - t)^2 / sum m and d loss / d params (packed)."""
    w = unpack(p)
    y, (x, h1, h2) = forward(p, x)
    m = np.asarray(m, dtype=np.float64)
    cnt = m.sum()
    d = y - np.asarray(t, dtype=np.float64)
    loss = float((m * d * d).sum() / cnt)
    dy = 2.0 * m * d / cnt
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    dh2 = (dy @ w["W3"]) * (h2 > 0)
    g["W2"] = dh2.T @ h1
    g["b2"] = dh2.sum(0)
    dh1 = (dh2 @ w["W2"]) * (h1 > 0)
    g["W1"] = dh1.T @ x
    g["b1"] = dh1.sum(0)
    return loss, pack(g)


def init(seed=0):
    """He-normal weights, zero biases."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SIZES:
        if name.startswith("W"):
            d[name] = rng.standard_normal(shape) * np.sqrt(2.0 / shape[1])
        else:
            d[name] = np.zeros(shape)
    return pack(d).astype(np.float32)

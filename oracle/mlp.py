"""CPU reference of the occluder-selection network (test infrastructure only:
the tests and the benchmark's checks use it; the library never does).

The reference has no learned part: its frame loop draws every occluder that
passes the visibility test, nearest first (SoftwareRasterizer/Main.cpp:184-206).
The library replaces that loop's ordering with an MLP 16 -> 64 -> 64 -> 1 (ReLU)
whose two matrix layers run as bf16 tensor-core MMA with fp32 accumulation.
This module restates the network in float64 with the same rounding points:

* the input features and W1, W2 are rounded to bf16 (round to nearest even);
* layer 1's ReLU output is rounded to bf16 before layer 2 (it is layer 2's
  MMA operand); biases, layer 2's output, w3 and b3 stay fp32;
* the loss is the mean squared error of the scores against the targets, and
  the gradient is that of this forward with the bf16 roundings treated as the
  identity (the fp32 master weights receive the gradient of their bf16 copy).

Parameter vector layout (5313 float32): W1 (64 x 16, row n = weights into
hidden unit n), b1 (64), W2 (64 x 64, same), b2 (64), w3 (64), b3 (1).
"""
from __future__ import annotations

import numpy as np

FEATURES = 16
HIDDEN = 64
OFFSETS = dict(W1=0, b1=1024, W2=1088, b2=5184, w3=5248, b3=5312)
PARAMS = 5313


def bf16(x) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32 (finite inputs)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def unpack(p: np.ndarray):
    p = np.asarray(p, np.float32)
    W1 = p[0:1024].reshape(HIDDEN, FEATURES)
    b1 = p[1024:1088]
    W2 = p[1088:5184].reshape(HIDDEN, HIDDEN)
    b2 = p[5184:5248]
    w3 = p[5248:5312]
    b3 = p[5312]
    return W1, b1, W2, b2, w3, b3


def forward(p: np.ndarray, x: np.ndarray, keep: bool = False):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    xb = bf16(x).astype(np.float64)
    z1 = xb @ bf16(W1).astype(np.float64).T + b1
    h1 = np.maximum(z1, 0.0)
    h1b = bf16(h1.astype(np.float32)).astype(np.float64)
    z2 = h1b @ bf16(W2).astype(np.float64).T + b2
    h2 = np.maximum(z2, 0.0)
    s = h2 @ w3.astype(np.float64) + float(b3)
    if keep:
        return s, dict(xb=xb, z1=z1, h1b=h1b, z2=z2, h2=h2)
    return s


def gradients(p: np.ndarray, x: np.ndarray, t: np.ndarray):
    """(loss, gradient as a flat float64 vector in the parameter layout)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    s, a = forward(p, x, keep=True)
    B = len(s)
    e = s - np.asarray(t, np.float64)
    loss = float(np.mean(e * e))
    ds = 2.0 * e / B
    g = np.zeros(PARAMS)
    g[5248:5312] = a["h2"].T @ ds
    g[5312] = ds.sum()
    dz2 = np.outer(ds, w3.astype(np.float64)) * (a["z2"] > 0)
    g[1088:5184] = (dz2.T @ a["h1b"]).ravel()
    g[5184:5248] = dz2.sum(axis=0)
    dz1 = (dz2 @ bf16(W2).astype(np.float64)) * (a["z1"] > 0)
    g[0:1024] = (dz1.T @ a["xb"]).ravel()
    g[1024:1088] = dz1.sum(axis=0)
    return loss, g


def adam(p, g, m, v, step: int, lr: float, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update in float32, as the library's kernel states it."""
    p, g, m, v = (np.asarray(a, np.float32) for a in (p, g, m, v))
    m = np.float32(beta1) * m + np.float32(1 - beta1) * g
    v = np.float32(beta2) * v + np.float32(1 - beta2) * g * g
    bc1 = np.float32(1 - beta1 ** step)
    bc2 = np.float32(1 - beta2 ** step)
    p = p - np.float32(lr) * (m / bc1) / (np.sqrt(v / bc2) + np.float32(eps))
    return p, m, v


def listwise_gradients(p: np.ndarray, x: np.ndarray, t: np.ndarray, group_start: np.ndarray):
    """Listwise loss: per group, cross-entropy between the target distribution
    t and the softmax of the scores; mean over groups.  (loss, gradient)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    s, a = forward(p, x, keep=True)
    t = np.asarray(t, np.float64)
    G = len(group_start) - 1
    ds = np.zeros_like(s)
    loss = 0.0
    for g in range(G):
        lo, hi = int(group_start[g]), int(group_start[g + 1])
        if hi <= lo:
            continue
        z = s[lo:hi] - s[lo:hi].max()
        lp = z - np.log(np.exp(z).sum())
        loss += -(t[lo:hi] * lp).sum()
        ds[lo:hi] = np.exp(lp) - t[lo:hi]
    ds /= G
    loss /= G
    g = np.zeros(PARAMS)
    g[5248:5312] = a["h2"].T @ ds
    g[5312] = ds.sum()
    dz2 = np.outer(ds, w3.astype(np.float64)) * (a["z2"] > 0)
    g[1088:5184] = (dz2.T @ a["h1b"]).ravel()
    g[5184:5248] = dz2.sum(axis=0)
    dz1 = (dz2 @ bf16(W2).astype(np.float64)) * (a["z1"] > 0)
    g[0:1024] = (dz1.T @ a["xb"]).ravel()
    g[1024:1088] = dz1.sum(axis=0)
    return loss, g

"""CPU checker of the learned calibration network (TEST INFRASTRUCTURE ONLY).

The learned warm start of the perplexity calibration has no counterpart in the reference
(its bisection, src/tsne.cpp:1394-1469, is what it seeds).  This module restates, in NumPy
FP64, the network the GPU kernels train -- K -> 64 -> 64 -> 1 with ReLU, input the row's
distances divided by their mean, target (log(beta * mean distance) - mu) / sd, loss the mean
squared error -- and its gradient by back-propagation, so that the GPU's forward / backward
kernels can be checked against it.  Parameter layout (as the GPU's): W1[64][K], b1[64],
W2[64][64], b2[64], w3[64], b3.

Only tests/ may use this module.
"""
from __future__ import annotations

import numpy as np

HID = 64


def param_count(K: int) -> int:
    return HID * K + HID + HID * HID + HID + HID + 1


def unpack(p: np.ndarray, K: int):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + HID * K].reshape(HID, K); o += HID * K
    b1 = p[o:o + HID]; o += HID
    W2 = p[o:o + HID * HID].reshape(HID, HID); o += HID * HID
    b2 = p[o:o + HID]; o += HID
    w3 = p[o:o + HID]; o += HID
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def pack(W1, b1, W2, b2, w3, b3) -> np.ndarray:
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, [b3]])


def features(dist: np.ndarray):
    s = dist.mean(axis=1)
    return dist / s[:, None], s


def forward(p, dist):
    K = dist.shape[1]
    W1, b1, W2, b2, w3, b3 = unpack(p, K)
    x, s = features(dist)
    a1 = x @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    return h2 @ w3 + b3, (x, a1, h1, a2, h2, s)


def loss_grad(p, dist, beta, mu=0.0, sd=1.0):
    """Mean squared error of the standardised target and its gradient (FP64)."""
    dist = np.asarray(dist, dtype=np.float64)
    K = dist.shape[1]
    W1, b1, W2, b2, w3, b3 = unpack(p, K)
    out, (x, a1, h1, a2, h2, s) = forward(p, dist)
    t = (np.log(np.asarray(beta) * s) - mu) / sd
    err = out - t
    n = len(err)
    dout = 2.0 * err / n
    gw3 = h2.T @ dout
    gb3 = dout.sum()
    dh2 = dout[:, None] * w3[None, :] * (a2 > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(axis=0)
    dh1 = (dh2 @ W2) * (a1 > 0)
    gW1 = dh1.T @ x
    gb1 = dh1.sum(axis=0)
    return float(np.mean(err * err)), pack(gW1, gb1, gW2, gb2, gw3, gb3)


def bisection_beta(d: np.ndarray, perplexity: float, tol: float = 1e-5) -> float:
    """beta of one row by the reference's bisection rule (src/tsne.cpp:1407-1454), for
    building test pairs; non-squared distances (quirk Q1)."""
    beta, lo, hi = 1.0, -np.inf, np.inf
    logU = np.log(perplexity)
    for _ in range(200):
        e = np.exp(-beta * d)
        sP = np.finfo(float).tiny + e.sum()
        H = beta * (d * e).sum() / sP + np.log(sP)
        if abs(H - logU) < tol:
            break
        if H > logU:
            lo = beta
            beta = beta * 2 if np.isinf(hi) else (beta + hi) / 2
        else:
            hi = beta
            beta = beta / 2 if np.isinf(lo) else (beta + lo) / 2
    return beta

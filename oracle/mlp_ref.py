"""Numpy restatement of the engine's cost model (test infrastructure only).

The model is 12 -> 32 (ReLU) -> 1 with parameters W1[32][12], b1[32], w2[32], b2 stored
flat in that order, fp16 weights and fp32 arithmetic; the loss is the mean squared
error.  The tests compare the engine's hand-written forward / backward kernels with
these functions.  The model has no counterpart in the reference.
"""
from __future__ import annotations

import numpy as np

F, H = 12, 32
NPARAM = H * F + 2 * H + 1


def unpack(p: np.ndarray):
    p = np.asarray(p, dtype=np.float32)
    w1 = p[: H * F].reshape(H, F)
    b1 = p[H * F: H * F + H]
    w2 = p[H * F + H: H * F + 2 * H]
    b2 = p[H * F + 2 * H]
    return w1, b1, w2, b2


def fp16(p: np.ndarray) -> np.ndarray:
    return np.asarray(p, dtype=np.float32).astype(np.float16).astype(np.float32)


def forward(p: np.ndarray, X: np.ndarray) -> np.ndarray:
    w1, b1, w2, b2 = unpack(fp16(p))
    z = X.astype(np.float64) @ w1.T.astype(np.float64) + b1
    return (np.maximum(z, 0.0) @ w2.astype(np.float64) + b2).astype(np.float64)


def loss_grad(p: np.ndarray, X: np.ndarray, y: np.ndarray):
    w1, b1, w2, b2 = [np.asarray(a, dtype=np.float64) for a in unpack(fp16(p))]
    X = X.astype(np.float64)
    n = len(y)
    z = X @ w1.T + b1
    a = np.maximum(z, 0.0)
    yhat = a @ w2 + b2
    r = yhat - y
    loss = float(np.mean(r * r))
    dy = 2.0 * r / n
    g_b2 = dy.sum()
    g_w2 = a.T @ dy
    dz = np.outer(dy, w2) * (z > 0)
    g_b1 = dz.sum(0)
    g_w1 = dz.T @ X
    g = np.concatenate([g_w1.ravel(), g_b1, g_w2, [g_b2]])
    return loss, g

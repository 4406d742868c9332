"""Rank-predictor MLP restated in numpy (test infrastructure only).

No counterpart in the reference.  Network: 8 inputs -> 64 -> 64 -> 64 -> 2
with ReLU on the hidden layers; packed parameters W1, b1, W2, b2, W3, b3, W4,
b4 with row-major W[out][in]; loss = (1/n) sum_samples sum_outputs
(y - t)^2 / 2.  Evaluated in float64 as the reference for the device's FP32
forward and backward kernels."""
from __future__ import annotations

import numpy as np

DIMS = (8, 64, 64, 64, 2)
N_PARAMS = sum(DIMS[i + 1] * DIMS[i] + DIMS[i + 1] for i in range(4))


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    assert p.size == N_PARAMS
    Ws, bs, o = [], [], 0
    for i in range(4):
        n_out, n_in = DIMS[i + 1], DIMS[i]
        Ws.append(p[o:o + n_out * n_in].reshape(n_out, n_in))
        o += n_out * n_in
        bs.append(p[o:o + n_out])
        o += n_out
    return Ws, bs


def pack(Ws, bs):
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in zip(Ws, bs)])


def forward(p, X):
    Ws, bs = unpack(p)
    h = np.asarray(X, dtype=np.float64)
    for i in range(4):
        h = h @ Ws[i].T + bs[i]
        if i < 3:
            h = np.maximum(h, 0.0)
    return h


def loss_and_grad(p, X, T):
    Ws, bs = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    n = X.shape[0]
    acts = [X]
    h = X
    for i in range(4):
        h = h @ Ws[i].T + bs[i]
        if i < 3:
            h = np.maximum(h, 0.0)
        acts.append(h)
    r = acts[-1] - T
    loss = 0.5 * float(np.sum(r * r)) / n
    d = r / n
    gW, gb = [None] * 4, [None] * 4
    for i in range(3, -1, -1):
        gW[i] = d.T @ acts[i]
        gb[i] = d.sum(axis=0)
        if i > 0:
            d = (d @ Ws[i]) * (acts[i] > 0)
    return loss, pack(gW, gb)


def adam_step(p, m, v, g, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return p, m, v

"""Rank-predictor MLP (oracle for the hand-written CUDA forward/backward/Adam).

The network is ``nin -> H -> H -> 1`` with ReLU hidden layers and a sigmoid
output, fitted with mean-squared error to the plain ID's rank fraction k/n.
It generalises the reference's hand-fitted ``rank ~ m*log10(n) - b`` table
(HSS2D/predict_rank.m:5-23).  Parameters are one flat float32 vector laid out
as [W1 (H x nin, row-major), b1 (H), W2 (H x H), b2 (H), W3 (1 x H), b3 (1)],
the same layout the GPU library uses.
"""
from __future__ import annotations

import numpy as np


def nparams(nin: int, H: int) -> int:
    return H * nin + H + H * H + H + H + 1


def unpack(p, nin, H):
    o = 0
    W1 = p[o:o + H * nin].reshape(H, nin); o += H * nin
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H].reshape(1, H); o += H
    b3 = p[o:o + 1]
    return W1, b1, W2, b2, W3, b3


def forward(p, X, nin, H):
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, np.float64), nin, H)
    X = np.asarray(X, np.float64)
    z1 = X @ W1.T + b1
    a1 = np.maximum(z1, 0.0)
    z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0.0)
    z3 = a2 @ W3.T + b3
    y = 1.0 / (1.0 + np.exp(-z3[:, 0]))
    return y, (X, z1, a1, z2, a2, y)


def loss_and_grad(p, X, t, nin, H):
    """Mean squared error 0.5*mean((y - t)^2) and its gradient (flat, same layout)."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, np.float64), nin, H)
    y, (X, z1, a1, z2, a2, _) = forward(p, X, nin, H)
    B = X.shape[0]
    t = np.asarray(t, np.float64)
    loss = 0.5 * np.mean((y - t) ** 2)
    dz3 = ((y - t) * y * (1.0 - y) / B)[:, None]
    gW3 = dz3.T @ a2
    gb3 = dz3.sum(axis=0)
    da2 = dz3 @ W3
    dz2 = da2 * (z2 > 0)
    gW2 = dz2.T @ a1
    gb2 = dz2.sum(axis=0)
    da1 = dz2 @ W2
    dz1 = da1 * (z1 > 0)
    gW1 = dz1.T @ X
    gb1 = dz1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def init_params(nin, H, seed=0):
    """He-uniform initialisation drawn from the shared counter RNG (oracle.rng)."""
    from . import rng
    n = nparams(nin, H)
    u = rng.uniform(seed, 0x4D4C50, n) * 2.0 - 1.0
    p = np.zeros(n)
    o = 0
    for fan_in, cnt, bias in ((nin, H * nin, H), (H, H * H, H), (H, H, 1)):
        lim = np.sqrt(6.0 / fan_in)
        p[o:o + cnt] = u[o:o + cnt] * lim
        o += cnt
        p[o:o + bias] = 0.0
        o += bias
    return p.astype(np.float32)


def adam_step(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v

"""Float64 reference of the cost MLP (16 -> 64 -> 64 -> 1, ReLU) and of the
gradient of mean((y - t)^2) - TEST INFRASTRUCTURE ONLY: the tests compare the
library's gs3d_mlp_forward / gs3d_mlp_backward / gs3d_mlp_infer kernels with it.
The layout of the parameter vector is the library's:
W1[64][16] | b1[64] | W2[64][64] | b2[64] | w3[64] | b3."""
from __future__ import annotations

import numpy as np

F, H = 16, 64


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, x):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, np.float64)
    h1 = np.maximum(0.0, x @ W1.T + b1)
    h2 = np.maximum(0.0, h1 @ W2.T + b2)
    return h2 @ w3 + b3, h1, h2


def grad(p, x, t):
    """d mean((y - t)^2) / d p in the library's layout."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, np.float64)
    y, h1, h2 = forward(p, x)
    n = len(x)
    dy = 2.0 * (y - np.asarray(t, np.float64)) / n
    dh2 = np.outer(dy, w3) * (h2 > 0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    return np.concatenate([(dh1.T @ x).ravel(), dh1.sum(0), (dh2.T @ h1).ravel(), dh2.sum(0),
                           h2.T @ dy, [dy.sum()]])

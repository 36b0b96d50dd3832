"""FP64 reference of the LM damping-controller MLP (test infrastructure).

ORACLE — only tests and the bench's checks use it.  The network is
16 -> 64 -> 64 -> 2 with exact GELU, x -> 0.5 x (1 + erf(x / sqrt 2)), between
the layers and a linear head.  Parameters are one flat FP32 vector in the order
W1 [64x16] (row-major, out x in), b1 [64], W2 [64x64], b2 [64], W3 [2x64], b3 [2].
Loss per sample: (out0 - t0)^2 + BCE-with-logits(out1, t1), averaged over the
batch.  No counterpart in the reference: S-PGO has no learned component.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

D_IN, D_H, D_OUT = 16, 64, 2
SHAPES = [(D_H, D_IN), (D_H,), (D_H, D_H), (D_H,), (D_OUT, D_H), (D_OUT,)]
N_PARAMS = sum(int(np.prod(s)) for s in SHAPES)


def unpack(theta):
    theta = np.asarray(theta, dtype=np.float64)
    out, o = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(theta[o:o + n].reshape(s))
        o += n
    return out


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward(theta, X):
    W1, b1, W2, b2, W3, b3 = unpack(theta)
    X = np.asarray(X, dtype=np.float64)
    z1 = X @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    out = h2 @ W3.T + b3
    return out, (X, z1, h1, z2, h2)


def loss_and_grad(theta, X, T):
    """Mean loss and its gradient with respect to theta (flat, FP64)."""
    W1, b1, W2, b2, W3, b3 = unpack(theta)
    out, (X, z1, h1, z2, h2) = forward(theta, X)
    T = np.asarray(T, dtype=np.float64)
    n = X.shape[0]
    d0 = out[:, 0] - T[:, 0]
    s = 1.0 / (1.0 + np.exp(-out[:, 1]))
    loss = np.mean(d0 ** 2 + np.logaddexp(0.0, out[:, 1]) - T[:, 1] * out[:, 1])
    dout = np.stack([2.0 * d0, s - T[:, 1]], 1) / n
    gW3 = dout.T @ h2
    gb3 = dout.sum(0)
    dz2 = (dout @ W3) * gelu_grad(z2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    gW1 = dz1.T @ X
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return float(loss), g


def init(seed=0):
    rng = np.random.default_rng(seed)
    parts = []
    for s in SHAPES:
        if len(s) == 2:
            parts.append(rng.normal(0.0, np.sqrt(2.0 / s[1]), s).ravel())
        else:
            parts.append(np.zeros(s))
    return np.concatenate(parts).astype(np.float32)

"""numpy restatement of the warm-start network: forward pass, loss and
gradients, in float64.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA forward/backward kernels
of geostatsprocesses.jl_gb300/csrc/learned.cu (same parameter layout).

Network, per system with n neighbours and features f_i (F = 8):
    h_i = relu(W1 f_i + b1)          H = 32
    g   = mean_i h_i
    q_i = relu(W2a h_i + W2b g + b2)
    y_i = w3 . q_i + b3
Loss per system: mean_i (y_i - t_i)^2; the batch loss is the sum over systems.
"""
from __future__ import annotations

import numpy as np

F, H = 8, 32
W1, B1 = 0, H * F
W2A = B1 + H
W2B = W2A + H * H
B2 = W2B + H * H
W3 = B2 + H
B3 = W3 + H
NPARAMS = B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[W1:B1].reshape(H, F), p[B1:W2A], p[W2A:W2B].reshape(H, H), p[W2B:B2].reshape(H, H),
            p[B2:W3], p[W3:B3], p[B3])


def forward(p, f, n):
    """y (n,) for one system's features f (n, F)."""
    w1, b1, w2a, w2b, b2, w3, b3 = unpack(p)
    f = np.asarray(f[:n], dtype=np.float64)
    h = np.maximum(f @ w1.T + b1, 0.0)
    g = h.mean(axis=0)
    q = np.maximum(h @ w2a.T + (w2b @ g + b2), 0.0)
    return q @ w3 + b3


def loss_and_grad(p, feat, count, target):
    """Summed per-system mean squared error and its gradient (NPARAMS,)."""
    w1, b1, w2a, w2b, b2, w3, b3 = unpack(p)
    grad = np.zeros(NPARAMS)
    gw1, gb1 = grad[W1:B1].reshape(H, F), grad[B1:W2A]
    gw2a, gw2b = grad[W2A:W2B].reshape(H, H), grad[W2B:B2].reshape(H, H)
    gb2, gw3 = grad[B2:W3], grad[W3:B3]
    total = 0.0
    for s in range(len(count)):
        n = int(count[s])
        if n <= 0:
            continue
        f = np.asarray(feat[s, :n], dtype=np.float64)
        t = np.asarray(target[s, :n], dtype=np.float64)
        z1 = f @ w1.T + b1
        h = np.maximum(z1, 0.0)
        g = h.mean(axis=0)
        z2 = h @ w2a.T + (w2b @ g + b2)
        q = np.maximum(z2, 0.0)
        y = q @ w3 + b3
        e = y - t
        total += float(e @ e) / n
        dy = 2.0 * e / n
        gw3 += dy @ q
        grad[B3] += dy.sum()
        dz2 = (dy[:, None] * w3[None, :]) * (z2 > 0)
        gw2a += dz2.T @ h
        sz = dz2.sum(axis=0)
        gw2b += np.outer(sz, g)
        gb2 += sz
        dg = w2b.T @ sz
        dh = dz2 @ w2a + dg[None, :] / n
        dz1 = dh * (z1 > 0)
        gw1 += dz1.T @ f
        gb1 += dz1.sum(axis=0)
    return total, grad


def init_params(seed=0):
    """He-style initialization (float32, NPARAMS)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS)
    p[W1:B1] = rng.standard_normal(H * F) * np.sqrt(2.0 / F)
    p[W2A:W2B] = rng.standard_normal(H * H) * np.sqrt(1.0 / H)
    p[W2B:B2] = rng.standard_normal(H * H) * np.sqrt(1.0 / H)
    p[W3:B3] = rng.standard_normal(H) * np.sqrt(1.0 / H) * 0.1
    return p.astype(np.float32)

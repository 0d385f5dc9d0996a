"""NumPy float64 restatement of the indicator network (50 -> 32 -> 32 -> 1,
tanh-form GELU, sigmoid output, mean binary cross-entropy): the checker for
the CUDA forward / backward / Adam kernels.

TEST INFRASTRUCTURE, NOT PRODUCT.

Parameter vector layout (float32 on the device, 2721 values):
    W1 [32][50]  at 0        b1 [32] at 1600
    W2 [32][32]  at 1632     b2 [32] at 2656
    w3 [32]      at 2688     b3      at 2720
"""
from __future__ import annotations

import numpy as np

N_IN, N_H = 50, 32
OFF = {"W1": 0, "b1": 1600, "W2": 1632, "b2": 2656, "w3": 2688, "b3": 2720}
N_PARAMS = 2721
K = np.sqrt(2.0 / np.pi)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[0:1600].reshape(32, 50), p[1600:1632], p[1632:2656].reshape(32, 32), p[2656:2688],
            p[2688:2720], p[2720])


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(K * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(K * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * K * (1.0 + 3 * 0.044715 * z * z)


def forward(p, X):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    z1 = X @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    return h2 @ w3 + b3, (X, z1, h1, z2, h2)


def loss_and_grad(p, X, y):
    """Mean BCE-with-logits over the batch and its gradient (same layout as p)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    logit, (X, z1, h1, z2, h2) = forward(p, X)
    y = np.asarray(y, dtype=np.float64)
    n = len(y)
    loss = np.mean(np.maximum(logit, 0) - logit * y + np.log1p(np.exp(-np.abs(logit))))
    d = (1.0 / (1.0 + np.exp(-logit)) - y) / n
    g = np.zeros(N_PARAMS)
    g[2688:2720] = h2.T @ d
    g[2720] = d.sum()
    dz2 = np.outer(d, w3) * gelu_grad(z2)
    g[1632:2656] = (dz2.T @ h1).ravel()
    g[2656:2688] = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    g[0:1600] = (dz1.T @ X).ravel()
    g[1600:1632] = dz1.sum(0)
    return loss, g


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def init_params(seed: int) -> np.ndarray:
    """He-style uniform initialisation used by the CUDA trainer's host side."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, dtype=np.float32)
    p[0:1600] = rng.uniform(-1, 1, 1600) * np.sqrt(6.0 / N_IN)
    p[1632:2656] = rng.uniform(-1, 1, 1024) * np.sqrt(6.0 / N_H)
    p[2688:2720] = rng.uniform(-1, 1, 32) * np.sqrt(6.0 / N_H)
    return p

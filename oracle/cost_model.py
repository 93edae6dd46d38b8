"""CPU oracle of the learned scheduler's network (hibf_gb300/csrc/cost_model.cu), for tests only.

float64 numpy statement of the same model -- 6 features -> 32 ReLU -> 32 ReLU -> 1, loss = mean((y - log1p(work))^2)
-- with the same flat parameter layout, so the device's forward and backward kernels can be checked against it.
The seqan/hibf reference has no learned part; this oracle is itself pinned by central finite differences
(tests/test_cost_model.py).
"""

from __future__ import annotations

import numpy as np

F, H = 6, 32
O_W1 = 0
O_B1 = O_W1 + H * F
O_W2 = O_B1 + H
O_B2 = O_W2 + H * H
O_W3 = O_B2 + H
O_B3 = O_W3 + H
PARAMS = O_B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[O_W1:O_B1].reshape(H, F), p[O_B1:O_W2], p[O_W2:O_B2].reshape(H, H), p[O_B2:O_W3], p[O_W3:O_B3],
            p[O_B3])


def forward(p, X):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64).reshape(-1, F)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ w3 + b3, h1, h2


def loss(p, X, work) -> float:
    y, _, _ = forward(p, X)
    return float(np.mean((y - np.log1p(np.asarray(work, dtype=np.float64))) ** 2))


def loss_grad(p, X, work):
    """(loss, gradient in the flat layout)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64).reshape(-1, F)
    y, h1, h2 = forward(p, X)
    e = y - np.log1p(np.asarray(work, dtype=np.float64))
    n = X.shape[0]
    dy = 2.0 * e / n
    g = np.zeros(PARAMS)
    g[O_B3] = dy.sum()
    g[O_W3:O_B3] = h2.T @ dy
    dh2 = np.outer(dy, w3) * (h2 > 0)
    g[O_B2:O_W3] = dh2.sum(0)
    g[O_W2:O_B2] = (dh2.T @ h1).reshape(-1)
    dh1 = (dh2 @ W2) * (h1 > 0)
    g[O_B1:O_W2] = dh1.sum(0)
    g[O_W1:O_B1] = (dh1.T @ X).reshape(-1)
    return float(np.mean(e ** 2)), g

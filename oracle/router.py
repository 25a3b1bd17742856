"""FP64 oracle of the learned router's network -- TEST INFRASTRUCTURE ONLY.

The reference has no learned part (its assignment scans every center, main/cuda/ClosestCenters.cu
:46-83), so there is nothing of the reference to pin this against; it restates the published
algorithms the library's kernels (kmeans_gb300/csrc/router_mlp.cu) implement, and is itself
pinned on the CPU against central finite differences (tests/test_router_cpu.py):

  forward   H = relu(X W1^T + b1),  Z = H W2^T + b2
  loss      mean over the batch of logsumexp(Z_i) - Z_i[y_i]  (softmax cross-entropy)
  backward  dZ = (softmax(Z) - onehot(y)) / B;  dW2 = dZ^T H;  db2 = sum_i dZ_i;
            dH = (dZ W2) * [H > 0];  dW1 = dH^T X;  db1 = sum_i dH_i
  Adam      (Kingma & Ba, 2015) m = b1 m + (1-b1) g;  v = b2 v + (1-b2) g^2;
            p -= lr (m / (1 - b1^t)) / (sqrt(v / (1 - b2^t)) + eps)

Parameters are one flat vector [W1 (hidden x d) | b1 | W2 (groups x hidden) | b2], row-major.
"""
from __future__ import annotations

import numpy as np


def unpack(p: np.ndarray, d: int, hidden: int, groups: int):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + hidden * d].reshape(hidden, d)
    o += hidden * d
    b1 = p[o:o + hidden]
    o += hidden
    W2 = p[o:o + groups * hidden].reshape(groups, hidden)
    o += groups * hidden
    b2 = p[o:o + groups]
    return W1, b1, W2, b2


def loss_and_grads(p, X, y, d: int, hidden: int, groups: int):
    """(mean cross-entropy, flat gradient) in FP64."""
    W1, b1, W2, b2 = unpack(p, d, hidden, groups)
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[0]
    H = np.maximum(X @ W1.T + b1, 0.0)
    Z = H @ W2.T + b2
    mx = Z.max(axis=1, keepdims=True)
    e = np.exp(Z - mx)
    s = e.sum(axis=1, keepdims=True)
    lse = mx[:, 0] + np.log(s[:, 0])
    loss = float(np.mean(lse - Z[np.arange(B), y]))
    dZ = e / s
    dZ[np.arange(B), y] -= 1.0
    dZ /= B
    gW2 = dZ.T @ H
    gb2 = dZ.sum(axis=0)
    dH = (dZ @ W2) * (H > 0)
    gW1 = dH.T @ X
    gb1 = dH.sum(axis=0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2])


def adam_train(p, X, y, d: int, hidden: int, groups: int, batch: int, steps: int,
               lr: float = 1e-3, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
    """`steps` Adam steps on consecutive batches (wrapping to row 0 when a batch would run past
    the end), as kmgb_router_mlp_train does. Returns (params, loss of the last batch before its
    update)."""
    p = np.asarray(p, dtype=np.float64).copy()
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    rows = X.shape[0]
    bsz = min(batch, rows)
    r0 = 0
    loss = 0.0
    for t in range(1, steps + 1):
        if r0 + bsz > rows:
            r0 = 0
        loss, g = loss_and_grads(p, X[r0:r0 + bsz], y[r0:r0 + bsz], d, hidden, groups)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p -= lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
        r0 += bsz
    return p, loss

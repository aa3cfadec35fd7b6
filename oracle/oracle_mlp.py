"""CPU oracle of the learned tau model (test infrastructure only).

The reference has no learned component; this is the oracle for the
library's MLP kernels (csrc/k_mlp.cu): the same network, loss and parameter
layout in float64 numpy, forward and backward written out by hand, plus a
central finite-difference gradient that pins the hand-written backward.

    parameters: W1[F][H] | b1[H] | W2[H][H] | b2[H] | w3[H] | b3
    f(x) = w3 . relu(W2^T relu(W1^T x + b1) + b2) + b3
    loss = mean((f(x) - y)^2)
"""
from __future__ import annotations

import numpy as np

F = 14
H = 32
NP = F * H + H + H * H + H + H + 1


def unpack(w: np.ndarray):
    w = np.asarray(w, dtype=np.float64)
    o = 0
    W1 = w[o:o + F * H].reshape(F, H); o += F * H
    b1 = w[o:o + H]; o += H
    W2 = w[o:o + H * H].reshape(H, H); o += H * H
    b2 = w[o:o + H]; o += H
    w3 = w[o:o + H]; o += H
    b3 = w[o]
    return W1, b1, W2, b2, w3, b3


def forward(w: np.ndarray, X: np.ndarray) -> np.ndarray:
    W1, b1, W2, b2, w3, b3 = unpack(w)
    X = np.asarray(X, dtype=np.float64)
    a1 = np.maximum(X @ W1 + b1, 0.0)
    a2 = np.maximum(a1 @ W2 + b2, 0.0)
    return a2 @ w3 + b3


def loss_grad(w: np.ndarray, X: np.ndarray, y: np.ndarray):
    """(loss, gradient) by the chain rule, float64."""
    W1, b1, W2, b2, w3, b3 = unpack(w)
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(y)
    z1 = X @ W1 + b1
    a1 = np.maximum(z1, 0.0)
    z2 = a1 @ W2 + b2
    a2 = np.maximum(z2, 0.0)
    p = a2 @ w3 + b3
    err = p - y
    loss = float(np.mean(err * err))
    gp = 2.0 * err / n                      # d loss / d p
    g_w3 = a2.T @ gp
    g_b3 = gp.sum()
    dz2 = (gp[:, None] * w3[None, :]) * (z2 > 0)
    g_W2 = a1.T @ dz2
    g_b2 = dz2.sum(0)
    dz1 = (dz2 @ W2.T) * (z1 > 0)
    g_W1 = X.T @ dz1
    g_b1 = dz1.sum(0)
    g = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [g_b3]])
    return loss, g


def numeric_grad(w: np.ndarray, X: np.ndarray, y: np.ndarray, idx, h: float = 1e-6) -> np.ndarray:
    """Central differences of the loss for the parameters in idx."""
    w = np.asarray(w, dtype=np.float64)
    out = np.zeros(len(idx))
    for t, q in enumerate(idx):
        wp = w.copy(); wp[q] += h
        wm = w.copy(); wm[q] -= h
        lp = np.mean((forward(wp, X) - y) ** 2)
        lm = np.mean((forward(wm, X) - y) ** 2)
        out[t] = (lp - lm) / (2 * h)
    return out


def init(seed: int) -> np.ndarray:
    """He-normal weights, zero biases (numpy's generator; the library's own
    initialiser is a different stream with the same law)."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / F), (F, H))
    W2 = rng.normal(0, np.sqrt(2.0 / H), (H, H))
    w3 = rng.normal(0, np.sqrt(1.0 / H), H)
    return np.concatenate([W1.ravel(), np.zeros(H), W2.ravel(), np.zeros(H), w3, [0.0]]).astype(np.float32)


def adam_train(w: np.ndarray, X: np.ndarray, y: np.ndarray, steps: int, lr: float) -> np.ndarray:
    """Full-batch Adam (b1 0.9, b2 0.999, eps 1e-8), float64."""
    w = np.asarray(w, dtype=np.float64).copy()
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    for t in range(1, steps + 1):
        _, g = loss_grad(w, X, y)
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        w -= lr * (m / (1 - 0.9 ** t)) / (np.sqrt(v / (1 - 0.999 ** t)) + 1e-8)
    return w

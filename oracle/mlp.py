"""NumPy FP64 forward/backward of the learned step-size controller's MLP (test
infrastructure: the gradient checker of the CUDA training kernels).

Layout of the flat parameter vector: W1[H][IN], b1[H], W2[H][H], b2[H], w3[H], b3.
"""

import numpy as np

IN, H = 8, 64


def split(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * IN].reshape(H, IN); o += H * IN
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, X):
    W1, b1, W2, b2, w3, b3 = split(p)
    h1 = np.tanh(X @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ w3 + b3, (h1, h2)


def loss_and_grad(p, X, T, norm):
    """sum_i (y_i - t_i)^2 / norm and its gradient."""
    W1, b1, W2, b2, w3, b3 = split(p)
    X = np.asarray(X, dtype=np.float64)
    y, (h1, h2) = forward(p, X)
    r = y - T
    loss = float(np.sum(r * r) / norm)
    dy = 2.0 * r / norm
    gw3 = h2.T @ dy
    gb3 = dy.sum()
    dz2 = np.outer(dy, w3) * (1 - h2 * h2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (1 - h1 * h1)
    gW1 = dz1.T @ X
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return loss, g

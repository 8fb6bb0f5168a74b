"""CPU reference of the rank model's forward pass and mean-squared-error
gradient -- TEST INFRASTRUCTURE ONLY (the expected values for the GPU kernels' tests).

FP64 numpy, same parameter layout as the library: W1 (F x H) | b1 (H) |
W2 (H x H) | b2 (H) | W3 (H) | b3 (1), row-major.
"""
import numpy as np


def unpack(p, F, H):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + F * H].reshape(F, H); o += F * H
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o:o + 1]
    return W1, b1, W2, b2, W3, b3


def forward(p, x, F, H):
    W1, b1, W2, b2, W3, b3 = unpack(p, F, H)
    h1 = np.maximum(x @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    return h2 @ W3 + b3[0]


def loss_and_grad(p, x, t, F, H):
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(p, F, H)
    z1 = x @ W1 + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0.0)
    y = h2 @ W3 + b3[0]
    N = x.shape[0]
    e = y - t
    loss = float(np.mean(e * e))
    dy = 2.0 * e / N
    gW3 = h2.T @ dy
    gb3 = np.array([dy.sum()])
    dz2 = np.outer(dy, W3) * (z2 > 0)
    gW2 = h1.T @ dz2
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2.T) * (z1 > 0)
    gW1 = x.T @ dz1
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, gb3])
    return loss, g

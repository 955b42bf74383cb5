"""Oracle (test infrastructure only): float64 numpy restatement of the sizing
MLP's forward pass and mean-squared-error gradient, with the same parameter
layout as the GPU kernels -- W1[32][6], b1[32], W2[32][32], b2[32], W3[32],
b3 -- followed by the normalisation block (feature mean[6], std[6], target
mean, std).  Used to check the GPU training kernels."""
from __future__ import annotations

import numpy as np

NF, H1, H2 = 6, 32, 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + H1 * NF
OFF_W2 = OFF_B1 + H1
OFF_B2 = OFF_W2 + H2 * H1
OFF_W3 = OFF_B2 + H2
OFF_B3 = OFF_W3 + H2
NP = OFF_B3 + 1


def unpack(p):
    p = np.asarray(p, np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(H1, NF)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(H2, H1)
    b2 = p[OFF_B2:OFF_W3]
    W3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    norm = p[NP:NP + 2 * NF + 2]
    return W1, b1, W2, b2, W3, b3, norm


def forward(p, feat):
    W1, b1, W2, b2, W3, b3, norm = unpack(p)
    x = (np.asarray(feat, np.float64) - norm[:NF]) / norm[NF:2 * NF]
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    y = h2 @ W3 + b3
    return x, h1, h2, y


def predict(p, feat):
    norm = unpack(p)[6]
    return forward(p, feat)[3] * norm[2 * NF + 1] + norm[2 * NF]


def gradient(p, feat, target):
    """Mean-squared-error gradient (NP entries) followed by the loss."""
    W1, b1, W2, b2, W3, b3, norm = unpack(p)
    x, h1, h2, y = forward(p, feat)
    t = (np.asarray(target, np.float64) - norm[2 * NF]) / norm[2 * NF + 1]
    e = y - t
    n = len(e)
    dy = 2.0 * e
    d2 = np.where(h2 > 0, dy[:, None] * W3[None, :], 0.0)
    d1 = np.where(h1 > 0, d2 @ W2, 0.0)
    g = np.zeros(NP + 1)
    g[OFF_W1:OFF_B1] = (d1.T @ x / n).ravel()
    g[OFF_B1:OFF_W2] = d1.mean(0)
    g[OFF_W2:OFF_B2] = (d2.T @ h1 / n).ravel()
    g[OFF_B2:OFF_W3] = d2.mean(0)
    g[OFF_W3:OFF_B3] = (dy[:, None] * h2).mean(0)
    g[OFF_B3] = dy.mean()
    g[NP] = (e * e).mean()
    return g

"""The MLP oracle itself: its analytic gradient against finite differences
(CPU only)."""
import numpy as np

from oracle import mlp_ref as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = np.concatenate([rng.normal(0, 0.3, M.NP), np.zeros(M.NF), np.ones(M.NF), [0.0, 1.0]])
    feat = rng.normal(0, 1, (64, M.NF))
    target = rng.normal(0, 1, 64)
    g = M.gradient(p, feat, target)
    loss = lambda q: M.gradient(q, feat, target)[M.NP]
    for k in list(range(0, M.NP, 97)) + [M.OFF_B3]:
        h = 1e-6
        q1, q2 = p.copy(), p.copy()
        q1[k] += h
        q2[k] -= h
        fd = (loss(q1) - loss(q2)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, g[k])

"""CPU: the MLP restatement (oracle/mlp_oracle.py) -- bfloat16 rounding and
analytic gradients against central finite differences in FP64."""
from __future__ import annotations

import numpy as np

from oracle import mlp_oracle as MO


def test_bf16_rounding():
    x = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, -2.5, 1e-30, 3.0e38], np.float32)
    got = MO.bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == np.float32(1 + 2 ** -6)
    assert got[3] == -2.5
    # every result is a bfloat16 value (low 16 bits zero)
    assert (got.view(np.uint32) & 0xFFFF == 0).all()


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n_par = 256 * 64 + 256 + 2 * (256 * 256 + 256) + 256 + 1
    p = rng.normal(scale=0.05, size=n_par)
    X = rng.normal(size=(12, 64))
    t = rng.normal(size=12)
    sw = rng.uniform(0.5, 2.0, size=12)
    mu, inv = np.zeros(64), np.ones(64)
    loss, g = MO.loss_and_grads(p, mu, inv, X, t, sw, bf=False)
    idx = rng.choice(n_par, size=40, replace=False)
    idx = np.concatenate([idx, [n_par - 1, n_par - 2, 256 * 64 + 3]])
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp = MO.loss_and_grads(q, mu, inv, X, t, sw, bf=False)[0]
        q[i] -= 2 * h
        lm = MO.loss_and_grads(q, mu, inv, X, t, sw, bf=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_adamw_first_step_moves_by_lr():
    p = np.ones(256 * 64 + 256 + 2 * (256 * 256 + 256) + 256 + 1)
    g = np.full_like(p, 0.3)
    new, m, v = MO.adamw(p, np.zeros_like(p), np.zeros_like(p), g, 1, lr=1e-2, wd=0.0)
    assert np.allclose(p - new, 1e-2, rtol=1e-6)

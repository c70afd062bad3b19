"""The numpy restatement of the learned warm start's MLP against finite differences (CPU)."""
from __future__ import annotations

import numpy as np

from oracle import mlp


def _random_params(rng):
    w = {"W1": rng.normal(0, 0.4, (64, 16)), "b1": rng.normal(0, 0.1, 64), "W2": rng.normal(0, 0.2, (64, 64)),
         "b2": rng.normal(0, 0.1, 64), "W3": rng.normal(0, 0.2, (8, 64)), "b3": rng.normal(0, 0.1, 8)}
    w["W1"][:, 14:] = 0
    w["W3"][2:] = 0
    w["b3"][2:] = 0
    return mlp.pack(w)


def test_exact_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = _random_params(rng)
    x = rng.normal(0, 1, (64, 14)).astype(np.float32)
    t = rng.normal(0, 1, (64, 2)).astype(np.float32)
    mu, sg = np.zeros(14, np.float32), np.ones(14, np.float32)
    _, ge = mlp.gradients_exact(p.astype(np.float64), x, t, mu, sg)
    for i in rng.choice(mlp.N_PARAMS, 40, replace=False):
        if ge[i] == 0.0:
            continue
        eps = 1e-6
        pp, pm = p.astype(np.float64), p.astype(np.float64)
        pp[i] += eps
        pm[i] -= eps
        fd = (mlp.loss_f64(pp, x, t, mu, sg) - mlp.loss_f64(pm, x, t, mu, sg)) / (2 * eps)
        assert abs(fd - ge[i]) <= 1e-5 * max(1.0, abs(ge[i])), (i, fd, ge[i])


def test_rounded_gradient_close_to_exact():
    rng = np.random.default_rng(1)
    p = _random_params(rng)
    x = rng.normal(0, 1, (256, 14)).astype(np.float32)
    t = rng.normal(0, 1, (256, 2)).astype(np.float32)
    mu, sg = np.zeros(14, np.float32), np.ones(14, np.float32)
    _, g = mlp.gradients(p, x, t, mu, sg)
    _, ge = mlp.gradients_exact(p, x, t, mu, sg)
    assert np.linalg.norm(g - ge) <= 0.03 * np.linalg.norm(ge)


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e38, 1e-40], dtype=np.float32)
    r = mlp.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == -2.5
    assert np.all(np.isfinite(r))

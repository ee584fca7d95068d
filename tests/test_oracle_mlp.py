"""Rank-predictor oracle (oracle/mlp.py): gradient, initialisation and Adam (CPU)."""
import numpy as np

from oracle import mlp, rng


def _data(B=64, nin=8, seed=0):
    r = np.random.default_rng(seed)
    X = r.standard_normal((B, nin))
    t = r.uniform(0.05, 0.95, B)
    return X, t


def test_gradient_matches_finite_differences():
    nin, H = 8, 32
    p = mlp.init_params(nin, H, seed=3).astype(np.float64)
    p[nin * H:nin * H + H] = 0.05      # nonzero biases so every path is exercised
    X, t = _data()
    _, g = mlp.loss_and_grad(p, X, t, nin, H)
    r = np.random.default_rng(1)
    for q in r.choice(p.size, 40, replace=False):
        e = np.zeros_like(p)
        e[q] = 1e-6
        fd = (mlp.loss_and_grad(p + e, X, t, nin, H)[0] - mlp.loss_and_grad(p - e, X, t, nin, H)[0]) / 2e-6
        assert abs(fd - g[q]) <= 1e-6 + 1e-4 * abs(g[q])


def test_init_layout_and_stream():
    nin, H = 8, 32
    p = mlp.init_params(nin, H, seed=7)
    assert p.dtype == np.float32 and p.size == mlp.nparams(nin, H) == 1377
    W1, b1, W2, b2, W3, b3 = mlp.unpack(p, nin, H)
    assert not b1.any() and not b2.any() and not b3.any()
    u = rng.uniform(7, 0x4D4C50, p.size)
    assert np.float32((u[5] * 2 - 1) * np.sqrt(6.0 / nin)) == W1.ravel()[5]
    assert np.abs(W2).max() <= np.sqrt(6.0 / H)


def test_adam_fits_a_smooth_target():
    nin, H = 8, 32
    X, _ = _data(B=256, seed=2)
    t = 1.0 / (1.0 + np.exp(-(0.8 * X[:, 0] - 0.5 * X[:, 3])))
    p = mlp.init_params(nin, H, seed=1).astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    l0 = mlp.loss_and_grad(p, X, t, nin, H)[0]
    for s in range(1, 301):
        _, g = mlp.loss_and_grad(p, X, t, nin, H)
        p, m, v = mlp.adam_step(p, g, m, v, s, 3e-3)
    assert mlp.loss_and_grad(p, X, t, nin, H)[0] < 0.05 * l0

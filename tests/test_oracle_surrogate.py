"""The oracle's FP64 MLP gradient (hand back-propagation) against central finite differences (no GPU)."""
import numpy as np

import oracle


def test_mlp_gradient_matches_finite_differences():
    n = oracle.mlp_num_params()
    assert n == 5125
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, n)
    X = rng.normal(0, 1, (24, 9)).astype(np.float32)
    Y = rng.normal(0, 1, (24, 5)).astype(np.float32)
    loss, g = oracle.mlp_loss_grad(p, X, Y)
    h = 1e-6
    for i in rng.choice(n, 60, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (oracle.mlp_loss_grad(pp, X, Y)[0] - oracle.mlp_loss_grad(pm, X, Y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * (abs(fd) + abs(g[i])) + 1e-10


def test_mlp_forward_matches_numpy():
    rng = np.random.default_rng(1)
    p = rng.normal(0, 0.3, 5125).astype(np.float32)
    X = rng.normal(0, 1, (7, 9)).astype(np.float32)
    W1, b1 = p[:576].reshape(64, 9), p[576:640]
    W2, b2 = p[640:4736].reshape(64, 64), p[4736:4800]
    W3, b3 = p[4800:5120].reshape(5, 64), p[5120:5125]
    x = X.astype(np.float64)
    ref = np.tanh(np.tanh(x @ W1.T + b1) @ W2.T + b2) @ W3.T + b3
    assert np.allclose(oracle.mlp_forward(p, X), ref, rtol=1e-12, atol=1e-12)

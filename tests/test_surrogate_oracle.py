"""The surrogate's CPU restatement checked against finite differences (no
GPU): the force-matching gradient is the parameter gradient of
sum_i v_i . dt/dx(x_i), the energy-loss gradient that of mean((t-y)^2), and
the direct-force head's gradient that of sum_i v_i . w(x_i)."""
import numpy as np

from oracle import surrogate_ref as sref


def _exact(a):
    return np.asarray(a, np.float64)


def test_force_grad_is_gradient_of_directional_derivative():
    rng = np.random.default_rng(1)
    p = rng.standard_normal(6337) * 0.3
    x = rng.standard_normal((7, 32))
    v = rng.standard_normal((7, 32))
    g = sref.force_grad(p, x, v, rnd=_exact)
    h = 1e-6
    for k in rng.choice(6336, 40, replace=False):   # b3 does not enter
        dp = np.zeros_like(p)
        dp[k] = h
        fd = (sref.directional(p + dp, x, v) - sref.directional(p - dp, x, v)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), k


def test_loss_grad_is_gradient_of_loss():
    rng = np.random.default_rng(2)
    p = rng.standard_normal(6337) * 0.3
    x = rng.standard_normal((9, 32))
    y = rng.standard_normal(9)

    def loss(q):
        W1, b1, W2, b2, w3, b3 = sref.unpack(q)
        t = np.tanh(np.tanh(x @ W1.T + b1) @ W2.T + b2) @ w3 + b3
        return ((t - y) ** 2).mean()

    # the oracle's gradient with its roundings switched off
    orig = sref.bf16
    try:
        sref.bf16 = _exact
        _, g = sref.loss_grad(p, x, y)
    finally:
        sref.bf16 = orig
    h = 1e-6
    for k in list(rng.choice(6337, 40, replace=False)) + [6336]:
        dp = np.zeros_like(p)
        dp[k] = h
        fd = (loss(p + dp) - loss(p - dp)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), k


def test_head_grad_is_gradient_of_projection():
    rng = np.random.default_rng(3)
    H = 32
    n = 32 * H + H + H * H + H + 32 * H + 32
    p = rng.standard_normal(n) * 0.3
    x = rng.standard_normal((6, 32))
    v = rng.standard_normal((6, 32))
    g = sref.head_grad(p, x, v, H)
    assert g.shape == (n,)
    h = 1e-6
    for k in rng.choice(n, 60, replace=False):
        dp = np.zeros_like(p)
        dp[k] = h
        fd = ((sref.head_forward(p + dp, x, H) * v).sum()
              - (sref.head_forward(p - dp, x, H) * v).sum()) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), k

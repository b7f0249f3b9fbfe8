"""The FP64 surrogate reference: analytic gradients agree with central
finite differences (CPU only)."""
import numpy as np

from oracle import surrogate_ref as sr


def test_param_count_of_the_configured_net():
    # 2 -> 24 -> 24 -> 24 -> 1 with 3^3 kernels and biases
    assert sr.param_count(24) == 27 * (2 * 24 + 24 * 24 * 2 + 24) + 24 * 3 + 1


def test_analytic_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    ch = 4
    u = rng.random((5, 6, 7))
    k = 0.02 + 0.13 * rng.random((5, 6, 7))
    target = 0.01 * rng.standard_normal((5, 6, 7))
    p = sr.init_params(ch, seed=3)
    p[-1] = 0.05   # a non-zero last bias
    loss, g = sr.loss_and_grad(p, u, k, target, ch)
    idx = rng.choice(p.size, 40, replace=False)
    eps = 1e-6
    for i in idx:
        pp = p.copy()
        pm = p.copy()
        pp[i] += eps
        pm[i] -= eps
        lp, _ = sr.loss_and_grad(pp, u, k, target, ch)
        lm, _ = sr.loss_and_grad(pm, u, k, target, ch)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])


def test_forward_is_translation_equivariant_on_the_torus():
    rng = np.random.default_rng(2)
    u = rng.random((6, 6, 6))
    k = rng.random((6, 6, 6))
    p = sr.init_params(3, seed=4)
    a, _ = sr.forward(p, u, k, 3)
    b, _ = sr.forward(p, np.roll(u, 2, axis=1), np.roll(k, 2, axis=1), 3)
    np.testing.assert_allclose(np.roll(a, 2, axis=1), b, rtol=1e-12, atol=1e-14)

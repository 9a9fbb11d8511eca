"""The CPU oracle of the spectral surrogate network: BF16 rounding and the
analytic gradient against central finite differences (no GPU)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle"))
import mlp_ref  # noqa: E402


def test_bf16_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -3.14159, 0.0], dtype=np.float32)
    r = mlp_ref.bf16_round(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even (1); 1 + 3*2^-8 ties up to 1 + 2^-6
    np.testing.assert_array_equal(r[:4], np.array([1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6], dtype=np.float32))
    assert abs(r[4] - np.float32(-3.140625)) == 0.0
    assert r[5] == 0.0
    assert np.all(mlp_ref.bf16_round(r) == r)


def test_gradient_matches_finite_differences():
    widths = [6, 16, 16, 5]
    rng = np.random.default_rng(3)
    p = mlp_ref.init_params(widths, seed=1).astype(np.float64)
    p += rng.normal(0, 0.05, p.size)  # non-zero biases
    x = rng.normal(size=(7, 6))
    t = rng.normal(size=(7, 5))
    loss, g = mlp_ref.loss_and_grad(p, widths, x, t, bf16=False)
    assert g.size == mlp_ref.n_params(widths)
    idx = rng.choice(p.size, 40, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = mlp_ref.loss_and_grad(p + e, widths, x, t, bf16=False)
        lm, _ = mlp_ref.loss_and_grad(p - e, widths, x, t, bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(fd), (i, fd, g[i])


def test_gelu_derivative():
    z = np.linspace(-6, 6, 101)
    h = 1e-6
    fd = (mlp_ref.gelu(z + h) - mlp_ref.gelu(z - h)) / (2 * h)
    np.testing.assert_allclose(mlp_ref.gelu_grad(z), fd, atol=1e-8)

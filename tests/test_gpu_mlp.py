"""The surrogate network's GPU kernels (dg_mlp_*) against the CPU oracle
(oracle/mlp_ref.py): forward pass, loss and parameter gradient with the
GEMMs on the tensor cores and on the CUDA cores (the default), and a short
training run. The GPU accumulates in FP32 with BF16 weights; the oracle uses
the same BF16 weights in float64."""
import os
import sys

import numpy as np
import pytest

from conftest import rel_l2

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle"))
import mlp_ref  # noqa: E402

pytestmark = pytest.mark.gpu

SURROGATE_WIDTHS = [6, 256, 256, 256, 256, 512]


@pytest.mark.parametrize("tc", [True, False])
@pytest.mark.parametrize("widths,n", [([6, 32, 32, 7], 5), ([6, 256, 256, 256, 256, 512], 300),
                                      ([6, 100, 70, 9], 131)])
def test_forward_matches_oracle(pkg, widths, n, tc):
    rng = np.random.default_rng(1)
    p = mlp_ref.init_params(widths, seed=2)
    p[mlp_ref.n_params(widths) - widths[-1]:] = rng.normal(0, 0.1, widths[-1])
    x = rng.normal(size=(n, widths[0])).astype(np.float32)
    net = pkg.gpu.Network(widths)
    assert not net.tensor_cores
    net.set_tensor_cores(tc)
    assert net.tensor_cores == tc
    net.set_params(p)
    np.testing.assert_array_equal(net.get_params(), p)
    y = net.forward(x)
    y_ref, _ = mlp_ref.forward(p, widths, x)
    assert rel_l2(y, y_ref) <= 1e-5


@pytest.mark.parametrize("tc", [True, False])
@pytest.mark.parametrize("widths,n", [([6, 32, 32, 7], 9), (SURROGATE_WIDTHS, 128), ([6, 100, 70, 9], 200)])
def test_gradient_matches_oracle(pkg, widths, n, tc):
    rng = np.random.default_rng(4)
    p = mlp_ref.init_params(widths, seed=5)
    x = rng.normal(size=(n, widths[0])).astype(np.float32)
    t = rng.normal(size=(n, widths[-1])).astype(np.float32)
    net = pkg.gpu.Network(widths)
    net.set_tensor_cores(tc)
    net.set_params(p)
    g, loss = net.gradient(x, t)
    loss_ref, g_ref = mlp_ref.loss_and_grad(p, widths, x, t)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    # per layer, weights and biases separately
    pos = 0
    for k, m in zip(widths[:-1], widths[1:]):
        for size in (m * k, m):
            assert rel_l2(g[pos:pos + size], g_ref[pos:pos + size]) <= 1e-4, (k, m, size)
            pos += size


def test_training_reduces_loss(pkg):
    widths = [6, 64, 64, 16]
    rng = np.random.default_rng(7)
    x = rng.uniform(-1, 1, size=(2048, 6)).astype(np.float32)
    W = rng.normal(size=(6, 16))
    t = np.sin(x @ W).astype(np.float32)
    net = pkg.gpu.Network(widths)
    net.set_params(mlp_ref.init_params(widths, seed=8))
    net.set_data(x, t)
    losses = net.train(600, 128, 3e-3, 3e-5, seed=9)
    assert losses.shape == (600,)
    assert np.mean(losses[-50:]) < 0.1 * np.mean(losses[:10])
    # the network's own loss on the training rows agrees with the oracle's
    _, loss = net.gradient(x, t)
    loss_ref, _ = mlp_ref.loss_and_grad(net.get_params(), widths, x, t)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref


def test_invalid_arguments(pkg):
    with pytest.raises(pkg.gpu.SolverError):
        pkg.gpu.Network([6])
    net = pkg.gpu.Network([6, 8, 3])
    with pytest.raises(ValueError):
        net.set_params(np.zeros(5, dtype=np.float32))
    net.set_data(np.zeros((4, 6), np.float32), np.zeros((4, 3), np.float32))
    with pytest.raises(pkg.gpu.SolverError, match="fewer training rows"):
        net.train(3, 8, 1e-3, 1e-4)

"""CPU oracle of the spectral surrogate network (test infrastructure only).

A float64 numpy restatement of what the GPU kernels of
dgfem-acoustic_gb300/csrc/mlp.cu compute: a fully connected network with
exact-erf GELU hidden layers and a linear output layer, whose weights enter
the forward and backward passes rounded to BF16 (round to nearest even),
trained on the mean squared error. The reference has no such network (it
answers every query with a DG run); this file is the checker of the GPU
forward pass and gradients, and is imported only by the tests.

Parameter layout (as in the C ABI): one flat vector, per layer W [out][in]
row-major then b [out].
"""
import math

import numpy as np

_erf = np.vectorize(math.erf, otypes=[np.float64])


def bf16_round(x):
    """float32 values rounded to the nearest BF16 (ties to even), as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def unpack(params, widths):
    """[(W, b)] per layer from the flat parameter vector."""
    out, pos = [], 0
    for k, n in zip(widths[:-1], widths[1:]):
        W = np.asarray(params[pos:pos + n * k]).reshape(n, k)
        pos += n * k
        b = np.asarray(params[pos:pos + n])
        pos += n
        out.append((W, b))
    return out


def n_params(widths):
    return sum(n * k + n for k, n in zip(widths[:-1], widths[1:]))


def forward(params, widths, x, bf16=True):
    """Outputs and the per-layer (input, pre-activation) cache, float64."""
    layers = unpack(params, widths)
    a = np.asarray(x, dtype=np.float64)
    cache = []
    for li, (W, b) in enumerate(layers):
        Wq = bf16_round(W).astype(np.float64) if bf16 else np.asarray(W, dtype=np.float64)
        z = a @ Wq.T + np.asarray(b, dtype=np.float64)
        cache.append((a, z, Wq))
        a = z if li == len(layers) - 1 else gelu(z)
    return a, cache


def loss_and_grad(params, widths, x, t, bf16=True):
    """Mean squared error over every output and its gradient with respect to
    the flat parameters (the BF16 weights are treated as the weights: the
    gradient is taken at the rounded values, as the GPU backward pass does)."""
    y, cache = forward(params, widths, x, bf16)
    d = y - np.asarray(t, dtype=np.float64)
    loss = float(np.mean(d * d))
    dy = 2.0 * d / d.size
    grads = []
    L = len(cache)
    for li in range(L - 1, -1, -1):
        a, z, Wq = cache[li]
        dz = dy if li == L - 1 else dy * gelu_grad(z)
        grads.append((dz.T @ a, dz.sum(axis=0)))
        dy = dz @ Wq
    flat = []
    for dW, db in reversed(grads):
        flat += [dW.reshape(-1), db]
    return loss, np.concatenate(flat)


def init_params(widths, seed=0):
    """He-style initialisation (normal, std sqrt(2/fan_in)), zero biases."""
    rng = np.random.default_rng(seed)
    flat = []
    for k, n in zip(widths[:-1], widths[1:]):
        flat += [rng.normal(0.0, math.sqrt(2.0 / k), size=n * k), np.zeros(n)]
    return np.concatenate(flat).astype(np.float32)

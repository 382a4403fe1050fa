"""CPU checks of the warm-start MLP oracle (oracle/mlp.py): bfloat16
rounding known answers and float64 backpropagation against central finite
differences, so the oracle the CUDA kernels are compared with is itself
right."""

import numpy as np

from oracle import mlp


def test_bf16_round_to_nearest_even():
    one = 1.0
    assert mlp.bf16(one) == one
    assert mlp.bf16(1 + 2.0**-8) == 1.0  # tie -> even mantissa (0)
    assert mlp.bf16(1 + 3 * 2.0**-8) == 1 + 2.0**-6  # tie -> even mantissa (2)
    assert mlp.bf16(1 + 2.0**-8 + 2.0**-12) == 1 + 2.0**-7  # above the tie
    assert mlp.bf16(-3.0) == -3.0
    x = np.random.default_rng(0).normal(size=1000)
    r = mlp.bf16(x)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0**-8)


def _setup(seed=0):
    rng = np.random.default_rng(seed)
    dims = [5, 7, 6, 3]
    layers = [(rng.normal(size=(dims[i + 1], dims[i])) / np.sqrt(dims[i]),
               rng.normal(size=dims[i + 1]) * 0.1) for i in range(3)]
    x = rng.normal(size=(4, dims[0]))
    t = rng.normal(size=(4, dims[-1]))
    return layers, x, t


def _loss(layers, x, t):
    y = mlp.forward(layers, x, rounding=False)["y"]
    return mlp.mse(y, t, rounding=False)[0]


def test_backward_matches_finite_differences():
    layers, x, t = _setup()
    cache = mlp.forward(layers, x, rounding=False)
    _, dy = mlp.mse(cache["y"], t, rounding=False)
    grads = mlp.backward(layers, cache, dy, rounding=False)
    h = 1e-6
    for li, (w, b) in enumerate(layers):
        for arr, g in ((w, grads[li][0]), (b, grads[li][1])):
            num = np.zeros_like(arr)
            for idx in np.ndindex(arr.shape):
                old = arr[idx]
                arr[idx] = old + h
                lp = _loss(layers, x, t)
                arr[idx] = old - h
                lm = _loss(layers, x, t)
                arr[idx] = old
                num[idx] = (lp - lm) / (2 * h)
            np.testing.assert_allclose(g, num, rtol=1e-6, atol=1e-9)


def test_gelu_grad_matches_finite_differences():
    v = np.linspace(-4, 4, 33)
    h = 1e-6
    num = (mlp.gelu(v + h) - mlp.gelu(v - h)) / (2 * h)
    np.testing.assert_allclose(mlp.gelu_grad(v), num, rtol=1e-7, atol=1e-9)


def test_adam_first_step_moves_by_lr():
    w = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -0.1, 0.0])
    w1, m, v = mlp.adam(w, g, np.zeros(3), np.zeros(3), 1, lr=1e-2)
    # bias-corrected first step: -lr * sign(g) (up to eps)
    np.testing.assert_allclose(w1, w - 1e-2 * np.sign(g), rtol=1e-6, atol=1e-9)

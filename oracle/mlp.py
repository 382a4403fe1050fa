"""The warm-start MLP's forward pass, loss, backward pass and Adam (oracle).

TEST INFRASTRUCTURE ONLY. voltax has no learned warm start (its DC Newton
starts from the caller's guess or zeros, voltax/analysis.py:410-431), so
there is no reference implementation to restate; this module is the
textbook algorithm written in float64 numpy:

* layers ``y = act(x W^T + b)``, GELU ``v Phi(v)`` (exact erf form) on the
  two hidden layers, none on the output;
* loss ``sum (y - t)^2 / (M N)``, output gradient ``2 (y - t) / (M N)``;
* backpropagation ``dW = dY^T X``, ``db = sum_m dY``,
  ``dX = (dY W) * gelu'(pre)``;
* Adam (Kingma & Ba 2015, Algorithm 1) with bias correction.

With ``rounding=True`` it rounds to bfloat16 (round to nearest even) at the
points where the CUDA kernels store BF16 -- normalised inputs, weights,
hidden activations and the gradients handed from layer to layer -- and
forms the normalisation in float32 as they do, so the kernels can be
compared with it up to the order of their FP32 sums. With
``rounding=False`` it is plain float64 backpropagation, which the CPU tests
check against finite differences.
"""

from __future__ import annotations

import math

import numpy as np

_erf = np.vectorize(math.erf, otypes=[np.float64])


def bf16(x) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(v):
    return 0.5 * v * (1.0 + _erf(v / math.sqrt(2.0)))


def gelu_grad(v):
    return 0.5 * (1.0 + _erf(v / math.sqrt(2.0))) + v * np.exp(-0.5 * v * v) / math.sqrt(
        2.0 * math.pi)


def normalize(x, mean, inv_std, rounding=True):
    if not rounding:
        return (np.asarray(x, np.float64) - mean) * inv_std
    xf = np.asarray(x, np.float64).astype(np.float32)
    return bf16((xf - np.float32(0) - mean.astype(np.float32)) * inv_std.astype(np.float32))


def forward(layers, x, rounding=True):
    """layers: [(W (out, in), b (out,)), ...] float weights. Returns the
    cache of every layer: inputs, pre-activations and the output."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    h = np.asarray(x, np.float64)
    cache = {"inputs": [], "pre": []}
    for i, (w, b) in enumerate(layers):
        cache["inputs"].append(h)
        pre = h @ r(w).T + np.asarray(b, np.float64)
        cache["pre"].append(pre)
        last = i == len(layers) - 1
        h = pre if last else r(gelu(pre))
    cache["y"] = h
    return cache


def mse(y, t, rounding=True):
    M, N = y.shape
    d = y - t
    loss = float(np.sum(d * d) / (M * N))
    dy = 2.0 * d / (M * N)
    return loss, (bf16(dy) if rounding else dy)


def backward(layers, cache, dy, rounding=True):
    """Gradients [(dW, db), ...] of the loss whose output gradient is dy."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    grads = [None] * len(layers)
    g = dy
    for i in range(len(layers) - 1, -1, -1):
        w, _ = layers[i]
        x = cache["inputs"][i]
        grads[i] = (g.T @ x, g.sum(0))
        if i > 0:
            g = r((g @ r(w)) * gelu_grad(cache["pre"][i - 1]))
    return grads


def adam(w, g, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step; returns (w, m, v)."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v

"""FP64 NumPy restatement of the proposal MLP -- TEST INFRASTRUCTURE ONLY.

Same parameter layout as tailor_gb300/csrc/tlr_mlp.cu: for each layer,
W [out][in] row-major then b [out]; SiLU between layers, linear output;
loss = mean((Y - T)^2).  Used to check the GPU forward pass and gradients.
"""
from __future__ import annotations

import numpy as np


def layer_sizes(n_in, width, depth, n_out):
    sizes = [n_in] + [width] * depth + [n_out]
    return list(zip(sizes[:-1], sizes[1:]))


def unpack(params, n_in, width, depth, n_out):
    out, off = [], 0
    for i, o in layer_sizes(n_in, width, depth, n_out):
        W = params[off:off + i * o].reshape(o, i)
        off += i * o
        b = params[off:off + o]
        off += o
        out.append((W, b))
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(params, X, shape):
    layers = unpack(np.asarray(params, np.float64), *shape)
    a = np.asarray(X, np.float64)
    cache = [(a, None)]
    for k, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = silu(z) if k + 1 < len(layers) else z
        cache.append((a, z))
    return a, cache, layers


def loss_and_grad(params, X, T, shape):
    Y, cache, layers = forward(params, X, shape)
    n, o = Y.shape
    d = Y - np.asarray(T, np.float64)
    loss = float(np.mean(d * d))
    dA = 2.0 * d / (n * o)
    grads = []
    for k in range(len(layers) - 1, -1, -1):
        W, b = layers[k]
        z = cache[k + 1][1]
        if k + 1 < len(layers):
            s = 1.0 / (1.0 + np.exp(-z))
            dA = dA * (s * (1.0 + z * (1.0 - s)))
        a_prev = cache[k][0]
        grads.append((dA.T @ a_prev, dA.sum(0)))
        dA = dA @ W
    flat = []
    for gW, gb in reversed(grads):
        flat += [gW.reshape(-1), gb]
    return loss, np.concatenate(flat)

"""CPU restatement (float64 numpy) of the sizing model's network -- TEST INFRASTRUCTURE ONLY.

Checks the CUDA forward / backward kernels of the learned sizer: same layer layout (W of layer l
is dims[l] x dims[l+1] row-major, then b), ReLU on hidden layers, loss = mean squared error over
the batch.  The reference has no learned component; this is the checker of our own network.
"""
from __future__ import annotations

import numpy as np


def unpack(params, dims):
    layers, off = [], 0
    for k, m in zip(dims[:-1], dims[1:]):
        W = np.asarray(params[off:off + k * m], dtype=np.float64).reshape(k, m)
        off += k * m
        b = np.asarray(params[off:off + m], dtype=np.float64)
        off += m
        layers.append((W, b))
    assert off == len(params)
    return layers


def forward(params, dims, X):
    acts = [np.asarray(X, dtype=np.float64)]
    layers = unpack(params, dims)
    for i, (W, b) in enumerate(layers):
        z = acts[-1] @ W + b
        acts.append(np.maximum(z, 0.0) if i + 1 < len(layers) else z)
    return acts[-1][:, 0], acts


def loss_and_grad(params, dims, X, T):
    """(mean squared error, gradient w.r.t. the flat parameter vector) by backpropagation."""
    y, acts = forward(params, dims, X)
    T = np.asarray(T, dtype=np.float64)
    n = len(T)
    layers = unpack(params, dims)
    dz = (2.0 * (y - T) / n)[:, None]
    grads = []
    for i in range(len(layers) - 1, -1, -1):
        W, _ = layers[i]
        a_in = acts[i]
        grads.append((a_in.T @ dz, dz.sum(0)))
        if i > 0:
            dz = (dz @ W.T) * (acts[i] > 0)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return float(np.mean((y - T) ** 2)), flat


def numeric_grad(params, dims, X, T, eps=1e-6):
    """Central differences of the loss (to check loss_and_grad itself)."""
    p = np.asarray(params, dtype=np.float64).copy()
    g = np.zeros_like(p)
    for i in range(len(p)):
        p[i] += eps
        lp = np.mean((forward(p, dims, X)[0] - T) ** 2)
        p[i] -= 2 * eps
        lm = np.mean((forward(p, dims, X)[0] - T) ** 2)
        p[i] += eps
        g[i] = (lp - lm) / (2 * eps)
    return g

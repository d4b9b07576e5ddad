"""FP64 numpy MLP (test infrastructure): forward, analytic backward of the
batch mean squared error and finite differences, on the parameter layout of
planet_renderer_gb300.atmosphere.mlp (per layer W (out x in) row-major, b).
Checks the GPU training kernel's gradients."""

from __future__ import annotations

import numpy as np


def _unpack(params, shapes):
    out, o = [], 0
    for n_out, n_in in shapes:
        W = params[o:o + n_out * n_in].reshape(n_out, n_in)
        o += n_out * n_in
        b = params[o:o + n_out]
        o += n_out
        out.append((W, b))
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(params, shapes, x):
    a = np.asarray(x, dtype=np.float64)
    layers = _unpack(np.asarray(params, dtype=np.float64), shapes)
    for i, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = z if i == len(layers) - 1 else silu(z)
    return a


def loss(params, shapes, x, t, weights=None):
    y = forward(params, shapes, x)
    w = 1.0 if weights is None else np.asarray(weights, dtype=np.float64)
    return float(np.mean(w * (y - np.asarray(t, dtype=np.float64)) ** 2))


def gradient(params, shapes, x, t, weights=None):
    """d loss / d params, analytic, float64; loss = mean(w (y - t)^2)."""

    p = np.asarray(params, dtype=np.float64)
    layers = _unpack(p, shapes)
    acts, zs = [np.asarray(x, dtype=np.float64)], []
    for i, (W, b) in enumerate(layers):
        z = acts[-1] @ W.T + b
        zs.append(z)
        acts.append(z if i == len(layers) - 1 else silu(z))
    y = acts[-1]
    w = 1.0 if weights is None else np.asarray(weights, dtype=np.float64)
    d = 2.0 * w * (y - np.asarray(t, dtype=np.float64)) / y.size
    grads = []
    for i in range(len(layers) - 1, -1, -1):
        W, _ = layers[i]
        grads.append((d.T @ acts[i], d.sum(axis=0)))
        if i > 0:
            z = zs[i - 1]
            s = 1.0 / (1.0 + np.exp(-z))
            d = (d @ W) * (s * (1.0 + z * (1.0 - s)))
    flat = []
    for gW, gb in reversed(grads):
        flat.extend([gW.ravel(), gb])
    return np.concatenate(flat)


def finite_difference(params, shapes, x, t, indices, h=1e-6, weights=None):
    p = np.asarray(params, dtype=np.float64).copy()
    out = []
    for i in indices:
        old = p[i]
        p[i] = old + h
        up = loss(p, shapes, x, t, weights)
        p[i] = old - h
        dn = loss(p, shapes, x, t, weights)
        p[i] = old
        out.append((up - dn) / (2 * h))
    return np.array(out)

"""FP64 numpy reference of the learned surrogate (test infrastructure only).

The network (no counterpart in the reference library): four 3x3x3
convolutions on a periodic grid, channels 2 -> C -> C -> C -> 1, GELU after
the first three, and a residual update u' = u + conv4(...).  Inputs are the
field u and the coefficient kappa.  This module computes the forward pass,
the MSE loss against a target increment and the analytic gradients, so the
GPU kernels' forward and backward passes can be checked; the analytic
gradient is itself checked against finite differences in
tests/test_surrogate_oracle.py.

Layouts: fields (nz, ny, nx); activations (nz, ny, nx, C); weights
W[tap][cin][cout] with tap = (dz+1)*9 + (dy+1)*3 + (dx+1); the flat
parameter vector is W1, b1, W2, b2, W3, b3, W4, b4.
"""
from __future__ import annotations

import math

import numpy as np

TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def layer_shapes(channels: int = 24):
    c = channels
    return [(2, c), (c, c), (c, c), (c, 1)]


def param_count(channels: int = 24) -> int:
    return sum(27 * ci * co + co for ci, co in layer_shapes(channels))


def unflatten(params: np.ndarray, channels: int = 24):
    out = []
    o = 0
    for ci, co in layer_shapes(channels):
        w = params[o:o + 27 * ci * co].reshape(27, ci, co)
        o += 27 * ci * co
        b = params[o:o + co]
        o += co
        out.append((w, b))
    return out


def flatten(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([w.reshape(-1), b.reshape(-1)]) for w, b in layers])


def init_params(channels: int = 24, seed: int = 0) -> np.ndarray:
    """He-style init scaled down for the last layer (the net starts close to
    the identity map u' = u)."""
    rng = np.random.default_rng(seed)
    layers = []
    for li, (ci, co) in enumerate(layer_shapes(channels)):
        std = math.sqrt(2.0 / (27 * ci))
        if li == 3:
            std *= 0.1
        layers.append((rng.normal(0.0, std, (27, ci, co)), np.zeros(co)))
    return flatten(layers)


def shift(x: np.ndarray, tap) -> np.ndarray:
    """s[v] = x[v + offset(tap)] on the torus (x has spatial axes 0..2)."""
    dz, dy, dx = tap
    return np.roll(x, shift=(-dz, -dy, -dx), axis=(0, 1, 2))


def conv(x: np.ndarray, w: np.ndarray, b: np.ndarray) -> np.ndarray:
    out = np.zeros(x.shape[:3] + (w.shape[2],))
    for t, tap in enumerate(TAPS):
        out += shift(x, tap) @ w[t]
    return out + b


def gelu(z):
    from scipy.special import erf
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    from scipy.special import erf
    return 0.5 * (1.0 + erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(params: np.ndarray, u: np.ndarray, kappa: np.ndarray, channels: int = 24):
    """Returns (du, cache); u' = u + du."""
    layers = unflatten(params, channels)
    x = np.stack([u, kappa], axis=-1)
    cache = {"x": [x], "z": []}
    h = x
    for li, (w, b) in enumerate(layers):
        z = conv(h, w, b)
        cache["z"].append(z)
        if li < 3:
            h = gelu(z)
            cache["x"].append(h)
        else:
            h = z
    return h[..., 0], cache


def loss_and_grad(params: np.ndarray, u, kappa, target_du, channels: int = 24):
    """MSE between du and target_du (mean over cells) and d loss / d params."""
    layers = unflatten(params, channels)
    du, cache = forward(params, u, kappa, channels)
    n = du.size
    diff = du - target_du
    loss = float(np.mean(diff * diff))
    g = (2.0 / n) * diff[..., None]          # d loss / d z4
    grads = [None] * 4
    for li in range(3, -1, -1):
        w, b = layers[li]
        xin = cache["x"][li]
        gw = np.zeros_like(w)
        for t, tap in enumerate(TAPS):
            xs = shift(xin, tap)
            gw[t] = xs.reshape(-1, xs.shape[-1]).T @ g.reshape(-1, g.shape[-1])
        gb = g.reshape(-1, g.shape[-1]).sum(axis=0)
        grads[li] = (gw, gb)
        if li > 0:
            # d loss / d xin: transpose convolution (the taps mirrored)
            gx = np.zeros_like(xin)
            for t, tap in enumerate(TAPS):
                neg = (-tap[0], -tap[1], -tap[2])
                gx += shift(g, neg) @ w[t].T
            g = gx * gelu_grad(cache["z"][li - 1])
    return loss, flatten(grads)

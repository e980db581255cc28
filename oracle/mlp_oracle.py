"""The learned closure's network in numpy -- TEST INFRASTRUCTURE ONLY.

A float64 restatement of the fully connected net of gfs-dycore_gb300's
gd_mlp (no counterpart in the reference: the closure is this project's own
addition): nin -> nhidden (GELU with the exact normal CDF) x nlayers -> nout,
parameters packed layer after layer as W [fout][fin] row-major then b
[fout], the forward pass reading the weights rounded to BF16 (round to
nearest even) and the biases as they are, the loss the mean of the squared
errors over all outputs.  Only tests use it, to check the GPU forward pass
and gradients, and it is itself checked against finite differences.
"""
import numpy as np
from scipy.special import erf

SQRT1_2 = 0.70710678118654752
INV_SQRT2PI = 0.39894228040143268


def bf16(x):
    """float32 values rounded to bfloat16 (nearest, ties to even), as float32."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def shapes(nin, nhidden, nlayers, nout):
    sizes = [nin] + [nhidden] * nlayers + [nout]
    return [(sizes[i + 1], sizes[i]) for i in range(len(sizes) - 1)]


def unpack(params, shp, round_weights=True):
    """(W, b) per layer in float64: with round_weights the weights as the GPU
    reads them (float32 parameters rounded to BF16, biases float32), without
    it the parameters exactly as given."""
    out, o = [], 0
    for fo, fi in shp:
        W = np.asarray(params[o:o + fo * fi]).reshape(fo, fi)
        o += fo * fi
        b = np.asarray(params[o:o + fo])
        o += fo
        if round_weights:
            W, b = bf16(W.astype(np.float32)), b.astype(np.float32)
        out.append((W.astype(np.float64), b.astype(np.float64)))
    assert o == len(params)
    return out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z * SQRT1_2))


def gelu_d(z):
    return 0.5 * (1.0 + erf(z * SQRT1_2)) + z * INV_SQRT2PI * np.exp(-0.5 * z * z)


def forward(params, shp, x, round_weights=True):
    """y [n][nout] and the per-layer (input, pre-activation) cache."""
    layers = unpack(params, shp, round_weights)
    a = np.asarray(x, np.float64)
    cache = []
    for i, (W, b) in enumerate(layers):
        z = a @ W.T + b
        cache.append((a, z))
        a = gelu(z) if i < len(layers) - 1 else z
    return a, cache


def loss_grad(params, shp, x, t, round_weights=True):
    """Mean squared error and its gradient in the packed layout; with
    round_weights the gradient is taken at the BF16-rounded weights."""
    layers = unpack(params, shp, round_weights)
    y, cache = forward(params, shp, x, round_weights)
    d = y - np.asarray(t, np.float64)
    loss = float(np.mean(d * d))
    g = 2.0 * d / d.size
    grads = []
    for i in range(len(layers) - 1, -1, -1):
        a_in, z = cache[i]
        W, _ = layers[i]
        if i < len(layers) - 1:
            g = g * gelu_d(z)
        grads.append((g.T @ a_in, g.sum(axis=0)))
        g = g @ W
    grads.reverse()
    packed = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, packed

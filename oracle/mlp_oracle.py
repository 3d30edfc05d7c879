"""CPU oracle of the learned TRSK correction network (test infrastructure).

A numpy restatement of the network the CUDA kernels train and apply:
24 -> 64 -> 64 -> 1 with GELU (tanh form), BF16 inputs and weights for the two
matrix products with FP32 accumulation, FP32 third layer, mean-squared-error
loss and Adam.  The rounding points follow the kernels: the inputs x, the
weights W1 and W2, the first hidden layer before the second product, and the
back-propagated gradients dZ2 and dZ1 before their products are rounded to
BF16 (round to nearest, ties to even); everything else is FP32.

Parameter vector layout (FP32, 5825 values), shared with the library:
    W1[64][24] (out-major), b1[64], W2[64][64] (out-major), b2[64], w3[64], b3
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf

NIN, NH = 24, 64
SIZES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("w3", (NH,)),
         ("b3", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=np.float32).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float32).ravel() for name, _ in SIZES])


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).copy()
    nan = np.isnan(a)
    out[nan] = a[nan]
    return out


def bf16_bits(a):
    return (bf16(a).view(np.uint32) >> 16).astype(np.uint16)


_C = math.sqrt(2.0 / math.pi)
_A = 0.044715


def gelu(z):
    """GELU, tanh form (Hendrycks & Gimpel 2016), as the kernels use."""
    z64 = z.astype(np.float64)
    return (0.5 * z64 * (1.0 + np.tanh(_C * (z64 + _A * z64 ** 3)))).astype(np.float32)


def gelu_grad(z):
    z64 = z.astype(np.float64)
    th = np.tanh(_C * (z64 + _A * z64 ** 3))
    return (0.5 * (1.0 + th) + 0.5 * z64 * (1.0 - th * th) * _C * (1.0 + 3.0 * _A * z64 * z64)
            ).astype(np.float32)


def init_params(seed: int = 0):
    """Uniform Glorot initialisation, zero biases."""
    rng = np.random.default_rng(seed)
    d = {}
    a1 = math.sqrt(6.0 / (NIN + NH))
    a2 = math.sqrt(6.0 / (NH + NH))
    a3 = math.sqrt(6.0 / (NH + 1))
    d["W1"] = rng.uniform(-a1, a1, (NH, NIN))
    d["b1"] = np.zeros(NH)
    d["W2"] = rng.uniform(-a2, a2, (NH, NH))
    d["b2"] = np.zeros(NH)
    d["w3"] = rng.uniform(-a3, a3, NH)
    d["b3"] = np.zeros(1)
    return pack(d)


def forward(p, x):
    """y[N] and the intermediates for x[N, 24] (float32, rounded to BF16)."""
    P = unpack(p)
    xb = bf16(x).astype(np.float64)
    z1 = (xb @ bf16(P["W1"]).astype(np.float64).T + P["b1"]).astype(np.float32)
    h1 = gelu(z1)
    h1b = bf16(h1)
    z2 = (h1b.astype(np.float64) @ bf16(P["W2"]).astype(np.float64).T + P["b2"]).astype(np.float32)
    h2 = gelu(z2)
    y = (h2.astype(np.float64) @ P["w3"].astype(np.float64) + P["b3"][0]).astype(np.float32)
    return y, {"xb": xb, "z1": z1, "h1b": h1b, "z2": z2, "h2": h2}


def loss_and_grad(p, x, t, w=None):
    """Weighted mean squared error sum w (y - t)^2 / n and its gradient
    (parameter-vector layout); w None means all weights 1."""
    P = unpack(p)
    y, c = forward(p, x)
    n = x.shape[0]
    w = np.ones(n) if w is None else np.asarray(w, dtype=np.float64)
    r = (y - t).astype(np.float64)
    loss = float(np.mean(w * r * r))
    dy = (2.0 * w * r / n).astype(np.float32)
    g = {}
    g["w3"] = (c["h2"].astype(np.float64).T @ dy).astype(np.float32)
    g["b3"] = np.array([dy.sum(dtype=np.float64)], dtype=np.float32)
    dz2 = (dy[:, None] * P["w3"][None, :] * gelu_grad(c["z2"])).astype(np.float32)
    dz2b = bf16(dz2).astype(np.float64)
    g["W2"] = (dz2b.T @ c["h1b"].astype(np.float64)).astype(np.float32)
    # bias gradients are sums of the BF16-rounded dZ (the kernels form them
    # with the same tensor-core product as the weight gradients)
    g["b2"] = dz2b.sum(axis=0).astype(np.float32)
    dh1 = (dz2b @ bf16(P["W2"]).astype(np.float64)).astype(np.float32)
    dz1 = (dh1 * gelu_grad(c["z1"])).astype(np.float32)
    dz1b = bf16(dz1).astype(np.float64)
    g["W1"] = (dz1b.T @ c["xb"]).astype(np.float32)
    g["b1"] = dz1b.sum(axis=0).astype(np.float32)
    return loss, pack(g)


def adam(p, g, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (t counts from 1); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return (p - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32), m, v

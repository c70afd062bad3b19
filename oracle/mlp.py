"""Oracle (test infrastructure only): the learned warm start's MLP restated in numpy.

Mirrors the GPU kernels' arithmetic: bf16 rounding (round to nearest even) of the normalised inputs,
the weights and the hidden activations, f32 accumulation, ReLU; the loss is the mean over rows of
the squared error summed over the two outputs; backward rounds dy, dh2 and dh1 to bf16 where the
GPU feeds them to the tensor cores and keeps the bias gradients in f32. Also a float64 reference
without any rounding, and Adam. Parameter layout: W1 [64][16], b1 [64], W2 [64][64], b2 [64],
W3 [8][64], b3 [8].
"""
from __future__ import annotations

import numpy as np

N_IN, N_PAD, H, N_OUT, OUT_PAD = 14, 16, 64, 2, 8
SHAPES = [("W1", (H, N_PAD)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (OUT_PAD, H)), ("b3", (OUT_PAD,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    """Named parameter arrays (float64 when p is float64, else float32)."""
    p = np.asarray(p)
    dt = np.float64 if p.dtype == np.float64 else np.float32
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=dt).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float32).reshape(-1) for name, _ in SHAPES])


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = rounded.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


def normalise(x, mu, sigma):
    xn = np.zeros((len(x), N_PAD), dtype=np.float32)
    xn[:, :N_IN] = (np.asarray(x, dtype=np.float32) - mu.astype(np.float32)) / sigma.astype(np.float32)
    return xn


def forward(p, x, mu, sigma):
    w = unpack(p)
    xb = bf16(normalise(x, mu, sigma))
    z1 = xb @ bf16(w["W1"]).T + w["b1"]
    h1 = bf16(np.maximum(z1, 0.0))
    z2 = h1 @ bf16(w["W2"]).T + w["b2"]
    h2 = bf16(np.maximum(z2, 0.0))
    y = h2 @ bf16(w["W3"]).T + w["b3"]
    return y[:, :N_OUT].astype(np.float32), (xb, z1, h1, z2, h2)


def gradients(p, x, t, mu, sigma):
    """(loss, gradient in the parameter layout) with the GPU's rounding points."""
    w = unpack(p)
    y, (xb, z1, h1, z2, h2) = forward(p, x, mu, sigma)
    n = len(x)
    e = y - t
    loss = float((e.astype(np.float64) ** 2).sum() / n)
    dy = np.zeros((n, OUT_PAD), dtype=np.float32)
    dy[:, :N_OUT] = 2.0 * e / n
    g = {}
    g["b3"] = dy.sum(axis=0)
    g["W3"] = bf16(dy).T @ h2
    d2 = (dy[:, :N_OUT] @ bf16(w["W3"])[:N_OUT]) * (z2 > 0)
    g["b2"] = d2.sum(axis=0)
    d2b = bf16(d2)
    g["W2"] = d2b.T @ h1
    d1 = (d2b @ bf16(w["W2"])) * (h1 > 0)
    g["b1"] = d1.sum(axis=0)
    g["W1"] = bf16(d1).T @ xb
    g["W1"][:, N_IN:] = 0.0
    g["W3"][N_OUT:] = 0.0
    g["b3"][N_OUT:] = 0.0
    return loss, pack(g)


def gradients_exact(p, x, t, mu, sigma):
    """float64 loss and gradient with no rounding anywhere (the true gradient of the f64 network)."""
    w = {k: v.astype(np.float64) for k, v in unpack(p).items()}
    xn = normalise(x, mu, sigma).astype(np.float64)
    z1 = xn @ w["W1"].T + w["b1"]
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = np.maximum(z2, 0.0)
    y = (h2 @ w["W3"].T + w["b3"])[:, :N_OUT]
    n = len(x)
    e = y - t
    dy = np.zeros((n, OUT_PAD))
    dy[:, :N_OUT] = 2.0 * e / n
    g = {"b3": dy.sum(0), "W3": dy.T @ h2}
    d2 = (dy @ w["W3"]) * (z2 > 0)
    g["b2"], g["W2"] = d2.sum(0), d2.T @ h1
    d1 = (d2 @ w["W2"]) * (z1 > 0)
    g["b1"], g["W1"] = d1.sum(0), d1.T @ xn
    g["W1"][:, N_IN:] = 0.0
    g["W3"][N_OUT:] = 0.0
    g["b3"][N_OUT:] = 0.0
    return float((e ** 2).sum() / n), np.concatenate([g[k].reshape(-1) for k, _ in SHAPES])


def loss_f64(p, x, t, mu, sigma):
    return gradients_exact(p, x, t, mu, sigma)[0]

"""float64 NumPy restatement of the radius model, used to check the GPU forward and backward
kernels: inputs scaled to [0,1]^D, sin/cos of 32 fixed random projections (Fourier features),
then 64 -> 64 -> 1 with ReLU; loss = mean squared error on the log k-th distance.
Parameter layout: W1[64][E] b1[64] W2[64][64] b2[64] w3[64] b3 | B[D][32] lo[D] inv_range[D]
margin, with E = D + 64."""

import numpy as np

H = 64
F = 32


def split(params, d):
    p = np.asarray(params, np.float64)
    e = d + 2 * F
    o = 0
    out = {}
    for name, shape in (("W1", (H, e)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("w3", (H,)), ("b3", ())):
        size = int(np.prod(shape)) if shape else 1
        out[name] = p[o:o + size].reshape(shape) if shape else p[o]
        o += size
    out["trainable"] = o
    out["B"] = p[o:o + d * F].reshape(d, F)
    o += d * F
    out["lo"] = p[o:o + d]
    out["inv_range"] = p[o + d:o + 2 * d]
    out["margin"] = p[o + 2 * d]
    return out


def features(m, x):
    z = (np.asarray(x, np.float64) - m["lo"]) * m["inv_range"]
    a = 2 * np.pi * (z @ m["B"])
    return np.concatenate([z, np.sin(a), np.cos(a)], axis=1)


def loss_and_grad(params, d, x, t):
    m = split(params, d)
    e = features(m, x)
    a1 = e @ m["W1"].T + m["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ m["W2"].T + m["b2"]
    h2 = np.maximum(a2, 0)
    y = h2 @ m["w3"] + m["b3"]
    n = len(t)
    err = y - np.asarray(t, np.float64)
    loss = np.sum(err * err) / n
    dy = 2 * err / n
    d2 = np.outer(dy, m["w3"]) * (a2 > 0)
    d1 = (d2 @ m["W2"]) * (a1 > 0)
    grad = np.concatenate([(d1.T @ e).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), h2.T @ dy, [dy.sum()]])
    return loss, grad


def predict(params, d, x):
    m = split(params, d)
    e = features(m, x)
    h1 = np.maximum(e @ m["W1"].T + m["b1"], 0)
    h2 = np.maximum(h1 @ m["W2"].T + m["b2"], 0)
    return h2 @ m["w3"] + m["b3"]

"""float64 NumPy restatement of the radius model (D -> 64 -> 64 -> 1, ReLU, MSE on the log
k-th distance) used to check the GPU forward and backward kernels.  Parameter layout:
W1[64][D] b1[64] W2[64][64] b2[64] w3[64] b3 | mu[D] inv_sd[D] margin."""

import numpy as np

H = 64


def split(params, d):
    p = np.asarray(params, np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (H, d)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("w3", (H,)), ("b3", ())):
        size = int(np.prod(shape)) if shape else 1
        out[name] = p[o:o + size].reshape(shape) if shape else p[o]
        o += size
    out["trainable"] = o
    out["mu"] = p[o:o + d]
    out["inv_sd"] = p[o + d:o + 2 * d]
    out["margin"] = p[o + 2 * d]
    return out


def loss_and_grad(params, d, x, t):
    m = split(params, d)
    xn = (np.asarray(x, np.float64) - m["mu"]) * m["inv_sd"]
    a1 = xn @ m["W1"].T + m["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ m["W2"].T + m["b2"]
    h2 = np.maximum(a2, 0)
    y = h2 @ m["w3"] + m["b3"]
    n = len(t)
    err = y - np.asarray(t, np.float64)
    loss = np.sum(err * err) / n
    dy = 2 * err / n
    g_w3 = h2.T @ dy
    g_b3 = dy.sum()
    d2 = np.outer(dy, m["w3"]) * (a2 > 0)
    g_W2 = d2.T @ h1
    g_b2 = d2.sum(0)
    d1 = (d2 @ m["W2"]) * (a1 > 0)
    g_W1 = d1.T @ xn
    g_b1 = d1.sum(0)
    grad = np.concatenate([g_W1.ravel(), g_b1, g_W2.ravel(), g_b2, g_w3, [g_b3]])
    return loss, grad


def predict(params, d, x):
    m = split(params, d)
    xn = (np.asarray(x, np.float64) - m["mu"]) * m["inv_sd"]
    h1 = np.maximum(xn @ m["W1"].T + m["b1"], 0)
    h2 = np.maximum(h1 @ m["W2"].T + m["b2"], 0)
    return h2 @ m["w3"] + m["b3"]

"""CPU oracle of the warm-start set encoder (forward, loss, gradient, Adam).

TEST INFRASTRUCTURE ONLY: the tests compare the GPU kernels of
sv_encoder.cu with this restatement; the product package never imports it.
The encoder has no reference counterpart (it only moves the starting point of
gp.py:169-177), so this oracle restates the network's own definition:

    h1 = bf16(GELU(W1 x + b1)),  h2 = GELU(W2 h1 + b2),  pool = mean h2
    g = GELU(W3 pool + b3),      out = W4 g + b4,  loss = sum w (out - t)^2

in float64, with the weights and inputs rounded to bfloat16 exactly as the
kernels read them (float32 -> bfloat16, round to nearest even), h1 rounded
to bfloat16 as the kernels store it, and the backward's GEMM operands dz2 and
dz1 rounded to bfloat16 as the kernels feed them to the tensor cores (the
bias gradients use the unrounded values, as the kernels do).  What remains
between the two is float32 accumulation order and the float32 GELU, so the
comparisons use relative tolerances of ~1e-3 on whole gradient blocks.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

H, F, O = 128, 32, 16
LAYOUT = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)),
          ("b3", (H,)), ("W4", (O, H)), ("b4", (O,))]


def unflatten(p):
    out, o = {}, 0
    for name, shp in LAYOUT:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def flatten(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in LAYOUT])


def bf16(a):
    """float32 -> bfloat16 (round to nearest even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(a, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    r = ((f + 0x7FFF + ((f >> 16) & 1)) >> 16) << 16
    return (r.astype(np.uint32)).view(np.float32).astype(np.float64)


def pack(features):
    """The kernels' input rounding: float64 -> float32 -> bfloat16."""
    return bf16(np.asarray(features, dtype=np.float64).astype(np.float32))


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def _ident(a):
    return np.asarray(a, dtype=np.float64)


def forward(p32, x, cnt, keep=False, rounding=True):
    """p32: flat float32 parameters; x: (nset, S, 16) bfloat16 values
    (as float64); cnt: points per set.  Returns out (nset, 16).
    rounding=False drops every bfloat16 rounding (the exact float64 network,
    used to check the chain rule itself by finite differences)."""
    r16 = bf16 if rounding else _ident
    P = unflatten(np.asarray(p32, dtype=np.float32) if rounding else np.asarray(p32, dtype=np.float64))
    W = {k: (r16(v) if k.startswith("W") else v) for k, v in P.items()}
    outs, saved = [], []
    for b in range(x.shape[0]):
        xs = x[b, :int(cnt[b])]
        z1 = xs @ W["W1"].T + W["b1"]
        h1 = r16(gelu(z1))
        z2 = h1 @ W["W2"].T + W["b2"]
        h2 = gelu(z2)
        pool = h2.mean(0)
        zg = W["W3"] @ pool + W["b3"]
        g = gelu(zg)
        outs.append(W["W4"] @ g + W["b4"])
        saved.append((xs, z1, h1, z2, pool, zg, g))
    out = np.array(outs)
    return (out, saved, W) if keep else out


def loss_and_grad(p32, x, cnt, target, wts, rounding=True):
    r16 = bf16 if rounding else _ident
    out, saved, W = forward(p32, x, cnt, keep=True, rounding=rounding)
    r = out - target
    loss = float(np.sum(wts * r * r))
    G = {name: np.zeros(shp) for name, shp in LAYOUT}
    for b, (xs, z1, h1, z2, pool, zg, g) in enumerate(saved):
        dout = 2.0 * wts[b] * r[b]
        G["W4"] += np.outer(dout, g)
        G["b4"] += dout
        dzg = (W["W4"].T @ dout) * gelu_d(zg)
        G["W3"] += np.outer(dzg, pool)
        G["b3"] += dzg
        dpool = W["W3"].T @ dzg
        c = xs.shape[0]
        dz2 = (dpool / c)[None, :] * gelu_d(z2)
        G["b2"] += dz2.sum(0)
        dz2r = r16(dz2)
        G["W2"] += dz2r.T @ h1
        dh1 = dz2r @ W["W2"]
        dz1 = dh1 * gelu_d(z1)
        G["b1"] += dz1.sum(0)
        G["W1"] += r16(dz1).T @ xs
    return loss, out, flatten(G)


def adam(p, g, m, v, lr, b1, b2, eps, step, wd):
    g = g + wd * p
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v

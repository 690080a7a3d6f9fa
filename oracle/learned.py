"""CPU reference of the learned warm-start network -- TEST INFRASTRUCTURE ONLY.

The network has no counterpart in the reference.  This numpy restatement is the
checker for the GPU forward and backward kernels (movfem_gb300/csrc/mvf_learn.cu).
It follows the same rounding points: the input, the weights and every hidden
activation are rounded to BF16 (round to nearest even), and the last layer's output
stays unrounded.  Sums run in float64, so the GPU's FP32 accumulation is the only
difference left.

Layout: grids [X][Y][Z][C]; parameters layer by layer, weights [k^3][cin][cout] then
bias [cout]; a 3x3x3 convolution with dilation d reads in[v + (t - 1) * d] with zero
padding; ReLU after every 3x3x3 layer, none after the final 1x1x1 layer.
"""
from __future__ import annotations

import numpy as np


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def layers(cin, width, cout, dilations):
    """[(cin, cout, ks, dil, relu, woff, boff)] and the parameter count."""
    out, off, c = [], 0, cin
    for li in range(len(dilations) + 1):
        hidden = li < len(dilations)
        co = width if hidden else cout
        ks = 3 if hidden else 1
        woff = off
        off += ks ** 3 * c * co
        out.append((c, co, ks, dilations[li] if hidden else 1, hidden, woff, off))
        off += co
        c = co
    return out, off


def _shift(a, di, dj, dk):
    """b[v] = a[v + (di, dj, dk)] with zeros outside."""
    X, Y, Z = a.shape[:3]
    b = np.zeros_like(a)
    xs, xd = slice(max(di, 0), X + min(di, 0)), slice(max(-di, 0), X + min(-di, 0))
    ys, yd = slice(max(dj, 0), Y + min(dj, 0)), slice(max(-dj, 0), Y + min(-dj, 0))
    zs, zd = slice(max(dk, 0), Z + min(dk, 0)), slice(max(-dk, 0), Z + min(-dk, 0))
    b[xd, yd, zd] = a[xs, ys, zs]
    return b


def _offsets(ks, dil):
    h = ks // 2
    return [((t // (ks * ks) - h) * dil, ((t // ks) % ks - h) * dil, (t % ks - h) * dil) for t in range(ks ** 3)]


def forward(params, x, cin, width, cout, dilations, rounding=True):
    """Activations [input, hidden..., output]; hidden ones BF16-rounded (unless
    ``rounding`` is off: plain float64, for finite-difference checks)."""
    L, _ = layers(cin, width, cout, dilations)
    rnd = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    p = np.asarray(params, dtype=np.float32 if rounding else np.float64)
    acts = [rnd(x)]
    for (ci, co, ks, dil, relu, woff, boff) in L:
        W = rnd(p[woff:boff]).reshape(ks ** 3, ci, co)
        b = p[boff:boff + co].astype(np.float64)
        a = acts[-1]
        out = np.zeros(a.shape[:3] + (co,)) + b
        for t, (di, dj, dk) in enumerate(_offsets(ks, dil)):
            out += _shift(a, di, dj, dk) @ W[t]
        if relu:
            out = rnd(np.maximum(out, 0.0))
        acts.append(out)
    return acts


def loss_and_grad(params, x, target, cin, width, cout, dilations, rounding=True):
    """Mean squared error and its gradient with respect to the parameters."""
    L, n = layers(cin, width, cout, dilations)
    rnd = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    p = np.asarray(params, dtype=np.float32 if rounding else np.float64)
    acts = forward(params, x, cin, width, cout, dilations, rounding)
    out = acts[-1]
    d = out - np.asarray(target, dtype=np.float64)
    loss = float(np.mean(d * d))
    g = 2.0 * d / d.size
    grad = np.zeros(n)
    for li in range(len(L) - 1, -1, -1):
        ci, co, ks, dil, relu, woff, boff = L[li]
        W = rnd(p[woff:boff]).reshape(ks ** 3, ci, co)
        a = acts[li]
        offs = _offsets(ks, dil)
        gw = np.zeros((ks ** 3, ci, co))
        for t, (di, dj, dk) in enumerate(offs):
            gw[t] = np.einsum("xyzc,xyzd->cd", _shift(a, di, dj, dk), g)
        grad[woff:boff] = gw.ravel()
        grad[boff:boff + co] = g.sum(axis=(0, 1, 2))
        if li > 0:
            gin = np.zeros(a.shape)
            for t, (di, dj, dk) in enumerate(offs):
                gin += _shift(g @ W[t].T, -di, -dj, -dk)
            if L[li - 1][4]:
                gin *= a > 0
            g = gin
    return loss, grad

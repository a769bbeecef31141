"""CPU oracle for the learned surrogate's network — TEST INFRASTRUCTURE ONLY.
Only tests/ may import this module; the product never does.

The surrogate has no counterpart in the reference: it is a learned form
added on top of the plain layered angular-spectrum method
(HologramGenerator_GPU.cpp:246-302), which produces its training targets and
judges it.  This file states its mathematics in float64 numpy, in the same
NHWC layouts the CUDA kernels use:

  conv3x3 (zero padding 1) / conv1x1, bias, ReLU
  2x2 average pooling, nearest 2x upsampling, channel concatenation
  the 4-level U-Net: encoder level l = conv-ReLU-conv-ReLU (c_l channels),
  pooling between levels; decoder level l = upsample the level below,
  concatenate [encoder_l, upsampled], conv-ReLU-conv-ReLU; 1x1 head to 2
  channels; loss = mean over pixels and channels of (pred - target)^2
  and the exact backward pass of all of it.

Weights are [cout][taps][cin] (tap = 3 * (dy + 1) + (dx + 1)); weight
gradients are returned in the same layout.
"""
from __future__ import annotations

import numpy as np

OFFS = [(dy, dx) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def shift(x, dy, dx):
    """y[n, i, j] = x[n, i + dy, j + dx] with zeros outside (NHWC)."""
    n, h, w, c = x.shape
    y = np.zeros_like(x)
    ys0, ys1 = max(0, -dy), min(h, h - dy)
    xs0, xs1 = max(0, -dx), min(w, w - dx)
    if ys1 > ys0 and xs1 > xs0:
        y[:, ys0:ys1, xs0:xs1] = x[:, ys0 + dy:ys1 + dy, xs0 + dx:xs1 + dx]
    return y


def conv(x, w, b=None, relu=False):
    """x [n,h,w,cin], w [cout,taps,cin] (taps 9 or 1) -> [n,h,w,cout]."""
    taps = w.shape[1]
    offs = OFFS if taps == 9 else [(0, 0)]
    y = np.zeros(x.shape[:3] + (w.shape[0],), dtype=np.float64)
    for t, (dy, dx) in enumerate(offs):
        y += shift(x, dy, dx) @ w[:, t, :].T
    if b is not None:
        y += b
    return np.maximum(y, 0.0) if relu else y


def conv_dgrad(dz, w):
    """Gradient with respect to the input: dx[p] = sum_t dz[p - off_t] W_t."""
    taps = w.shape[1]
    offs = OFFS if taps == 9 else [(0, 0)]
    dx = np.zeros(dz.shape[:3] + (w.shape[2],), dtype=np.float64)
    for t, (dy, ddx) in enumerate(offs):
        dx += shift(dz, -dy, -ddx) @ w[:, t, :]
    return dx


def conv_wgrad(x, dz, taps=9):
    """dW[co, t, ci] = sum_p dz[p, co] x[p + off_t, ci]."""
    offs = OFFS if taps == 9 else [(0, 0)]
    cin, cout = x.shape[3], dz.shape[3]
    dw = np.zeros((cout, taps, cin), dtype=np.float64)
    d2 = dz.reshape(-1, cout)
    for t, (dy, dx) in enumerate(offs):
        dw[:, t, :] = d2.T @ shift(x, dy, dx).reshape(-1, cin)
    return dw


def pool(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def pool_back(d):
    return np.repeat(np.repeat(d, 2, axis=1), 2, axis=2) / 4.0


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_back(d):
    n, h, w, c = d.shape
    return d.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def layer_shapes(in_ch=4, chans=(32, 64, 128, 256), out_ch=2):
    """(name, cin, cout, taps) of every layer, in parameter order."""
    L = []
    c_prev = in_ch
    for l, c in enumerate(chans):
        L.append((f"enc{l}a", c_prev, c, 9))
        L.append((f"enc{l}b", c, c, 9))
        c_prev = c
    for l in range(len(chans) - 2, -1, -1):
        L.append((f"dec{l}a", chans[l] + chans[l + 1], chans[l], 9))
        L.append((f"dec{l}b", chans[l], chans[l], 9))
    L.append(("head", chans[0], out_ch, 1))
    return L


def _same(a):
    return a


def forward(params, x, chans=(32, 64, 128, 256), rnd=_same):
    """params: dict name -> (W [cout,taps,cin], b [cout]).  Returns (pred, cache).
    rnd is applied to every stored activation (identity: exact float64;
    a BF16 rounding function: the storage precision of the CUDA kernels)."""
    cache = {}
    h = x
    enc = []
    for l in range(len(chans)):
        a = rnd(conv(h, *params[f"enc{l}a"], relu=True))
        e = rnd(conv(a, *params[f"enc{l}b"], relu=True))
        cache[f"enc{l}a_in"], cache[f"enc{l}a_out"], cache[f"enc{l}b_out"] = h, a, e
        enc.append(e)
        if l + 1 < len(chans):
            h = rnd(pool(e))
    d = enc[-1]
    for l in range(len(chans) - 2, -1, -1):
        cat = np.concatenate([enc[l], up(d)], axis=3)
        a = rnd(conv(cat, *params[f"dec{l}a"], relu=True))
        d = rnd(conv(a, *params[f"dec{l}b"], relu=True))
        cache[f"dec{l}a_in"], cache[f"dec{l}a_out"], cache[f"dec{l}b_out"] = cat, a, d
    pred = conv(d, *params["head"])
    cache["head_in"] = d
    return pred, cache


def loss_and_grads(params, x, target, chans=(32, 64, 128, 256), rnd=_same):
    """Mean squared error over all pixels and output channels, the gradient
    of every weight and bias (dict name -> (dW, db)) and the prediction.
    rnd: as in forward, applied to the stored activations and activation
    gradients (weight and bias gradients stay unrounded)."""
    pred, c = forward(params, x, chans, rnd)
    diff = pred - target
    loss = float(np.mean(diff ** 2))
    dpred = 2.0 * diff / diff.size
    return loss, backward(params, c, dpred, chans, rnd), pred


def backward(params, c, dpred, chans=(32, 64, 128, 256), rnd=_same):
    """Gradients of every layer given d(loss)/d(pred) and the forward cache."""
    nlev = len(chans)
    g = {}
    Wh, _ = params["head"]
    g["head"] = (conv_wgrad(c["head_in"], dpred, 1), dpred.sum(axis=(0, 1, 2)))
    dd = conv_dgrad(dpred, Wh)          # d(output of dec0b)
    dz_b = rnd(dd * (c["dec0b_out"] > 0))
    denc = [None] * nlev
    # decoder levels from 0 (top, last computed) to nlev-2; dz_b is the
    # gradient of dec{l}b's pre-activation
    for l in range(0, nlev - 1):
        g[f"dec{l}b"] = (conv_wgrad(c[f"dec{l}a_out"], dz_b), dz_b.sum(axis=(0, 1, 2)))
        dz_a = rnd(conv_dgrad(dz_b, params[f"dec{l}b"][0]) * (c[f"dec{l}a_out"] > 0))
        g[f"dec{l}a"] = (conv_wgrad(c[f"dec{l}a_in"], dz_a), dz_a.sum(axis=(0, 1, 2)))
        dcat = rnd(conv_dgrad(dz_a, params[f"dec{l}a"][0]))
        denc[l] = dcat[..., :chans[l]]
        below = c[f"dec{l + 1}b_out"] if l + 1 < nlev - 1 else c[f"enc{nlev - 1}b_out"]
        dz_b = rnd(up_back(dcat[..., chans[l]:]) * (below > 0))
    # encoder from the bottleneck up; dz_b is the gradient of enc{l}b's pre-activation
    for l in range(nlev - 1, -1, -1):
        if l < nlev - 1:
            dz_b = rnd((denc[l] + pool_back(dpool)) * (c[f"enc{l}b_out"] > 0))
        g[f"enc{l}b"] = (conv_wgrad(c[f"enc{l}a_out"], dz_b), dz_b.sum(axis=(0, 1, 2)))
        dz_a = rnd(conv_dgrad(dz_b, params[f"enc{l}b"][0]) * (c[f"enc{l}a_out"] > 0))
        g[f"enc{l}a"] = (conv_wgrad(c[f"enc{l}a_in"], dz_a), dz_a.sum(axis=(0, 1, 2)))
        if l > 0:
            dpool = rnd(conv_dgrad(dz_a, params[f"enc{l}a"][0]))   # d(pooled input of level l)
    return g

"""CPU FP64 oracle for the learned preconditioner's layers — TEST
INFRASTRUCTURE ONLY.

Written from the definitions (no reference counterpart exists: Jet has no
learned components). Layout matches the GPU kernels: activations
channels-last (nz, ny, nx, C); weights w[tap, co, ci] with
tap = (dz+1)*9 + (dy+1)*3 + (dx+1); 3x3x3 convolution, stride 1, zero
padding 1.
"""
from __future__ import annotations

import numpy as np


def _taps():
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                yield (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1), dz, dy, dx


def _shift(x, dz, dy, dx):
    """y[k, j, i] = x[k+dz, j+dy, i+dx] with zeros outside."""
    nz, ny, nx = x.shape[:3]
    y = np.zeros_like(x)
    zs = slice(max(0, -dz), nz - max(0, dz))
    ys = slice(max(0, -dy), ny - max(0, dy))
    xs = slice(max(0, -dx), nx - max(0, dx))
    zd = slice(max(0, dz), nz - max(0, -dz))
    yd = slice(max(0, dy), ny - max(0, -dy))
    xd = slice(max(0, dx), nx - max(0, -dx))
    y[zs, ys, xs] = x[zd, yd, xd]
    return y


def conv3d(x, w, bias=None, relu=False):
    """x: (nz, ny, nx, ci); w: (27, co, ci) -> (nz, ny, nx, co), FP64."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    out = np.zeros(x.shape[:3] + (w.shape[1],))
    for t, dz, dy, dx in _taps():
        out += _shift(x, dz, dy, dx) @ w[t].T
    if bias is not None:
        out += np.asarray(bias, np.float64)
    if relu:
        out = np.maximum(out, 0.0)
    return out


def conv3d_dgrad(dy, w):
    """Gradient of conv3d (no bias/activation) w.r.t. its input."""
    dy = np.asarray(dy, np.float64)
    w = np.asarray(w, np.float64)
    dx = np.zeros(dy.shape[:3] + (w.shape[2],))
    for t, dz, dyy, dxx in _taps():
        dx += _shift(dy, -dz, -dyy, -dxx) @ w[t]
    return dx


def conv3d_wgrad(x, dy):
    """Gradient w.r.t. w[tap, co, ci]."""
    x = np.asarray(x, np.float64)
    dy = np.asarray(dy, np.float64)
    co, ci = dy.shape[3], x.shape[3]
    dw = np.zeros((27, co, ci))
    for t, dz, dyy, dxx in _taps():
        xs = _shift(x, dz, dyy, dxx).reshape(-1, ci)
        dw[t] = dy.reshape(-1, co).T @ xs
    return dw


def bf16_round(a):
    """Round FP32 values to BF16 (round to nearest even), returned as FP32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)

"""FP64 restatement of the veiling-glare layer (TEST INFRASTRUCTURE ONLY).

Follows render_veil (veil_render.cu:243-414): bake g(r) = (a^2/(r^2+a^2))^p
on a 1024^2 grid with a = 1024/32 texels (:94-105), normalise to unit sum
(:339-352), box-sum downsample by the largest power of two <= pitch / (3
texels) capped at 128 (:357-373), then area-weighted resample per output pixel
within the footprint (:170-231, :386-396).  The reference's renderer is
GPU-only, so this restatement is the pin ("parity unpinned" against the
reference's own numbers).
"""
from __future__ import annotations

import math

import numpy as np


def sprite(falloff: float, N: int = 1024):
    p = min(max(falloff if falloff >= 1.0 else 1.0, 1.0), 3.0)
    a = N / 32.0
    j, i = np.mgrid[0:N, 0:N].astype(np.float64)
    g = (a * a / ((i - N // 2) ** 2 + (j - N // 2) ** 2 + a * a)) ** p
    return g / g.sum()


def render(sources, width, height, hw, hh, spread=0.12, falloff=1.5, gain=0.03, fmt=None):
    """(3, H, W) float64; sources (N, 5) [px, py, r, g, b]."""
    N = 1024
    fw, fh = (width, height) if fmt is None else fmt
    half_ref = hh if hh > 0 else hw
    sp = spread if spread > 0 else 0.12
    sp = min(max(sp, 1e-3), 4.0)
    a_tex = N / 32.0
    dx = sp * half_ref / a_tex
    pxx, pxy = 2 * hw / fw, 2 * hh / fh
    target = min(pxx / (dx * 3), pxy / (dx * 3))
    ds = 1
    while ds * 2 <= target and ds * 2 <= N // 8:
        ds *= 2
    M = N // ds
    S = sprite(falloff, N).reshape(M, ds, M, ds).sum(axis=(1, 3))
    sxd = dx * ds
    rx = min(int(math.ceil(0.5 * M * sxd / pxx)) + 1, width)
    ry = min(int(math.ceil(0.5 * M * sxd / pxy)) + 1, height)
    out = np.zeros((3, height, width))
    # prefix sums of the sprite for exact area integrals of the piecewise-constant texels
    for (px, py, r, g, b) in np.asarray(sources, np.float64).reshape(-1, 5):
        cx, cy = int(math.floor(px)), int(math.floor(py))
        xs = np.arange(max(0, cx - rx), min(width, cx + rx + 1))
        ys = np.arange(max(0, cy - ry), min(height, cy + ry + 1))
        xlo = (xs - px) * pxx / sxd + 0.5 * M
        xhi = (xs + 1 - px) * pxx / sxd + 0.5 * M
        ylo = (ys - py) * pxy / sxd + 0.5 * M
        yhi = (ys + 1 - py) * pxy / sxd + 0.5 * M
        # overlap of each pixel span with each texel [i, i+1)
        ti = np.arange(M)
        wx = np.clip(np.minimum(xhi[:, None], ti[None, :] + 1) - np.maximum(xlo[:, None], ti[None, :]), 0, None)
        wy = np.clip(np.minimum(yhi[:, None], ti[None, :] + 1) - np.maximum(ylo[:, None], ti[None, :]), 0, None)
        v = wy @ S @ wx.T                                   # (len(ys), len(xs))
        for c, col in enumerate((r, g, b)):
            out[c][np.ix_(ys, xs)] += v * col * gain
    return out

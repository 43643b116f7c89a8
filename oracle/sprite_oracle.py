"""FP64 restatement of the reference's SPRITE starburst engine.

TEST INFRASTRUCTURE ONLY — imported by tests/; never by the product.

Follows render_starburst's sprite path (JaydenB/ghostlight,
ghostlight/src/starburst_render.cu:969-1073) step by step in float64 numpy:
  psf_from_fft_kernel (:202)   |FFT(pupil)|^2, DC moved to the grid centre
  reduce + scale (:1003-1006)  normalised to unit sum
  bake_sprite_kernel (:255)    sum_l cmf_l PSF(c + d lambda_ref/lambda_l) (lambda_ref/lambda_l)^2,
                               bilinear (bilinear_psf :240), zero outside
  downsample_kernel (:283)     ds x ds box sum
  splat_resample_kernel (:316) per output pixel, the area-weighted integral of
                               the sprite over the pixel's footprint, x colour x gain
The reference's own code for this path is CUDA with cuFFT and cannot run on
the host, so this restatement is the pin for the device engine.
"""
from __future__ import annotations

import numpy as np


def psf(pupil):
    """(N, N) PSF, DC at (N/2, N/2), unnormalised."""
    F = np.fft.fft2(np.asarray(pupil, np.float64))
    return np.fft.fftshift(np.abs(F) ** 2)


def _bilinear(p, fx, fy):
    N = p.shape[0]
    ok = (fx >= 0) & (fy >= 0) & (fx < N - 1) & (fy < N - 1)
    x0 = np.where(ok, np.floor(fx), 0).astype(np.int64)
    y0 = np.where(ok, np.floor(fy), 0).astype(np.int64)
    tx, ty = fx - x0, fy - y0
    a = p[y0, x0] * (1 - tx) + p[y0, x0 + 1] * tx
    b = p[y0 + 1, x0] * (1 - tx) + p[y0 + 1, x0 + 1] * tx
    return np.where(ok, a * (1 - ty) + b * ty, 0.0)


def sprite(pupil, spec, ds, lambda_ref=550.0):
    """(M, M, 3) sprite, M = N / ds, from the pupil amplitude and the
    spectral table (n, 4) [lambda, cmf_r, cmf_g, cmf_b]."""
    P = psf(pupil)
    P = P / P.sum()
    N = P.shape[0]
    idx = np.arange(N, dtype=np.float64) - N // 2
    dx, dy = np.meshgrid(idx, idx)
    half = float(N // 2)
    out = np.zeros((N, N, 3))
    for lam, cr, cg, cb in np.asarray(spec, np.float64):
        k = lambda_ref / lam
        v = _bilinear(P, half + dx * k, half + dy * k) * k * k
        out[..., 0] += cr * v
        out[..., 1] += cg * v
        out[..., 2] += cb * v
    M = N // ds
    return out.reshape(M, ds, M, ds, 3).sum(axis=(1, 3))


def _overlap(lo, hi, M):
    """(len(lo), M) overlap of [lo, hi) with the texel cells [i, i+1)."""
    i = np.arange(M, dtype=np.float64)[None, :]
    return np.clip(np.minimum(hi[:, None], i + 1) - np.maximum(lo[:, None], i), 0.0, None)


def splat(spr, sources, sx_ds, sy_ds, px_mm_x, px_mm_y, rx, ry, gain, width, height):
    """(3, H, W) float64: every source's area-weighted resample of the sprite
    over the pixels of its footprint (2 rx + 1) x (2 ry + 1)."""
    M = spr.shape[0]
    out = np.zeros((3, height, width))
    for px, py, r, g, b in np.asarray(sources, np.float64).reshape(-1, 5):
        cx, cy = int(np.floor(np.float32(px))), int(np.floor(np.float32(py)))
        xs = np.arange(max(cx - rx, 0), min(cx + rx, width - 1) + 1)
        ys = np.arange(max(cy - ry, 0), min(cy + ry, height - 1) + 1)
        if len(xs) == 0 or len(ys) == 0:
            continue
        xlo = (xs - px) * px_mm_x / sx_ds + 0.5 * M
        xhi = (xs + 1.0 - px) * px_mm_x / sx_ds + 0.5 * M
        ylo = (ys - py) * px_mm_y / sy_ds + 0.5 * M
        yhi = (ys + 1.0 - py) * px_mm_y / sy_ds + 0.5 * M
        Wx, Wy = _overlap(xlo, xhi, M), _overlap(ylo, yhi, M)
        for c, w in enumerate((r, g, b)):
            out[c][np.ix_(ys, xs)] += (Wy @ spr[..., c] @ Wx.T) * w * gain
    return out

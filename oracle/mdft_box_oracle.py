"""FP64 restatement of the reference's matrix-DFT starburst engine.

TEST INFRASTRUCTURE ONLY (the parity reference of the device form; nothing
in the product imports it).  It follows ghostlight/src/mdft_render.cu:199-340:

1. C, the compact pupil autocorrelation: G = fft2(|fft2(A)|^2), the lags
   |l| <= mc = ceil(fill N) + 4 (:233-235) read at (l mod N), conjugated
   and scaled by 1 / (G[0,0] N^2) (:249-262), so the pattern sums to one
   texel area over a period;
2. per source and wavelength (:295-327) the exact pixel-box integral of the
   intensity over the window of half a pattern period around the source
   (:275-279): I = Re(Py C Px), Px[b][k] = sinc(m px / S_l)
   exp(-2 pi i m xrel_k / S_l), m = b - mc, xrel_k = (k0 + k + 0.5 - src) px,
   S_l = N dx lambda / lambda_ref; accumulated with cmf (lambda_ref/lambda)^2;
3. the window times (px_x px_y) / (dx_x dx_y) x gain x source colour added
   into the frame (:177-196, :282-283).

Everything is evaluated in float64 (numpy FFT and matmul).
"""
from __future__ import annotations

import math

import numpy as np


def support_radius(N: int, pupil_fill: float) -> int:
    fill = pupil_fill if 0.02 < pupil_fill < 0.9 else 0.30
    mc = int(math.ceil(float(np.float32(fill)) * float(N))) + 4
    return min(mc, N // 2 - 1)


def autocorrelation(A, pupil_fill: float):
    """(C (Mc, Mc) complex128 with C[a][b], a the y lag and b the x lag, mc)."""
    A = np.asarray(A, np.float64)
    N = A.shape[0]
    mc = support_radius(N, pupil_fill)
    G = np.fft.fft2(np.abs(np.fft.fft2(A)) ** 2)
    idx = (np.arange(2 * mc + 1) - mc) % N
    g00 = G[0, 0].real
    if not g00 > 0.0:
        return None, mc
    return np.conj(G[np.ix_(idx, idx)]) / (g00 * N * N), mc


def window(src_px, half, size):
    k0 = max(0, int(math.floor(src_px)) - half)
    k1 = min(size, int(math.floor(src_px)) + half + 1)
    return k0, k1


def render(A, pupil_fill, spec, lambda_ref, dx_x, dx_y, px_mm_x, px_mm_y, sources, gain, width, height):
    """sources: (n, 5) [px, py, r, g, b] in buffer pixels; spec: (n_l, 4)
    [lambda, cmf_r, cmf_g, cmf_b].  Returns (3, H, W) float64."""
    out = np.zeros((3, height, width))
    C, mc = autocorrelation(A, pupil_fill)
    if C is None:
        return out
    N = np.asarray(A).shape[0]
    f = np.float32
    Sx, Sy = float(f(f(N) * f(dx_x))), float(f(f(N) * f(dx_y)))
    half_x = max(1, int(math.floor(0.5 * Sx / float(px_mm_x))))
    half_y = max(1, int(math.floor(0.5 * Sy / float(px_mm_y))))
    knorm_gain = (px_mm_x * px_mm_y) / (dx_x * dx_y) * gain
    m = np.arange(2 * mc + 1, dtype=np.float64) - mc
    for (px, py, r, g, b) in np.asarray(sources, np.float64).reshape(-1, 5):
        kx0, kx1 = window(px, half_x, width)
        ky0, ky1 = window(py, half_y, height)
        if kx1 <= kx0 or ky1 <= ky0:
            continue
        xr = (np.arange(kx0, kx1) + 0.5 - px) * px_mm_x
        yr = (np.arange(ky0, ky1) + 0.5 - py) * px_mm_y
        win = np.zeros((3, ky1 - ky0, kx1 - kx0))
        for lam, cr, cg, cb in np.asarray(spec, np.float64).reshape(-1, 4):
            Sxl, Syl = Sx * lam / lambda_ref, Sy * lam / lambda_ref
            k2 = (lambda_ref / lam) ** 2
            Px = np.sinc(m * px_mm_x / Sxl)[:, None] * np.exp(-2j * np.pi * np.outer(m, xr) / Sxl)
            Py = np.sinc(m * px_mm_y / Syl)[None, :] * np.exp(-2j * np.pi * np.outer(yr, m) / Syl)
            I = (Py @ (C @ Px)).real
            win += np.array([cr, cg, cb])[:, None, None] * k2 * I[None]
        out[:, ky0:ky1, kx0:kx1] += win * knorm_gain * np.array([r, g, b])[:, None, None]
    return out


def pupil(contains, N: int, pupil_fill: float):
    """The 4 x 4-supersampled stop amplitude (build_pupil_kernel,
    starburst_render.cu:155-191) given a vectorised point-in-stop test
    ``contains(uv (n, 2)) -> bool (n,)``."""
    fill = pupil_fill if 0.02 < pupil_fill < 0.9 else 0.30
    i = np.arange(N, dtype=np.float32)
    s = ((np.arange(4, dtype=np.float32) + np.float32(0.5)) * np.float32(0.25)).astype(np.float32)
    # coordinate of supersample s of texel i, in the reference's float order
    c = (((i[:, None] + s[None, :]) / np.float32(N) * np.float32(2.0) - np.float32(1.0)) /
         np.float32(fill)).astype(np.float32).reshape(-1)           # (N*4,)
    cnt = np.zeros((N, N))
    for sy in range(4):
        v = c.reshape(N, 4)[:, sy]
        for sx in range(4):
            u = c.reshape(N, 4)[:, sx]
            uu, vv = np.meshgrid(u, v, indexing="xy")               # (N rows = v, N cols = u)
            inside = contains(np.stack([uu.ravel(), vv.ravel()], 1)).reshape(N, N)
            cnt += inside
    return cnt / 16.0

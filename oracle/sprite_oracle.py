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


# ---- off-axis cat's-eye (starburst_render.cu:393-583), float launches, the
# oracle's float host trace (the reference's host arithmetic) ----------------
def _launch(ax, ay):
    f = np.float32
    bx, by = f(np.tan(f(ax))), f(np.tan(f(ay)))
    ln = f(np.sqrt(f(f(bx * bx) + f(by * by)) + f(1.0)))
    inv = f(f(1.0) / ln)
    return bx, by, (f(bx * inv), f(by * inv), inv)


def _survive(surfs, pts, z, d, lam=550.0):
    from oracle import oracle as O
    pts = np.asarray(pts, np.float32).reshape(-1, 2)
    if len(pts) == 0:
        return np.zeros(0, bool)
    rays = np.zeros((len(pts), 7), np.float32)
    rays[:, 0:2] = pts
    rays[:, 2] = z
    rays[:, 3:6] = d
    rays[:, 6] = lam
    r = O.trace(surfs, -1, -1, rays, fp64=False)
    return (r[:, 4] == 0) & np.isfinite(r[:, 0]) & np.isfinite(r[:, 1])


def survivor_center(surfs, ax, ay):
    """solve_survivor_center: (cx, cy, any)."""
    f = np.float32
    front_R = f(surfs[0].semi_aperture)
    if front_R <= 0:
        return 0.0, 0.0, False
    z = f(f(surfs[0].z) - f(20.0))
    bx, by, d = _launch(ax, ay)
    span_x = f(f(f(1.1) * front_R) + f(f(20.0) * f(abs(bx))))
    span_y = f(f(f(1.1) * front_R) + f(f(20.0) * f(abs(by))))
    S, K = 81, 8
    pos = lambda span, k: f(span * f(f(f(2.0) * f(k)) / f(S - 1) - f(1.0)))
    grid = [(pos(span_x, i), pos(span_y, j)) for j in range(S) for i in range(S)]
    surv = _survive(surfs, grid, z, d).reshape(S, S)
    hx, hy = f(span_x / f(S - 1)), f(span_y / f(S - 1))
    inv_k2 = f(f(1.0) / f(K * K))
    sx = sy = w = 0.0
    pending = []
    for j in range(S):
        for i in range(S):
            s = surv[j, i]
            bnd = any(0 <= i + di < S and 0 <= j + dj < S and surv[j + dj, i + di] != s
                      for dj in (-1, 0, 1) for di in (-1, 0, 1) if di or dj)
            lx, ly = grid[j * S + i]
            if not bnd:
                if s:
                    sx += float(lx)
                    sy += float(ly)
                    w += 1.0
                continue
            for a in range(K):
                lly = f(ly + f(hy * f(f(f(2.0) * f(a + 0.5)) / f(K) - f(1.0))))
                for b in range(K):
                    llx = f(lx + f(hx * f(f(f(2.0) * f(b + 0.5)) / f(K) - f(1.0))))
                    pending.append((llx, lly))
    if pending:
        ok = _survive(surfs, pending, z, d)
        for (llx, lly), o in zip(pending, ok):
            if o:
                sx += float(llx) * float(inv_k2)
                sy += float(lly) * float(inv_k2)
                w += float(inv_k2)
    if w > 0:
        return float(f(sx / w)), float(f(sy / w)), True
    return 0.0, 0.0, False


def survivor_envelope(surfs, ep_x, ep_y, cx, cy, ax, ay, ME):
    """build_survivor_envelope: (ME, ME) float32."""
    from oracle import oracle as O
    f = np.float32
    z = f(f(surfs[0].z) - f(20.0))
    _, _, d = _launch(ax, ay)
    coord = lambda k: f(f(f(f(k) + f(0.5)) / f(ME)) * f(2.0) - f(1.0))
    cells = [(coord(i), coord(j)) for j in range(ME) for i in range(ME)]
    inside = O.pupil_contains(surfs, cells, aspect_one=True).reshape(ME, ME)
    env = np.full((ME, ME), -1.0, np.float32)
    launch = [(f(f(cx) + f(u * f(ep_x))), f(f(cy) + f(v * f(ep_y)))) for (u, v), ins in zip(cells, inside.ravel())
              if ins]
    env[inside] = _survive(surfs, launch, z, d).astype(np.float32)
    base = env.copy()
    K = 10
    du = f(f(2.0) / f(ME))
    for j in range(ME):
        for i in range(ME):
            e = base[j, i]
            if e < 0:
                continue
            bnd = any(0 <= i + di < ME and 0 <= j + dj < ME and base[j + dj, i + di] >= 0
                      and (base[j + dj, i + di] > 0.5) != (e > 0.5)
                      for dj in (-1, 0, 1) for di in (-1, 0, 1) if di or dj)
            if not bnd:
                continue
            u0, v0 = cells[j * ME + i]
            sub = [(f(u0 + f(du * f(f(f(sx) + f(0.5)) / f(K) - f(0.5)))),
                    f(v0 + f(du * f(f(f(sy) + f(0.5)) / f(K) - f(0.5))))) for sy in range(K) for sx in range(K)]
            ins = O.pupil_contains(surfs, sub, aspect_one=True)
            pts = [(f(f(cx) + f(u * f(ep_x))), f(f(cy) + f(v * f(ep_y)))) for (u, v), k in zip(sub, ins) if k]
            if pts:
                env[j, i] = f(f(int(_survive(surfs, pts, z, d).sum())) / f(len(pts)))
    out = env.copy()
    for j in range(ME):
        for i in range(ME):
            if env[j, i] >= 0:
                continue
            best = 0.0
            for dj in range(-2, 3):
                for di in range(-2, 3):
                    if 0 <= i + di < ME and 0 <= j + dj < ME and env[j + dj, i + di] >= 0:
                        best = max(best, float(env[j + dj, i + di]))
            out[j, i] = best
    return out

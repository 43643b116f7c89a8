"""Restatement of the PSF grid splat (psf_kernel, psf_render.cu:30-232) over
rays traced by the float oracle (TEST INFRASTRUCTURE ONLY): every (source,
pupil sample, wavelength) primary ray, landing relative to the tile centre,
bilinear or normalised-Gaussian splat clipped to the tile, in float64."""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O


def render(surfs, cells, colors, grid, spec, tile_w, tile_h, grid_nx, comp_w, comp_h, mm_pp, mono=False,
           sigma_px=0.0, radius_px=0):
    out = np.zeros((3, comp_h, comp_w))
    grid = np.asarray(grid, np.float32).reshape(-1, 2)
    spec = np.asarray(spec, np.float32).reshape(-1, 4)
    R0 = np.float32(surfs[0].semi_aperture)
    z0 = np.float32(surfs[0].z) - np.float32(20.0)
    rw = 1.0 / len(grid)
    for i, (c, col) in enumerate(zip(cells, colors)):
        bx, by = np.float32(math.tan(np.float32(c["beam_ax"]))), np.float32(math.tan(np.float32(c["beam_ay"])))
        d = np.array([bx, by, 1.0], np.float32)
        d = (d * (np.float32(1.0) / np.float32(np.sqrt(np.float32(d @ d))))).astype(np.float32)
        tx0, ty0 = (i % grid_nx) * tile_w, (i // grid_nx) * tile_h
        for lam, cr_, cg_, cb_ in spec:
            rays = np.zeros((len(grid), 7), np.float32)
            rays[:, 0] = grid[:, 0] * R0 - np.float32(20.0) * bx
            rays[:, 1] = grid[:, 1] * R0 - np.float32(20.0) * by
            rays[:, 2] = z0
            rays[:, 3:6] = d
            rays[:, 6] = lam
            res = O.trace(surfs, -1, -1, rays, fp64=False)
            ok = (res[:, 4] == 0) & np.isfinite(res[:, 0]) & np.isfinite(res[:, 1])
            for x, y, w in res[ok][:, [0, 1, 3]]:
                tx = (x - c["chief_x_mm"]) / mm_pp + tile_w * 0.5
                ty = (y - c["chief_y_mm"]) / mm_pp + tile_h * 0.5
                margin = radius_px + 1 if radius_px > 0 else 1
                if tx < -margin or tx > tile_w + margin or ty < -margin or ty > tile_h + margin:
                    continue
                px, py = tx + tx0, ty + ty0
                ww = w * rw
                vals = ((col[0] + col[1] + col[2]) / 3.0 * cg_ * ww, 0.0, 0.0) if mono else \
                    (col[0] * cr_ * ww, col[1] * cg_ * ww, col[2] * cb_ * ww)
                taps = []
                if sigma_px <= 0:
                    x0, y0 = math.floor(px - 0.5), math.floor(py - 0.5)
                    fx, fy = px - 0.5 - x0, py - 0.5 - y0
                    taps = [(x0, y0, (1 - fx) * (1 - fy)), (x0 + 1, y0, fx * (1 - fy)),
                            (x0, y0 + 1, (1 - fx) * fy), (x0 + 1, y0 + 1, fx * fy)]
                else:
                    cx, cy = math.floor(px), math.floor(py)
                    ox, oy = px - (cx + 0.5), py - (cy + 0.5)
                    ks = [(dx, dy, math.exp(-((dx - ox) ** 2 + (dy - oy) ** 2) / (2 * sigma_px ** 2)))
                          for dy in range(-radius_px, radius_px + 1) for dx in range(-radius_px, radius_px + 1)]
                    s = sum(k[2] for k in ks)
                    taps = [(cx + dx, cy + dy, v / s) for dx, dy, v in ks if v / s >= 1e-6]
                for xi, yi, wt in taps:
                    if not (tx0 <= xi < tx0 + tile_w and ty0 <= yi < ty0 + tile_h):
                        continue
                    for ch in range(3):
                        out[ch, yi, xi] += vals[ch] * wt
    return out

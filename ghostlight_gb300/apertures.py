"""Seeded pupil amplitudes for the starburst workloads.

``curved_blade_mask``: an n x n bladed iris whose edges are circular arcs
(curvature in [-1, 1]: 0 straight blades, +1 a circle), anti-aliased over a
given width in pixels, with uniform-random dust occluders of radius r_min..r_max
pixels covering a given area fraction — the configuration-3 aperture (512^2,
9 curved blades, 2 px edge, 0.5% dust of radius 1-4 px).
"""
from __future__ import annotations

import numpy as np


def curved_blade_mask(n: int = 512, blades: int = 9, curvature: float = 0.35, fill: float = 0.45,
                      aa_px: float = 2.0, dust_density: float = 0.005, dust_r=(1.0, 4.0), rotation: float = 0.0,
                      seed: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = 0.5 * (n - 1)
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    dx, dy = x - c, y - c
    r = np.hypot(dx, dy)
    R = fill * n                              # circumscribed radius (px)
    sector = 2.0 * np.pi / blades
    th = np.mod(np.arctan2(dy, dx) - rotation, sector) - 0.5 * sector
    apothem = R * np.cos(0.5 * sector)
    straight = apothem / np.cos(th)           # polygon edge radius at this angle
    # curved edge: blend the straight chord toward the circumscribed circle
    edge = straight + curvature * (R - straight)
    sd = edge - r                             # signed distance (px), + inside
    amp = np.clip(sd / aa_px + 0.5, 0.0, 1.0)
    # dust discs
    inside = amp > 0
    area = float(inside.sum())
    target = dust_density * area
    covered = 0.0
    dust = np.ones_like(amp)
    while covered < target:
        rad = rng.uniform(*dust_r)
        cx_, cy_ = rng.uniform(c - R, c + R, 2)
        d = np.hypot(x - cx_, y - cy_)
        disc = np.clip((d - rad) / 1.0 + 0.5, 0.0, 1.0)
        covered += np.pi * rad * rad
        dust = np.minimum(dust, disc)
    return (amp * dust).astype(np.float32)

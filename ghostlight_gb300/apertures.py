"""Seeded pupil amplitudes for the starburst workloads.

``curved_blade_mask``: an n x n bladed iris, its edge the authored blade
silhouette of a bladed stop (ApertureProfile, ghostlight/src/
aperture_profile.h: each half blade edge a conic arc in 1/r from the waist
to the tip; curvature in [-1, 1]: 0 straight blades, +1 a circle, < 0
scalloped; optional twist and tip notch), anti-aliased over a given width in
pixels, with uniform-random dust occluders of radius r_min..r_max pixels
covering a given area fraction — the configuration-3 aperture (512^2, 9
curved blades, 2 px edge, 0.5% dust of radius 1-4 px).
"""
from __future__ import annotations

import ctypes as C

import numpy as np


def blade_radius(theta, blades: int, rotation: float = 0.0, curvature: float = 0.0, twist: float = 0.0,
                 notch: float = 0.0, notch_angle: float = 0.0) -> np.ndarray:
    """Normalised boundary radius (1 = blade tip) of a bladed stop at angles
    theta (radians), through gl_blade_radius (host float arithmetic)."""
    from . import _native
    th = np.ascontiguousarray(theta, np.float32).reshape(-1)
    out = np.empty_like(th)
    P = C.POINTER(C.c_float)
    _native.check(_native.load().gl_blade_radius(int(blades), float(rotation), float(curvature), float(twist),
                                                 float(notch), float(notch_angle), th.ctypes.data_as(P),
                                                 len(th), out.ctypes.data_as(P)), "blade_radius")
    return out.reshape(np.shape(theta))


def curved_blade_mask(n: int = 512, blades: int = 9, curvature: float = 0.35, fill: float = 0.45,
                      aa_px: float = 2.0, dust_density: float = 0.005, dust_r=(1.0, 4.0), rotation: float = 0.0,
                      seed: int = 3, twist: float = 0.0, notch: float = 0.0, notch_angle: float = 0.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = 0.5 * (n - 1)
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    dx, dy = x - c, y - c
    r = np.hypot(dx, dy)
    R = fill * n                              # blade-tip radius (px)
    edge = R * blade_radius(np.arctan2(dy, dx), blades, rotation, curvature, twist, notch,
                            notch_angle).astype(np.float64)
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

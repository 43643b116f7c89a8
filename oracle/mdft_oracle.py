"""FP64 numpy oracle of the matrix-DFT starburst (TEST INFRASTRUCTURE ONLY).

Field form: E_l = W_y A W_x^T with
W[k][j] = exp(-2 pi i s_l (j - (n-1)/2)(k - c)), I_l = |E_l|^2,
out_c = sum_l w_c(l) I_l — the per-wavelength triple product of the
reference's mdft_render.cu:156-173 in its field form.  Rows and
columns can be restricted to a window so full-size outputs are checked on
sub-windows.
"""
from __future__ import annotations

import numpy as np


def dft_matrix(n: int, K: int, s: float, c: float, rows=None) -> np.ndarray:
    k = np.arange(K, dtype=np.float64) if rows is None else np.asarray(rows, np.float64)
    j = np.arange(n, dtype=np.float64) - 0.5 * (n - 1)
    ph = s * np.outer(k - c, j)
    ph = ph - np.rint(ph)
    return np.exp(-2j * np.pi * ph)


def eform(A, K, scale_x, scale_y, cx, cy, weights, rows=None, cols=None):
    """(3, len(rows), len(cols)) float64; K = side or (Kx, Ky)."""
    A = np.asarray(A, np.float64)
    n = A.shape[0]
    Kx, Ky = (K, K) if np.isscalar(K) else K
    rows = np.arange(Ky) if rows is None else np.asarray(rows)
    cols = np.arange(Kx) if cols is None else np.asarray(cols)
    out = np.zeros((3, len(rows), len(cols)))
    w = np.asarray(weights, np.float64).reshape(-1, 3)
    for l in range(len(scale_x)):
        Wx = dft_matrix(n, K, scale_x[l], cx, cols)
        Wy = dft_matrix(n, K, scale_y[l], cy, rows)
        E = Wy @ (A @ Wx.T)
        I = E.real ** 2 + E.imag ** 2
        for c in range(3):
            out[c] += w[l, c] * I
    return out


def test_pupil(n: int, seed: int = 3) -> np.ndarray:
    """A seeded pupil amplitude for tests: a 9-blade disc with a soft edge."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    c = 0.5 * (n - 1)
    r = np.hypot(x - c, y - c) / (0.4 * n)
    th = np.arctan2(y - c, x - c)
    edge = np.cos(np.pi / 9) / np.cos((th % (2 * np.pi / 9)) - np.pi / 9)
    a = np.clip((edge - r) * 0.4 * n / 2.0 + 0.5, 0.0, 1.0)
    a *= (rng.random((n, n)) > 0.005)
    return a.astype(np.float32)


def stop_pupil(aspect: float, n_blades: int, rot_rad: float, N: int, fill: float, blade_stop=None) -> np.ndarray:
    """4 x 4 supersampled stop silhouette in float32 arithmetic, the stop term
    of build_pupil_kernel (starburst_render.cu:155-191) with
    PupilMask::contains (aperture_sampler.h:63-82).  blade_stop: the stop
    surface record when its blade shape is authored (the boundary is then the
    profile's r(theta), aperture_sampler.h:70-73)."""
    f = np.float32
    apothem = f(np.cos(f(np.pi) / f(n_blades))) if n_blades >= 3 else f(1)
    sector = f(f(2) * f(np.pi) / f(n_blades)) if n_blades >= 3 else f(1)
    j, i = np.mgrid[0:N, 0:N]
    cnt = np.zeros((N, N), np.int32)
    for sy in range(4):
        for sx in range(4):
            u = ((i.astype(f) + (f(sx) + f(0.5)) * f(0.25)) / f(N) * f(2) - f(1)) / f(fill)
            v = ((j.astype(f) + (f(sy) + f(0.5)) * f(0.25)) / f(N) * f(2) - f(1)) / f(fill)
            ux = (u / f(aspect)).astype(f)
            r2 = (ux * ux + v * v).astype(f)
            inside = r2 <= f(1)
            if n_blades >= 3 and blade_stop is not None:
                from . import oracle as O
                rad = O.blade_radius(blade_stop, np.arctan2(v, ux).astype(f))
                inside &= np.sqrt(r2).astype(f) <= rad
            elif n_blades >= 3:
                ang = (np.arctan2(v, ux).astype(f) - f(rot_rad)).astype(f)
                sec = np.fmod(ang, sector).astype(f)
                sec = np.where(sec < 0, sec + sector, sec).astype(f)
                inside &= ~((np.sqrt(r2).astype(f) * np.cos(sec - sector * f(0.5)).astype(f)) > apothem)
            cnt += inside
    return (cnt.astype(f) * f(1.0 / 16.0))

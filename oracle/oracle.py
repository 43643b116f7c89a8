"""ctypes wrapper of the C oracle (oracle/gl_oracle.c).

TEST INFRASTRUCTURE ONLY — used by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg as the reference for parity and the CPU
baseline.  The product
(ghostlight_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
if str(HERE.parent) not in sys.path:
    sys.path.insert(0, str(HERE.parent))
from ghostlight_gb300._abi import gl_surface, surface_array  # noqa: E402

_lib = None


def _load():
    global _lib
    if _lib is None:
        from oracle import build as _b
        lib = C.CDLL(str(_b.build_oracle()))
        P, i, f, d = C.POINTER, C.c_int, C.c_float, C.c_double
        lib.orc_trace.argtypes = [P(gl_surface), i, i, i, P(f), i, i, P(d)]
        lib.orc_enumerate.argtypes = [P(gl_surface), i, P(i), i]
        lib.orc_filter.argtypes = [P(gl_surface), i, f, f, f, i, f, P(i), P(f), P(f), i]
        lib.orc_aperture_samples.argtypes = [P(gl_surface), i, i, i, i, i, f, P(f), i]
        lib.orc_blade_radius.argtypes = [P(gl_surface), P(f), i, P(f)]
        lib.orc_coating_register.argtypes = [i, i, i, i, P(f), f, i]
        lib.orc_image_register.argtypes = [i, i, i, P(f), f]
        lib.orc_pupil_contains.argtypes = [P(gl_surface), i, i, f, i, P(f), i, P(C.c_ubyte)]
        lib.orc_render.argtypes = [P(gl_surface), i, P(i), P(f), P(i), i, P(f), i, P(f), P(i),
                                   P(f), i, f, f, i, i, f, i, i, P(d)]
        _lib = lib
    return _lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def register_coating(table_id, model, axis0, r, axis1=None, angle_ref_ior=1.0, discard=False):
    """Give the oracle the table a surface names by ``ar_layers = table_id``
    (OpticalSystem::coating_tables, optical_system.h:288-295): 1-D models
    take keys ``axis0`` and ``r``; SPECTRAL_ANGULAR (model 3) wavelengths
    ``axis0``, angles ``axis1`` and ``r`` of shape (len(axis0), len(axis1))."""
    lib = _load()
    a0 = np.asarray(axis0, np.float32).ravel()
    a1 = np.zeros(0, np.float32) if axis1 is None else np.asarray(axis1, np.float32).ravel()
    data = np.ascontiguousarray(np.concatenate([a0, a1, np.asarray(r, np.float32).ravel()]), np.float32)
    if lib.orc_coating_register(int(table_id), int(model), len(a0), len(a1), _fp(data), float(angle_ref_ior),
                                int(bool(discard))) != 0:
        raise ValueError("oracle: bad coating table %d" % table_id)


def register_image(image_id, pixels, semi_diameter):
    """Give the oracle the bitmap an IMAGE surface names by aperture_blades."""
    lib = _load()
    px = np.ascontiguousarray(pixels, np.float32)
    if lib.orc_image_register(int(image_id), px.shape[1], px.shape[0], _fp(px), float(semi_diameter)) != 0:
        raise ValueError("oracle: bad aperture image %d" % image_id)


def pupil_contains(surfs, uv, blades_override=0, rotation_deg=0.0, aspect_one=False):
    """PupilMask::contains of the lens's stop at (n, 2) points -> bool (n,)."""
    lib = _load()
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    out = np.zeros(len(uv), np.uint8)
    lib.orc_pupil_contains(surface_array(surfs), len(surfs), int(blades_override), float(rotation_deg),
                           int(bool(aspect_one)), _fp(uv), len(uv), out.ctypes.data_as(C.POINTER(C.c_ubyte)))
    return out.astype(bool)


def trace(surfs, a, b, rays, fp64=True):
    """rays (n,7) -> (n,5) float64: x, y, z, weight, status.  b < 0: primary."""
    lib = _load()
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 7)
    out = np.zeros((rays.shape[0], 5), np.float64)
    lib.orc_trace(surface_array(surfs), len(surfs), a, b, _fp(rays), rays.shape[0], int(fp64), _dp(out))
    return out


def enumerate_pairs(surfs):
    lib = _load()
    cap = len(surfs) ** 2
    out = np.zeros((cap, 2), np.int32)
    n = lib.orc_enumerate(surface_array(surfs), len(surfs), _ip(out), cap)
    return out[:n].copy()


def filter_pairs(surfs, hw, hh, min_int=1e-7, normalize=True, max_boost=100.0, footprint=False):
    """Reference-exact filter; with footprint=True also the (n,2) green-probe
    footprint in mm that sizes adaptive pupil grids."""
    lib = _load()
    cap = len(surfs) ** 2
    ab = np.zeros((cap, 2), np.int32)
    bo = np.zeros(cap, np.float32)
    fp = np.zeros((cap, 2), np.float32)
    n = lib.orc_filter(surface_array(surfs), len(surfs), hw, hh, min_int, int(normalize), max_boost,
                       _ip(ab), _fp(bo), _fp(fp), cap)
    if footprint:
        return ab[:n].copy(), bo[:n].copy(), fp[:n].copy()
    return ab[:n].copy(), bo[:n].copy()


def blade_radius(stop, theta):
    """Normalised boundary radius of a bladed stop at angles theta (float32)."""
    lib = _load()
    th = np.ascontiguousarray(theta, np.float32).reshape(-1)
    out = np.zeros_like(th)
    if lib.orc_blade_radius(C.byref(stop), _fp(th), len(th), _fp(out)) != 0:
        raise ValueError("blade_radius: not a bladed stop")
    return out.reshape(np.shape(theta))


def aperture_samples(surfs, grid, jitter=0, seed=0, blades_override=0, rotation_deg=0.0):
    lib = _load()
    out = np.zeros((max(grid * grid, 1), 2), np.float32)
    n = lib.orc_aperture_samples(surface_array(surfs), len(surfs), grid, jitter, seed, blades_override,
                                 rotation_deg, _fp(out), grid * grid)
    return out[:n].copy()


def render(surfs, pairs, boosts, sources, grids, spec, hw, hh, W, H, gain, pair_grid=None,
           fp64=True, n_threads=0):
    """Ghost image (3, H, W) float64.  grids: list of (n,2) pupil grids (one
    shared grid when pair_grid is None)."""
    lib = _load()
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    boosts = np.ascontiguousarray(boosts, np.float32)
    sources = np.ascontiguousarray(sources, np.float32).reshape(-1, 5)
    if isinstance(grids, np.ndarray):
        grids = [grids]
    offs = np.zeros(len(grids) + 1, np.int32)
    for i, g in enumerate(grids):
        offs[i + 1] = offs[i] + len(g)
    flat = np.ascontiguousarray(np.concatenate([np.asarray(g, np.float32).reshape(-1, 2) for g in grids]))
    spec = np.ascontiguousarray(spec, np.float32).reshape(-1, 4)
    pg = None if pair_grid is None else np.ascontiguousarray(pair_grid, np.int32)
    out = np.zeros((3, H, W), np.float64)
    lib.orc_render(surface_array(surfs), len(surfs), _ip(pairs), _fp(boosts),
                   _ip(pg) if pg is not None else None, pairs.shape[0], _fp(sources),
                   sources.shape[0], _fp(flat), _ip(offs), _fp(spec), spec.shape[0], hw, hh, W, H,
                   gain, int(fp64), n_threads, _dp(out))
    return out

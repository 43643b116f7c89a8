"""ctypes wrapper of oracle/_ref/libghostlight_ref.so — the reference's own
CPU code for the flare path (TEST INFRASTRUCTURE ONLY; see ref_driver.cpp).

Available only where the reference checkout exists (it is built from the
reference sources by oracle/build.py); callers check ``available()``.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from ghostlight_gb300._abi import gl_surface, surface_array  # noqa: E402

_lib = None


def available() -> bool:
    try:
        _load()
        return True
    except Exception:
        return False


def _load():
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _b  # type: ignore
    path = _b.build_ref()
    if path is None:
        raise RuntimeError("reference sources absent")
    lib = C.CDLL(str(path))
    P = C.POINTER
    f, i = C.c_float, C.c_int
    lib.ref_sizeof_surface.restype = i
    lib.ref_load_lens.argtypes = [C.c_char_p, P(gl_surface), i, P(f)]
    lib.ref_finalize.argtypes = [P(gl_surface), i]
    lib.ref_trace.argtypes = [P(gl_surface), i, i, i, P(f), i, P(f)]
    lib.ref_enumerate.argtypes = [P(gl_surface), i, P(i), i]
    lib.ref_filter.argtypes = [P(gl_surface), i, f, f, f, i, f, P(i), P(f), i]
    lib.ref_aperture_samples.argtypes = [P(gl_surface), i, i, i, i, i, f, P(f), i]
    lib.ref_spectral_table.argtypes = [i, i, P(f), P(f)]
    lib.ref_color_matrices.argtypes = [i, i, P(f), P(f)]
    lib.ref_cie_profile.argtypes = [P(f), P(f), P(f), P(f), i]
    lib.ref_calibrate.argtypes = [P(gl_surface), i, f, P(f)]
    lib.ref_solve_source.argtypes = [P(gl_surface), i, P(f), f, f, f, f, P(f)]
    lib.ref_render_ghosts_cpu.argtypes = [P(gl_surface), i, P(i), P(f), i, P(f), i,
                                          P(f), i, P(f), i, f, f, i, i, f, i, P(f)]
    lib.ref_render_ghosts_cpu.restype = i
    lib.ref_coating_register.argtypes = [i, i, i, i, P(f), f, i]
    lib.ref_image_register.argtypes = [i, i, i, P(f), f]
    lib.ref_bake_layers.argtypes = [P(gl_surface), i, i, i, P(f), P(i), P(f), P(f), P(f), P(f), P(f), P(f), P(f)]
    lib.ref_load_lens_coating.argtypes = [C.c_char_p, i, P(i), P(f), P(f), i]
    assert lib.ref_sizeof_surface() == C.sizeof(gl_surface)
    _lib = lib
    return lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def load_lens(path):
    lib = _load()
    fl = C.c_float()
    n = lib.ref_load_lens(str(path).encode(), None, 0, C.byref(fl))
    if n < 0:
        raise RuntimeError("reference loader rejected %s" % path)
    arr = (gl_surface * n)()
    lib.ref_load_lens(str(path).encode(), arr, n, C.byref(fl))
    return list(arr), float(fl.value)


def register_coating(table_id, model, axis0, r, axis1=None, angle_ref_ior=1.0, discard=False):
    """Attach a coating table to every flat record that names ``table_id``
    in ar_layers (as OpticalSystem::coating_tables for the reference)."""
    lib = _load()
    a0 = np.asarray(axis0, np.float32).ravel()
    a1 = np.zeros(0, np.float32) if axis1 is None else np.asarray(axis1, np.float32).ravel()
    data = np.ascontiguousarray(np.concatenate([a0, a1, np.asarray(r, np.float32).ravel()]), np.float32)
    lib.ref_coating_register(int(table_id), int(model), len(a0), len(a1), _fp(data), float(angle_ref_ior),
                             int(bool(discard)))


def register_image(image_id, pixels, semi_diameter):
    """Attach a bitmap to every IMAGE record naming ``image_id`` (as
    OpticalSystem::aperture_images + Surface.aperture_semi_diameter)."""
    lib = _load()
    px = np.ascontiguousarray(pixels, np.float32)
    lib.ref_image_register(int(image_id), px.shape[1], px.shape[0], _fp(px), float(semi_diameter))


def bake_layers(surfs, index, layers):
    """OpticalSystem::bake_coating_layers: layers = [(thickness_nm, nk (K,3)
    of lambda_um, n, k)] -> (wavelengths, angles, r (31, 18), angle_ref_ior)."""
    lib = _load()
    th = np.array([t for t, _ in layers], np.float32)
    cnt = np.array([len(nk) for _, nk in layers], np.int32)
    nk = np.concatenate([np.asarray(nk, np.float32).reshape(-1, 3) for _, nk in layers])
    lam, nn, kk = (np.ascontiguousarray(nk[:, c]) for c in range(3))
    wl, ang, r = np.zeros(31, np.float32), np.zeros(18, np.float32), np.zeros((31, 18), np.float32)
    ref = C.c_float()
    if lib.ref_bake_layers(surface_array(surfs), len(surfs), index, len(layers), _fp(th), _ip(cnt), _fp(lam),
                           _fp(nn), _fp(kk), _fp(wl), _fp(ang), _fp(r), C.byref(ref)) != 0:
        raise RuntimeError("reference bake failed")
    return wl, ang, r, float(ref.value)


def load_lens_coating(path, index):
    """The reference loader's coating of surface ``index``: (model, axis0,
    axis1, r, angle_ref_ior, discard); empty arrays when it has no table."""
    lib = _load()
    meta = np.zeros(4, np.int32)
    ref = C.c_float()
    n = lib.ref_load_lens_coating(str(path).encode(), index, _ip(meta), C.byref(ref), None, 0)
    if n < 0:
        raise RuntimeError("reference loader rejected %s" % path)
    data = np.zeros(max(n, 1), np.float32)
    lib.ref_load_lens_coating(str(path).encode(), index, _ip(meta), C.byref(ref), _fp(data), n)
    m, n0, n1, disc = (int(v) for v in meta)
    a0 = data[:n0].copy()
    a1 = data[n0:n0 + n1].copy()
    r = data[n0 + n1:n].copy()
    if n1:
        r = r.reshape(n0, n1)
    return m, a0, a1, r, float(ref.value), bool(disc)


def trace(surfs, a, b, rays):
    lib = _load()
    rays = np.ascontiguousarray(rays, np.float32)
    out = np.zeros((rays.shape[0], 5), np.float32)
    lib.ref_trace(surface_array(surfs), len(surfs), a, b, _fp(rays), rays.shape[0], _fp(out))
    return out


def enumerate_pairs(surfs):
    lib = _load()
    cap = len(surfs) * len(surfs)
    out = np.zeros((cap, 2), np.int32)
    n = lib.ref_enumerate(surface_array(surfs), len(surfs), _ip(out), cap)
    return out[:n].copy()


def filter_pairs(surfs, hw, hh, min_int=1e-7, normalize=True, max_boost=100.0):
    lib = _load()
    cap = len(surfs) * len(surfs)
    ab = np.zeros((cap, 2), np.int32)
    bo = np.zeros(cap, np.float32)
    n = lib.ref_filter(surface_array(surfs), len(surfs), hw, hh, min_int, int(normalize),
                       max_boost, _ip(ab), _fp(bo), cap)
    return ab[:n].copy(), bo[:n].copy()


def aperture_samples(surfs, ray_grid, jitter=0, seed=0, blades_override=0, rotation_deg=0.0):
    lib = _load()
    cap = ray_grid * ray_grid
    out = np.zeros((max(cap, 1), 2), np.float32)
    n = lib.ref_aperture_samples(surface_array(surfs), len(surfs), ray_grid, jitter, seed,
                                 blades_override, rotation_deg, _fp(out), cap)
    return out[:n].copy()


def spectral_table(n, output_cs=0):
    lib = _load()
    out = np.zeros((max(n, 3), 4), np.float32)
    corr = np.zeros(9, np.float32)
    k = lib.ref_spectral_table(n, output_cs, _fp(out), _fp(corr))
    return out[:k].copy(), corr.reshape(3, 3)


def color_matrices(input_cs=0, output_cs=0):
    lib = _load()
    a = np.zeros(9, np.float32)
    b = np.zeros(9, np.float32)
    lib.ref_color_matrices(input_cs, output_cs, _fp(a), _fp(b))
    return a.reshape(3, 3), b.reshape(3, 3)


CALIB_FIELDS = ("sensor_half_w", "sensor_half_h", "max_half_angle_h", "max_half_angle_v",
                "image_circle_semi_w", "image_circle_semi_h", "focal_length_x",
                "focal_length_y", "entrance_pupil_semi_x", "entrance_pupil_semi_y",
                "f_number_x", "f_number_y", "pupil_area_frac")


def calibrate(surfs, focal_length=0.0):
    lib = _load()
    out = np.zeros(13, np.float32)
    lib.ref_calibrate(surface_array(surfs), len(surfs), focal_length, _fp(out))
    return dict(zip(CALIB_FIELDS, map(float, out)))


def solve_source(surfs, calib, ndc_x, ndc_y, eff_hw, eff_hh):
    lib = _load()
    c = np.array([calib[k] for k in CALIB_FIELDS], np.float32)
    out = np.zeros(5, np.float32)
    lib.ref_solve_source(surface_array(surfs), len(surfs), _fp(c), ndc_x, ndc_y, eff_hw,
                         eff_hh, _fp(out))
    return {"angle_x": float(out[0]), "angle_y": float(out[1]), "status": int(out[2]),
            "screen_x": float(out[3]), "screen_y": float(out[4])}


def render_ghosts_cpu(surfs, pairs, boosts, sources, grid, spec, hw, hh, W, H, gain,
                      n_threads=0):
    """Host mirror of ghost_kernel's full-pupil main path; returns (3,H,W)."""
    lib = _load()
    pairs = np.ascontiguousarray(pairs, np.int32)
    boosts = np.ascontiguousarray(boosts, np.float32)
    sources = np.ascontiguousarray(sources, np.float32).reshape(-1, 5)
    grid = np.ascontiguousarray(grid, np.float32).reshape(-1, 2)
    spec = np.ascontiguousarray(spec, np.float32).reshape(-1, 4)
    out = np.zeros((3, H, W), np.float32)
    lib.ref_render_ghosts_cpu(surface_array(surfs), len(surfs), _ip(pairs), _fp(boosts),
                              pairs.shape[0], _fp(sources), sources.shape[0], _fp(grid),
                              grid.shape[0], _fp(spec), spec.shape[0], hw, hh, W, H, gain,
                              n_threads, _fp(out))
    return out


def cie_profile():
    lib = _load()
    a = [np.zeros(128, np.float32) for _ in range(4)]
    n = lib.ref_cie_profile(*[_fp(x) for x in a], 128)
    return [x[:n].copy() for x in a]

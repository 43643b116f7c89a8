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

_lib = None
_gpu = None


def _sp(surfs):
    """(buffer, count) of a lens given as flat records: a numpy array of the
    packed ``gl_surface`` records (raw bytes, as the fixtures store them) or a
    list of ``ghostlight_gb300._abi.gl_surface`` (imported only then).  The
    buffer is a ctypes array that the call's argument tuple keeps alive."""
    if isinstance(surfs, np.ndarray):
        raw = np.ascontiguousarray(surfs).tobytes()
        size = _load().ref_sizeof_surface()
        if len(raw) % size:
            raise ValueError("lens records are not a whole number of gl_surface records")
        return (C.c_char * len(raw)).from_buffer_copy(raw), len(raw) // size
    from ghostlight_gb300._abi import surface_array
    return surface_array(surfs), len(surfs)


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
    vp = C.c_void_p
    lib.ref_sizeof_surface.restype = i
    lib.ref_load_lens.argtypes = [C.c_char_p, vp, i, P(f)]
    lib.ref_finalize.argtypes = [vp, i]
    lib.ref_trace.argtypes = [vp, i, i, i, P(f), i, P(f)]
    lib.ref_enumerate.argtypes = [vp, i, P(i), i]
    lib.ref_filter.argtypes = [vp, i, f, f, f, i, f, P(i), P(f), i]
    lib.ref_aperture_samples.argtypes = [vp, i, i, i, i, i, f, P(f), i]
    lib.ref_spectral_table.argtypes = [i, i, P(f), P(f)]
    lib.ref_color_matrices.argtypes = [i, i, P(f), P(f)]
    lib.ref_cie_profile.argtypes = [P(f), P(f), P(f), P(f), i]
    lib.ref_calibrate.argtypes = [vp, i, f, P(f)]
    lib.ref_solve_source.argtypes = [vp, i, P(f), f, f, f, f, P(f)]
    lib.ref_render_ghosts_cpu.argtypes = [vp, i, P(i), P(f), i, P(f), i,
                                          P(f), i, P(f), i, f, f, i, i, f, i, P(f)]
    lib.ref_render_ghosts_cpu.restype = i
    lib.ref_coating_register.argtypes = [i, i, i, i, P(f), f, i]
    lib.ref_image_register.argtypes = [i, i, i, P(f), f]
    lib.ref_bake_layers.argtypes = [vp, i, i, i, P(f), P(i), P(f), P(f), P(f), P(f), P(f), P(f), P(f)]
    lib.ref_load_lens_coating.argtypes = [C.c_char_p, i, P(i), P(f), P(f), i]
    lib.ref_render_frame_cpu.argtypes = [vp, i, P(i), P(f), P(i), i, P(f), P(f), i, vp, f, f, i, i, f, i, i,
                                         P(f), P(C.c_longlong)]
    lib.ref_render_frame_cpu.restype = i
    lib.ref_ghost_footprints.argtypes = [vp, i, P(i), i, P(f)]
    _lib = lib
    return lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def load_lens(path):
    from ghostlight_gb300._abi import gl_surface
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
    if lib.ref_bake_layers(*_sp(surfs), index, len(layers), _fp(th), _ip(cnt), _fp(lam),
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
    lib.ref_trace(*_sp(surfs), a, b, _fp(rays), rays.shape[0], _fp(out))
    return out


def enumerate_pairs(surfs):
    lib = _load()
    cap = len(surfs) * len(surfs)
    out = np.zeros((cap, 2), np.int32)
    n = lib.ref_enumerate(*_sp(surfs), _ip(out), cap)
    return out[:n].copy()


def filter_pairs(surfs, hw, hh, min_int=1e-7, normalize=True, max_boost=100.0):
    lib = _load()
    cap = len(surfs) * len(surfs)
    ab = np.zeros((cap, 2), np.int32)
    bo = np.zeros(cap, np.float32)
    n = lib.ref_filter(*_sp(surfs), hw, hh, min_int, int(normalize),
                       max_boost, _ip(ab), _fp(bo), cap)
    return ab[:n].copy(), bo[:n].copy()


def aperture_samples(surfs, ray_grid, jitter=0, seed=0, blades_override=0, rotation_deg=0.0):
    lib = _load()
    cap = ray_grid * ray_grid
    out = np.zeros((max(cap, 1), 2), np.float32)
    n = lib.ref_aperture_samples(*_sp(surfs), ray_grid, jitter, seed,
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
    lib.ref_calibrate(*_sp(surfs), focal_length, _fp(out))
    return dict(zip(CALIB_FIELDS, map(float, out)))


def solve_source(surfs, calib, ndc_x, ndc_y, eff_hw, eff_hh):
    lib = _load()
    c = np.array([calib[k] for k in CALIB_FIELDS], np.float32)
    out = np.zeros(5, np.float32)
    lib.ref_solve_source(*_sp(surfs), _fp(c), ndc_x, ndc_y, eff_hw,
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
    lib.ref_render_ghosts_cpu(*_sp(surfs), _ip(pairs), _fp(boosts),
                              pairs.shape[0], _fp(sources), sources.shape[0], _fp(grid),
                              grid.shape[0], _fp(spec), spec.shape[0], hw, hh, W, H, gain,
                              n_threads, _fp(out))
    return out


def cie_profile():
    lib = _load()
    a = [np.zeros(128, np.float32) for _ in range(4)]
    n = lib.ref_cie_profile(*[_fp(x) for x in a], 128)
    return [x[:n].copy() for x in a]


def render_frame_cpu(surfs, pairs, boosts, pair_side, source, spec, corr, hw, hh, W, H, gain,
                     cull=True, n_threads=0):
    """One full ghost frame on the host with the reference's own trace code
    (ref_driver.cpp: the probe cull, the main path of ghost_kernel over each
    pair's own regular grid, the colour correction).  Returns ((3,H,W) image,
    {"probe_traces", "render_traces", "kept_pairs", "threads"})."""
    lib = _load()
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    boosts = np.ascontiguousarray(boosts, np.float32)
    side = np.ascontiguousarray(pair_side, np.int32)
    src = np.ascontiguousarray(source, np.float32).reshape(-1)[:5].copy()
    spec = np.ascontiguousarray(spec, np.float32).reshape(-1, 4)
    corr_p = None
    if corr is not None:
        corr = np.ascontiguousarray(corr, np.float32).reshape(9)
        corr_p = corr.ctypes.data_as(C.c_void_p)
    out = np.zeros((3, H, W), np.float32)
    cnt = np.zeros(3, np.int64)
    nt = lib.ref_render_frame_cpu(*_sp(surfs), _ip(pairs), _fp(boosts), _ip(side), pairs.shape[0], _fp(src),
                                  _fp(spec), spec.shape[0], corr_p, hw, hh, W, H, gain, int(bool(cull)),
                                  n_threads, _fp(out), cnt.ctypes.data_as(C.POINTER(C.c_longlong)))
    return out, {"probe_traces": int(cnt[0]), "render_traces": int(cnt[1]), "kept_pairs": int(cnt[2]),
                 "threads": int(nt)}


def ghost_footprints(surfs, pairs):
    """(n_pairs, 2) landing extents in mm of the 8x8 spread probe."""
    lib = _load()
    pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    out = np.zeros((pairs.shape[0], 2), np.float32)
    lib.ref_ghost_footprints(*_sp(surfs), _ip(pairs), pairs.shape[0], _fp(out))
    return out


# ---- the reference's GPU renderer (oracle/_ref/libghostlight_ref_gpu.so) ----

class RefGpuCfg(C.Structure):
    """Mirror of RefGpuCfg in ref_driver.cpp: PointFlareConfig fields by name."""
    _fields_ = [(n, C.c_int) for n in ("ray_grid", "spectral_samples", "pupil_jitter", "jitter_seed")] + \
               [(n, C.c_float) for n in ("sensor_half_w", "sensor_half_h", "flare_gain", "min_ghost_intensity")] + \
               [(n, C.c_int) for n in ("cull_dead_pairs", "concentrate_samples", "adaptive_sample_budgets",
                                       "aperture_blades")] + \
               [(n, C.c_float) for n in ("source_x", "source_y", "source_r", "source_g", "source_b")] + \
               [(n, C.c_int) for n in ("starburst", "starburst_engine", "starburst_grid", "sb_spectral_samples")] + \
               [(n, C.c_float) for n in ("pupil_fill", "scale_trim")] + \
               [(n, C.c_int) for n in ("spectral_correction", "output_cs", "use_survivor_mask", "collect_stats",
                                       "veil", "pad2")] + \
               [(n, C.c_float) for n in ("veil_gain", "veil_spread", "veil_falloff")]

    def __init__(self, **kw):
        d = dict(ray_grid=64, spectral_samples=16, flare_gain=1000.0, min_ghost_intensity=1e-7,
                 cull_dead_pairs=1, concentrate_samples=1, adaptive_sample_budgets=1, source_x=0.5,
                 source_y=0.5, source_r=1.0, source_g=1.0, source_b=1.0, starburst_grid=1024,
                 pupil_fill=0.3, scale_trim=1.0, spectral_correction=1, use_survivor_mask=1, veil_gain=0.03,
                 veil_spread=0.12, veil_falloff=1.5)
        d.update(kw)
        super().__init__(**d)


def _load_gpu():
    global _gpu
    if _gpu is not None:
        return _gpu
    from . import build as _b  # type: ignore
    path = _b.build_ref_gpu()
    if path is None:
        raise RuntimeError("reference sources absent")
    lib = C.CDLL(str(path))
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    lib.refgpu_sizeof_cfg.restype = i
    lib.refgpu_render.argtypes = [vp, i, f, vp, C.POINTER(RefGpuCfg), vp, i, i, i, vp, vp,
                                  C.POINTER(C.c_double), vp, vp, i, vp]
    lib.refgpu_render.restype = i
    assert lib.refgpu_sizeof_cfg() == C.sizeof(RefGpuCfg)
    _gpu = lib
    return lib


def gpu_render(surfs, W, H, cfg, calib=None, focal_length=0.0, offsets=None, starburst=False, include=None,
               veil=False):
    """render_point_flare (offsets None) or render_source_flare of the
    reference's GPU renderer.  Returns (ghost (3,H,W), starburst (3,H,W) or
    None, wall ms of the call, stats dict or None)."""
    lib = _load_gpu()
    ghost = np.zeros((3, H, W), np.float32)
    star = np.zeros((3, H, W), np.float32) if starburst else None
    vl = np.zeros((3, H, W), np.float32) if veil else None
    cal = None
    if calib is not None:
        cal = np.array([calib[k] for k in CALIB_FIELDS], np.float32)
    offs = None
    n_off = 0
    if offsets is not None:
        offs = np.ascontiguousarray(offsets, np.float32).reshape(-1, 3)
        n_off = offs.shape[0]
    ms = C.c_double()
    stats = np.full(8, -1.0)
    buf, n = _sp(surfs)
    inc = None if include is None else np.ascontiguousarray(include, np.int32).reshape(-1, 2)
    rc = lib.refgpu_render(buf, n, focal_length, None if cal is None else cal.ctypes.data_as(C.c_void_p),
                           C.byref(cfg), None if offs is None else offs.ctypes.data_as(C.c_void_p), n_off,
                           W, H, ghost.ctypes.data_as(C.c_void_p),
                           None if star is None else star.ctypes.data_as(C.c_void_p), C.byref(ms),
                           stats.ctypes.data_as(C.c_void_p),
                           None if inc is None else inc.ctypes.data_as(C.c_void_p), 0 if inc is None else len(inc),
                           None if vl is None else vl.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise RuntimeError("reference GPU render failed")
    st = None
    if cfg.collect_stats:
        st = dict(zip(("ms_grid_build", "ms_upload", "ms_kernel", "ms_download", "ms_total", "n_pairs",
                       "traces_total", "traces_on_sensor"), stats.tolist()))
    if veil:
        return ghost, star, float(ms.value), st, vl
    return ghost, star, float(ms.value), st

"""The flare hot path behind the reference's Python call surface.

Reference functions mirrored (JaydenB/ghostlight, bindings/python/src):
  enumerate_ghost_pairs / filter_ghost_pairs   bind_ghost.cpp:24-35
  trace_ghost_ray / trace_primary_ray          bind_trace.cpp:57-67
  render_point_flare / render_source_flare     bind_renderers.cpp:85-134
Results are torch tensors on the CUDA device (planar float32 (H, W) per
channel, the reference's ``ghost_r/g/b`` keys).  Every device step runs in
libghostlight_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _native
from ._abi import (gl_filter_params, gl_flare_source, gl_ghost_pair, gl_ghost_render_params,
                   gl_pupil_sample, gl_sampler_params, gl_spectral_sample)
from .config import FlareConfig, LensCalibration, PointFlareConfig
from .optics import OpticalSystem, Ray, TraceResult, TraceStatus, Vec3f


def _torch():
    import torch
    return torch


@dataclass(frozen=True)
class GhostPair:
    surf_a: int
    surf_b: int

    def __repr__(self):
        return "GhostPair(%d, %d)" % (self.surf_a, self.surf_b)


# ---------------------------------------------------------------------------
# enumeration / filter
# ---------------------------------------------------------------------------
def enumerate_ghost_pairs(lens: OpticalSystem):
    lib = _native.load()
    arr = lens.to_array()
    n = C.c_int()
    _native.check(lib.gl_enumerate_ghost_pairs(arr, len(arr), None, 0, C.byref(n)), "enumerate_ghost_pairs")
    out = (gl_ghost_pair * max(n.value, 1))()
    _native.check(lib.gl_enumerate_ghost_pairs(arr, len(arr), out, n.value, C.byref(n)), "enumerate_ghost_pairs")
    return [GhostPair(out[i].surf_a, out[i].surf_b) for i in range(n.value)]


@dataclass
class FilterResult:
    pairs: np.ndarray        # (n, 2) int32
    boosts: np.ndarray       # (n,) float32
    footprint_mm: np.ndarray  # (n, 2) float32
    rechecked: int


def filter_ghosts_device(lens: OpticalSystem, sensor_half_w: float, sensor_half_h: float,
                         config: FlareConfig) -> FilterResult:
    lib = _native.load()
    arr = lens.to_array()
    cap = max(1, len(arr) * (len(arr) - 1) // 2)
    pairs = (gl_ghost_pair * cap)()
    boosts = (C.c_float * cap)()
    fp = (C.c_float * (2 * cap))()
    n, rk = C.c_int(), C.c_int()
    prm = gl_filter_params(float(config.min_ghost_intensity), int(bool(config.ghost_normalize)),
                           float(config.max_area_boost))
    _native.check(lib.gl_filter_ghost_pairs(arr, len(arr), float(sensor_half_w), float(sensor_half_h),
                                            C.byref(prm), pairs, boosts, fp, cap, C.byref(n),
                                            C.byref(rk)), "filter_ghost_pairs")
    k = n.value
    p = np.frombuffer(pairs, np.int32).reshape(-1, 2)[:k].copy()
    b = np.frombuffer(boosts, np.float32)[:k].copy()
    f = np.frombuffer(fp, np.float32).reshape(-1, 2)[:k].copy()
    return FilterResult(p, b, f, rk.value)


def filter_ghost_pairs(lens: OpticalSystem, sensor_half_w: float, sensor_half_h: float,
                       config: FlareConfig):
    """(pairs, boosts) like the reference binding (bind_ghost.cpp:28-35)."""
    r = filter_ghosts_device(lens, sensor_half_w, sensor_half_h, config)
    return [GhostPair(int(a), int(b)) for a, b in r.pairs], [float(x) for x in r.boosts]


# ---------------------------------------------------------------------------
# traces
# ---------------------------------------------------------------------------
def trace_rays(lens: OpticalSystem, rays, bounce_a: int = -1, bounce_b: int = -1, stream=None):
    """Batched trace on the device.  rays: (N, 7) float32 CUDA tensor
    (origin, direction, wavelength); returns (N, 5) float32 (x, y, z,
    weight, status).  bounce_b < 0 traces primary rays."""
    torch = _torch()
    lib = _native.load()
    if not (hasattr(rays, "is_cuda") and rays.is_cuda):
        raise ValueError("trace_rays: rays must be a CUDA tensor")
    rays = rays.to(torch.float32).contiguous()
    if rays.dim() != 2 or rays.shape[1] != 7:
        raise ValueError("trace_rays: rays must have shape (N, 7)")
    out = torch.empty((rays.shape[0], 5), dtype=torch.float32, device=rays.device)
    st = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
    arr = lens.to_array()
    _native.check(lib.gl_trace_rays(arr, len(arr), int(bounce_a), int(bounce_b), rays.data_ptr(),
                                    rays.shape[0], out.data_ptr(), st), "trace_rays")
    return out


def _ray_tensor(ray: Ray):
    torch = _torch()
    o, d = ray.origin, ray.dir
    return torch.tensor([[o.x, o.y, o.z, d.x, d.y, d.z, ray.lambda_]], dtype=torch.float32, device="cuda")


def trace_ghost_ray(ray: Ray, lens: OpticalSystem, bounce_a: int, bounce_b: int) -> TraceResult:
    """trace_ghost_ray (bind_trace.cpp:57-63): ValueError on bad indices."""
    n = lens.num_surfaces()
    if bounce_a < 0 or bounce_b < 0 or bounce_a >= bounce_b or bounce_b >= n:
        raise ValueError("bounce indices must satisfy 0 <= bounce_a < bounce_b < num_surfaces")
    r = trace_rays(lens, _ray_tensor(ray), bounce_a, bounce_b).cpu().numpy()[0]
    return TraceResult(Vec3f(r[0], r[1], r[2]), r[3], int(r[4]))


def trace_primary_ray(ray: Ray, lens: OpticalSystem) -> TraceResult:
    r = trace_rays(lens, _ray_tensor(ray), -1, -1).cpu().numpy()[0]
    return TraceResult(Vec3f(r[0], r[1], r[2]), r[3], int(r[4]))


# ---------------------------------------------------------------------------
# host tables
# ---------------------------------------------------------------------------
def spectral_table(n: int, output_cs: int = 0, custom_xyz_to_output=None):
    """(table (n,4) float32 [lambda, cmf_r, cmf_g, cmf_b], correction (3,3))."""
    lib = _native.load()
    n = max(3, int(n))
    out = (gl_spectral_sample * n)()
    corr = (C.c_float * 9)()
    cust = None
    if custom_xyz_to_output is not None:
        cust = (C.c_float * 9)(*np.asarray(custom_xyz_to_output, np.float32).reshape(-1))
    _native.check(lib.gl_build_spectral_table(n, int(output_cs), cust, out, corr), "spectral_table")
    return (np.frombuffer(out, np.float32).reshape(n, 4).copy(),
            np.frombuffer(corr, np.float32).reshape(3, 3).copy())


_grid_cache: dict = {}


def pupil_grid(lens: OpticalSystem, ray_grid: int, jitter: int = 0, seed: int = 0,
               blades_override: int = 0, rotation_deg: float = 0.0) -> np.ndarray:
    """Masked entrance-pupil samples (aperture_sampler.h:180-223), cached."""
    key = (lens.state_key(), ray_grid, jitter, seed, blades_override, float(rotation_deg))
    g = _grid_cache.get(key)
    if g is not None:
        return g
    lib = _native.load()
    arr = lens.to_array()
    sp = gl_sampler_params(int(ray_grid), int(jitter), int(seed), int(blades_override), float(rotation_deg))
    cap = max(1, ray_grid * ray_grid)
    out = (gl_pupil_sample * cap)()
    n = C.c_int()
    _native.check(lib.gl_build_aperture_samples(arr, len(arr), C.byref(sp), out, cap, C.byref(n)), "pupil_grid")
    g = np.frombuffer(out, np.float32).reshape(-1, 2)[:n.value].copy()
    if len(_grid_cache) > 256:
        _grid_cache.clear()
    _grid_cache[key] = g
    return g


def render_order_grid(lens: OpticalSystem, ray_grid: int, jitter: int = 0, seed: int = 0,
                      blades_override: int = 0, rotation_deg: float = 0.0) -> np.ndarray:
    """The same samples as ``pupil_grid`` in the order the batched render
    traces them (gl_morton_order), cached like the grid itself, so a plan
    build only checks the order instead of sorting again."""
    key = ("morton", lens.state_key(), ray_grid, jitter, seed, blades_override, float(rotation_deg))
    g = _grid_cache.get(key)
    if g is not None:
        return g
    base = pupil_grid(lens, ray_grid, jitter, seed, blades_override, rotation_deg)
    src = np.ascontiguousarray(base, np.float32)
    out = np.empty_like(src)
    P = C.POINTER(gl_pupil_sample)
    _native.check(_native.load().gl_morton_order(src.ctypes.data_as(P), len(src), out.ctypes.data_as(P)),
                  "morton_order")
    if len(_grid_cache) > 256:
        _grid_cache.clear()
    _grid_cache[key] = out
    return out


def color_matrices(config):
    lib = _native.load()
    mi, mo = (C.c_float * 9)(), (C.c_float * 9)()
    ci = (C.c_float * 9)(*np.asarray(config.custom_input_to_xyz, np.float32).reshape(-1))
    co = (C.c_float * 9)(*np.asarray(config.custom_xyz_to_output, np.float32).reshape(-1))
    _native.check(lib.gl_color_matrices(int(config.input_cs), ci, int(config.output_cs), co, mi, mo),
                  "color_matrices")
    return np.frombuffer(mi, np.float32).reshape(3, 3), np.frombuffer(mo, np.float32).reshape(3, 3)


def source_rgb(config, r, g, b):
    """input_cs -> XYZ -> output_cs in float32, SourceFlareRenderer.cpp:74-86."""
    f = np.float32
    Mi, Mo = color_matrices(config)
    r, g, b = f(r), f(g), f(b)
    x = [Mi[k, 0] * r + Mi[k, 1] * g + Mi[k, 2] * b for k in range(3)]
    return tuple(float(Mo[k, 0] * x[0] + Mo[k, 1] * x[1] + Mo[k, 2] * x[2]) for k in range(3))


def adaptive_grid_size(footprint_mm, sensor_half_w, sensor_half_h, width, height,
                       gmin=16, gmax=256) -> int:
    """Per-ghost pupil grid side from its probe footprint: about one pupil
    sample per two output pixels across the ghost, rounded up to a multiple of
    16 and clamped to [gmin, gmax]."""
    fx = float(footprint_mm[0]) / (2.0 * sensor_half_w) * width
    fy = float(footprint_mm[1]) / (2.0 * sensor_half_h) * height
    side = 0.5 * math.sqrt(max(fx, 1.0) * max(fy, 1.0))
    g = int(math.ceil(side / 16.0)) * 16
    return int(min(gmax, max(gmin, g)))


# ---------------------------------------------------------------------------
# render plan
# ---------------------------------------------------------------------------
class GhostRenderPlan:
    """Resident device state of one ghost render; ``execute`` only enqueues
    kernels (capturable in a CUDA graph)."""

    def __init__(self, lens: OpticalSystem, pairs, boosts, sources, grids, pair_grid, spec,
                 correction, width, height, sensor_half_w, sensor_half_h, gain,
                 apply_correction=True, plain_per_pair=False, fmt=None, cull_dead_pairs=False,
                 blades_override=0, rotation_deg=0.0):
        lib = _native.load()
        self._lib = lib
        self.width, self.height = int(width), int(height)
        pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        boosts = np.ascontiguousarray(boosts, np.float32).reshape(-1)
        sources = np.ascontiguousarray(sources, np.float32).reshape(-1, 5)
        offs = np.zeros(len(grids) + 1, np.int32)
        for i, g in enumerate(grids):
            offs[i + 1] = offs[i] + len(g)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(g, np.float32).reshape(-1, 2) for g in grids])
                                    if grids else np.zeros((0, 2), np.float32))
        pg = np.ascontiguousarray(pair_grid if pair_grid is not None else np.zeros(len(pairs)), np.int32)
        spec = np.ascontiguousarray(spec, np.float32).reshape(-1, 4)
        prm = gl_ghost_render_params()
        fw, fh, fx0, fy0 = fmt if fmt is not None else (width, height, 0, 0)
        prm.width, prm.height = self.width, self.height
        prm.fmt_w, prm.fmt_h, prm.fmt_x0, prm.fmt_y0 = int(fw), int(fh), int(fx0), int(fy0)
        prm.sensor_half_w, prm.sensor_half_h = float(sensor_half_w), float(sensor_half_h)
        prm.flare_gain = float(gain)
        prm.apply_correction = int(bool(apply_correction))
        for k, v in enumerate(np.asarray(correction, np.float32).reshape(-1)):
            prm.correction[k] = float(v)
        prm.plain_per_pair = int(bool(plain_per_pair))
        prm.cull_dead_pairs = int(bool(cull_dead_pairs))
        prm.blades_override = int(blades_override)
        prm.rotation_deg = float(rotation_deg)
        self.n_pairs = len(pairs)
        P = C.POINTER
        arr = lens.to_array()
        h = C.c_void_p()
        _native.check(lib.gl_ghost_plan_create(
            arr, len(arr), pairs.ctypes.data_as(P(gl_ghost_pair)), boosts.ctypes.data_as(P(C.c_float)),
            pg.ctypes.data_as(P(C.c_int32)), len(pairs), sources.ctypes.data_as(P(gl_flare_source)),
            len(sources), flat.ctypes.data_as(P(gl_pupil_sample)), offs.ctypes.data_as(P(C.c_int32)),
            len(grids), spec.ctypes.data_as(P(gl_spectral_sample)), len(spec), C.byref(prm),
            C.byref(h)), "render_ghosts")
        self._h = h
        rays, items, grid = C.c_longlong(), C.c_int(), C.c_int()
        lib.gl_ghost_plan_info(h, C.byref(rays), C.byref(items), C.byref(grid))
        self.rays = int(rays.value)
        self.n_items = int(items.value)
        self.persistent_ctas = int(grid.value)

    def stats(self, stream=None):
        """Per-pair counters of the diagnostic pass (gl_ghost_plan_stats):
        (n_pairs, 3) uint64 {traces, survived, on sensor}."""
        torch = _torch()
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        n = max(1, len(getattr(self, "pairs", [])) or 1)
        out = np.zeros((n, 3), np.uint64)
        _native.check(self._lib.gl_ghost_plan_stats(self._h, out.ctypes.data_as(C.POINTER(C.c_ulonglong)),
                                                    C.c_void_p(st)), "ghost_plan_stats")
        return out[:len(self.pairs)] if hasattr(self, "pairs") else out

    def execute(self, out_r, out_g, out_b, stream=None):
        torch = _torch()
        for t in (out_r, out_g, out_b):
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
                    and t.numel() == self.width * self.height):
                raise ValueError("render_ghosts: outputs must be contiguous float32 CUDA (H, W) tensors")
        st = stream if stream is not None else torch.cuda.current_stream(out_r.device).cuda_stream
        _native.check(self._lib.gl_ghost_plan_execute(self._h, out_r.data_ptr(), out_g.data_ptr(),
                                                      out_b.data_ptr(), st), "render_ghosts")
        return _native.last_launch_count()

    def set_launch(self, items_per_warp: int = 0, ctas_per_sm: int = 0, lambda_chunks: int = 1):
        """Launch shape of the batched render: 0 = persistent work queue over
        ctas_per_sm CTAs per SM (0 = all resident), > 0 = one-shot CTAs of that
        many 32-sample items per warp; lambda_chunks splits each item's
        wavelengths into that many tasks."""
        _native.check(self._lib.gl_ghost_plan_set_launch(self._h, int(items_per_warp), int(ctas_per_sm)),
                      "set_launch")
        _native.check(self._lib.gl_ghost_plan_set_lambda_split(self._h, int(lambda_chunks)), "set_launch")
        self.launch = (int(items_per_warp), int(ctas_per_sm), int(lambda_chunks))

    def traced(self) -> int:
        """Ray-wavelength traces the last execute ran (render + probes)."""
        v = C.c_longlong()
        _native.check(self._lib.gl_ghost_plan_traced(self._h, C.byref(v)), "traced")
        return int(v.value)

    def traced_split(self):
        """(render, probe) ray-wavelength traces of the last execute."""
        r, q = C.c_longlong(), C.c_longlong()
        _native.check(self._lib.gl_ghost_plan_traced_split(self._h, C.byref(r), C.byref(q)), "traced_split")
        return int(r.value), int(q.value)

    def set_timing(self, ev_probe=None, ev_render=None, ev_end=None):
        """torch.cuda.Event objects (enable_timing=True; None = none) that every
        later execute records before the probe launch, before the render launch
        and after it: ev_render.elapsed_time(ev_end) is the render kernel alone."""
        h = []
        for e in (ev_probe, ev_render, ev_end):
            if e is not None and not e.cuda_event:
                e.record()                       # torch creates its event on first record
            h.append(None if e is None else e.cuda_event)
        _native.check(self._lib.gl_ghost_plan_set_timing(self._h, *h), "set_timing")
        self._timing = (ev_probe, ev_render, ev_end)     # keep the events alive

    def pair_hits(self):
        """Probe hits per pair from the last execute (0 = culled)."""
        out = (C.c_int32 * max(1, self.n_pairs))()
        _native.check(self._lib.gl_ghost_plan_pair_hits(self._h, out, max(1, self.n_pairs)), "pair_hits")
        return np.frombuffer(out, np.int32)[: self.n_pairs].copy()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gl_ghost_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prepare_ghost_render(lens: OpticalSystem, sources, width: int, height: int, config: FlareConfig,
                         sensor_half_w: float, sensor_half_h: float, *, plain_per_pair=False,
                         stop_crossing_filter=None, filter_result: FilterResult | None = None):
    """Filter -> grids -> resident plan.  sources: (N, 5) [angle_x, angle_y,
    r, g, b] with r, g, b already in the output colour space."""
    fr = filter_result if filter_result is not None else filter_ghosts_device(
        lens, sensor_half_w, sensor_half_h, config)
    pairs, boosts, fps = fr.pairs, fr.boosts, fr.footprint_mm
    # GhostFilter include / exclude (ghost_render.cu:1491-1518), order kept.
    gf = config.ghost_filter
    if int(gf.mode) != 0 and gf.pairs:
        want = {(int(a), int(b)) for a, b in gf.pairs}
        keep = [((int(a), int(b)) in want) == (int(gf.mode) == 1) for a, b in pairs]
        keep = np.asarray(keep, bool)
        pairs, boosts, fps = pairs[keep], boosts[keep], fps[keep]
    if stop_crossing_filter is not None:
        keep = np.asarray([not stop_crossing_filter(int(a), int(b)) for a, b in pairs], bool)
        pairs, boosts, fps = pairs[keep], boosts[keep], fps[keep]
    ns = max(3, int(config.spectral_samples))
    spec, corr = spectral_table(ns, int(config.output_cs), config.custom_xyz_to_output)
    apply_corr = bool(config.spectral_correction) and ns != 3
    jitter, seed = int(config.pupil_jitter), int(config.jitter_seed)
    bo, rot = int(config.aperture_blades), float(config.aperture_rotation)
    if getattr(config, "adaptive_grids", False):
        sizes = [adaptive_grid_size(fp, sensor_half_w, sensor_half_h, width, height,
                                    config.adaptive_grid_min, config.adaptive_grid_max) for fp in fps]
        uniq = sorted(set(sizes))
        grids = [render_order_grid(lens, g, jitter, seed, bo, rot) for g in uniq]
        pair_grid = np.asarray([uniq.index(s) for s in sizes], np.int32)
    else:
        uniq = [int(config.ray_grid)]
        grids = [render_order_grid(lens, int(config.ray_grid), jitter, seed, bo, rot)]
        pair_grid = np.zeros(len(pairs), np.int32)
    plan = GhostRenderPlan(lens, pairs, boosts, sources, grids, pair_grid, spec, corr, width, height,
                           sensor_half_w, sensor_half_h, config.flare_gain, apply_corr, plain_per_pair,
                           cull_dead_pairs=bool(config.cull_dead_pairs), blades_override=bo,
                           rotation_deg=rot)
    plan.pairs, plan.boosts, plan.grids, plan.pair_grid = pairs, boosts, grids, pair_grid
    plan.grid_sides = list(uniq)
    plan.spec, plan.correction, plan.apply_correction = spec, corr, apply_corr
    return plan


def render_ghosts(lens: OpticalSystem, sources, width: int, height: int, config: FlareConfig,
                  sensor_half_w: float, sensor_half_h: float, *, plain_per_pair=False,
                  stop_crossing_filter=None, stream=None):
    """Ghost layer for explicit field-angle sources (the FlareSource form of
    launch_ghost_render).  Returns {"ghost_r", "ghost_g", "ghost_b"} tensors."""
    import time
    torch = _torch()
    if width <= 0 or height <= 0:
        raise ValueError("render_ghosts: width and height must be positive")
    t0 = time.perf_counter()
    plan = prepare_ghost_render(lens, sources, width, height, config, sensor_half_w, sensor_half_h,
                                plain_per_pair=plain_per_pair, stop_crossing_filter=stop_crossing_filter)
    t1 = time.perf_counter()
    out = {k: torch.zeros((height, width), dtype=torch.float32, device="cuda")
           for k in ("ghost_r", "ghost_g", "ghost_b")}
    if bool(getattr(config, "collect_stats", False)) and int(getattr(config, "aov_mode", 0)) != 1:
        torch.cuda.current_stream().synchronize()
        t2 = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        if len(plan.pairs):
            plan.execute(out["ghost_r"], out["ghost_g"], out["ghost_b"], stream)
        e1.record()
        e1.synchronize()
        cnt = plan.stats() if len(plan.pairs) else np.zeros((0, 3), np.uint64)
        t3 = time.perf_counter()
        out["stats"] = {
            "ms_grid_build": 1e3 * (t1 - t0), "ms_upload": 1e3 * (t2 - t1), "ms_kernel": float(e0.elapsed_time(e1)),
            "ms_download": 0.0, "ms_total": 1e3 * (t3 - t0),
            "n_pairs": int(len(plan.pairs)), "n_sources": int(np.asarray(sources).reshape(-1, 5).shape[0]),
            "n_grid": int(max((len(g) for g in plan.grids), default=0)), "n_spec": int(len(plan.spec)),
            "traces_total": int(cnt[:, 0].sum()), "traces_survived": int(cnt[:, 1].sum()),
            "traces_on_sensor": int(cnt[:, 2].sum()),
            "pair_surf_a": [int(a) for a, _ in plan.pairs], "pair_surf_b": [int(b) for _, b in plan.pairs],
            "pair_traces": [int(v) for v in cnt[:, 0]], "pair_survived": [int(v) for v in cnt[:, 1]],
            "pair_on_sensor": [int(v) for v in cnt[:, 2]], "ps_hits": [], "ps_rect": [], "ps_budget": []}
        plan.close()
        return out
    if int(getattr(config, "aov_mode", 0)) == 1 and len(plan.pairs):
        plan.close()
        out.update(_render_aov_layers(lens, plan, sources, width, height, config, sensor_half_w, sensor_half_h,
                                      out, stream))
        return out
    if len(plan.pairs):
        plan.execute(out["ghost_r"], out["ghost_g"], out["ghost_b"], stream)
    torch.cuda.current_stream().synchronize()
    plan.close()
    return out


def _render_aov_layers(lens, plan, sources, width, height, config, sensor_half_w, sensor_half_h, out, stream):
    """GhostAovMode.PER_PAIR (ghost_render.cu:1526-1563): each of the first
    aov_max_pairs (all when < 0) active pairs rendered on its own, without
    the off-sensor cull, into ghost_s{a}_s{b}_{r,g,b}; the combined ghost
    planes are the sum of those layers."""
    torch = _torch()
    n = len(plan.pairs) if int(config.aov_max_pairs) < 0 else min(len(plan.pairs), int(config.aov_max_pairs))
    layers = {}
    for i in range(n):
        a, b = (int(v) for v in plan.pairs[i])
        planes = [torch.zeros((height, width), dtype=torch.float32, device="cuda") for _ in range(3)]
        one = GhostRenderPlan(lens, plan.pairs[i:i + 1], plan.boosts[i:i + 1], sources, plan.grids,
                              plan.pair_grid[i:i + 1], plan.spec, plan.correction, width, height, sensor_half_w,
                              sensor_half_h, config.flare_gain, plan.apply_correction, False,
                              cull_dead_pairs=False, blades_override=int(config.aperture_blades),
                              rotation_deg=float(config.aperture_rotation))
        one.execute(*planes, stream)
        torch.cuda.current_stream().synchronize()
        one.close()
        for c, pl in zip("rgb", planes):
            layers["ghost_s%d_s%d_%s" % (a, b, c)] = pl
            out["ghost_" + c] += pl
    torch.cuda.current_stream().synchronize()
    return layers


def _eff_half(config, calib: LensCalibration):
    hw = config.sensor_half_w if config.sensor_half_w > 0 else calib.sensor_half_w
    hh = config.sensor_half_h if config.sensor_half_h > 0 else calib.sensor_half_h
    return float(hw), float(hh)


def render_source_flare(offsets, width: int, height: int, lens: OpticalSystem,
                        calibration: LensCalibration, config: PointFlareConfig, *, source_angle=None):
    """render_source_flare (SourceFlareRenderer.cpp:24-208), ghost layer.

    offsets: (N, 3) [d_angle_x, d_angle_y, weight] around the source centre.
    The centre is config.source_x/y solved to a field angle
    (source_map.cpp:182); pass ``source_angle=(ax, ay)`` to give it directly.
    """
    if width <= 0 or height <= 0:
        raise ValueError("render_source_flare: width and height must be positive")
    off = np.ascontiguousarray(offsets, np.float32)
    if off.ndim != 2 or off.shape[1] != 3 or off.shape[0] < 1:
        raise ValueError("render_source_flare: offsets must be a (N, 3) float32 array of "
                         "[d_angle_x, d_angle_y, weight] rows with N >= 1")
    if not np.isfinite(off).all():
        raise ValueError("render_source_flare: source offsets must be finite")
    if lens.num_surfaces() <= 0:
        raise ValueError("render_source_flare: lens has no surfaces")
    hw, hh = _eff_half(config, calibration)
    smap = None
    if source_angle is None:
        from .calibration import solve_source_angle
        f = np.float32
        smap = solve_source_angle(lens, calibration, float((f(config.source_x) - f(0.5)) * f(2.0)),
                                  float((f(config.source_y) - f(0.5)) * f(2.0)), hw, hh,
                                  precision=getattr(config, "setup_precision", "fp32"))
        ax0, ay0 = smap.angle_x, smap.angle_y
    else:
        ax0, ay0 = source_angle
    r, g, b = source_rgb(config, config.source_r, config.source_g, config.source_b)
    f = np.float32
    src = np.zeros((off.shape[0], 5), np.float32)
    for i, (dx, dy, w) in enumerate(off):
        src[i] = (f(ax0) + dx, f(ay0) + dy, f(r) * w, f(g) * w, f(b) * w)
    out = render_ghosts(lens, src, width, height, config, hw, hh)
    dc = getattr(config, "diffraction", None)
    want_sb = dc is not None and getattr(dc, "starburst", False)
    want_veil = dc is not None and getattr(dc, "veil", False)
    pos = None
    if want_sb or want_veil:
        # each source's image point, from the solve's forward map
        # (SourceFlareRenderer.cpp:105-118) or the paraxial map when the angle
        # was given directly
        pos = np.zeros((len(src), 5), np.float32)
        for i in range(len(src)):
            if smap is not None:
                sx, sy = smap.screen(float(src[i, 0]), float(src[i, 1]))
            else:
                sx = 0.5 + 0.5 * math.tan(float(src[i, 0])) / math.tan(calibration.max_half_angle_h) \
                    * calibration.sensor_half_w / hw
                sy = 0.5 + 0.5 * math.tan(float(src[i, 1])) / math.tan(calibration.max_half_angle_v) \
                    * calibration.sensor_half_h / hh
            pos[i] = (sx * width, sy * height, src[i, 2], src[i, 3], src[i, 4])
    if want_sb:
        field = (float(np.float32(np.mean(src[:, 0].astype(np.float64)))),
                 float(np.float32(np.mean(src[:, 1].astype(np.float64)))))
        out.update(starburst_layer_for(lens, calibration, config, pos, width, height, hw, hh, field)[0])
    if want_veil:
        from .veil import render_veil
        out.update(render_veil(pos, width, height, hw, hh, dc.veil_spread, dc.veil_falloff, dc.veil_gain))
    return out


def starburst_layer_for(lens, calibration, config, pos, width: int, height: int, hw: float, hh: float, field):
    """The starburst layer for sources at buffer pixels ``pos`` ((N, 5) px,
    py, r, g, b) whose mean direction is ``field``, with the engine
    render_starburst picks (starburst_render.cu:646-711): the SPRITE engine by
    default and whenever the pattern is prominent or the grid grows; the
    matrix-DFT engine otherwise when asked for, in the reference's
    pixel-integrated form (or the field form when diffraction.mdft_form ==
    "field").  Returns (layer dict, sprite geometry)."""
    from .starburst import mdft_box_starburst_layer, sprite_geometry, sprite_starburst_layer, starburst_layer
    dc = config.diffraction
    geo = sprite_geometry(calibration, config, pos, width, height, hw, hh,
                          front_R=lens.surfaces[0].semi_aperture if lens.surfaces else 0.0)
    if geo["engine"] == "sprite":
        layer = sprite_starburst_layer(lens, calibration, config, pos, width, height, hw, hh, geometry=geo,
                                       field=field)
    elif getattr(dc, "mdft_form", "pixel") == "field":
        layer = starburst_layer(lens, calibration, config, pos, width, height, hw, hh)
    else:
        layer = mdft_box_starburst_layer(lens, calibration, config, pos, width, height, hw, hh, geometry=geo,
                                         field=field)
    return layer, geo


def render_point_flare(width: int, height: int, lens: OpticalSystem, calibration: LensCalibration,
                       config: PointFlareConfig, *, source_angle=None):
    """render_point_flare (PointFlareRenderer.cpp:11-20): one zero offset."""
    return render_source_flare(np.array([[0.0, 0.0, 1.0]], np.float32), width, height, lens,
                               calibration, config, source_angle=source_angle)

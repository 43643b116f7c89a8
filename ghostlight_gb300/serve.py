"""Flare request serving on one GPU: resident lenses, continuous batching.

A request (lens, output size, wavelength count, pupil grid, source field)
renders the ghost layer of one point source.  The server keeps every
registered lens resident in HBM (gl_lens: packed surfaces, filtered pairs,
probe grids, cached IOR slices and pupil grids) and admits requests as they
arrive whenever a slot and enough of the HBM budget are free — not in
batches: a request that arrives while others are on the GPU starts at once on
its own CUDA stream, and its kernels share the SMs with theirs.  Requests run
as short CTAs (``items_per_warp`` items of 32 pupil samples per warp), so the
CTA scheduler interleaves them at CTA boundaries, preferring streams of higher
priority; the priority is the request's estimated trace count (shortest job
first by default; ``policy="lsf"`` reverses it).  Every request's device memory comes from a stream-ordered pool, and
nothing on the request path synchronises the device.

The reference has no serving layer: it renders one flare per blocking call
(bind_renderers.cpp:85-134 -> ghost_render.cu:630) under process-wide mutexes
(ghost_render.cu:504-511).

``Scheduler`` holds the admission policy and is pure Python (tested on the
CPU with a fake executor); ``CudaExecutor`` runs requests through the C-ABI.
"""
from __future__ import annotations

import collections
import ctypes as C
import dataclasses
import math
import time
from typing import Callable, Dict, List, Optional

import numpy as np

from . import _native
from ._abi import gl_flare_source, gl_ghost_pair, gl_ghost_render_params, gl_spectral_sample


@dataclasses.dataclass
class FlareRequest:
    lens_id: int
    width: int
    height: int
    n_spec: int
    ray_grid: int
    field_deg: float
    gain: float = 1000.0
    rid: int = 0
    starburst: bool = False         # add the starburst layer (the lens's resident SPRITE starburst)
    arrival: float = 0.0            # seconds on the serving clock
    # kind "psf": a PSF atlas (render_psf, PSFRenderer.cpp:260) of psf_grid^2
    # sources on a regular grid over psf_field_frac of the lens's covered
    # field, each in its own psf_tile^2 tile (width = height = psf_grid psf_tile)
    kind: str = "flare"
    psf_grid: int = 4
    psf_tile: int = 64
    psf_extent_mm: float = 0.4
    psf_field_frac: float = 0.7
    # filled by the server
    est_rays: int = 0
    device_bytes: int = 0
    priority: int = 0
    start: float = 0.0
    finish: float = 0.0
    traced: int = 0                 # ray-wavelength traces the device ran
    deferred: bool = False          # waited at least once for HBM budget
    rejected: bool = False          # needs more than the whole budget: never admitted

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


# ---------------------------------------------------------------------------
# admission policy (no CUDA)
# ---------------------------------------------------------------------------
class Scheduler:
    """Admit pending requests oldest first, skipping ahead past a request that
    does not fit the remaining HBM budget (so one large request cannot block
    small ones behind it while memory is short), never more than
    ``max_inflight`` at once."""

    def __init__(self, budget_bytes: int, max_inflight: int):
        if budget_bytes <= 0 or max_inflight <= 0:
            raise ValueError("scheduler: budget and slot count must be positive")
        self.budget = int(budget_bytes)
        self.max_inflight = int(max_inflight)
        self.used = 0
        self.inflight = 0
        self.pending: collections.deque = collections.deque()
        self.peak_used = 0
        self.peak_inflight = 0

    def submit(self, req: FlareRequest):
        if req.device_bytes > self.budget:
            raise ValueError("request %d needs %d bytes, above the %d-byte budget"
                             % (req.rid, req.device_bytes, self.budget))
        self.pending.append(req)

    def admit(self) -> List[FlareRequest]:
        out = []
        if not self.pending or self.inflight >= self.max_inflight:
            return out
        keep = collections.deque()
        while self.pending:
            r = self.pending.popleft()
            if self.inflight < self.max_inflight and self.used + r.device_bytes <= self.budget:
                self.used += r.device_bytes
                self.inflight += 1
                out.append(r)
            else:
                if self.inflight < self.max_inflight:
                    r.deferred = True       # a slot was free: the budget held it back
                keep.append(r)
        self.pending = keep
        self.peak_used = max(self.peak_used, self.used)
        self.peak_inflight = max(self.peak_inflight, self.inflight)
        return out

    def release(self, req: FlareRequest):
        self.used -= req.device_bytes
        self.inflight -= 1
        assert self.used >= 0 and self.inflight >= 0


POLICIES = ("sjf", "lsf", "sjf_fifo")


def size_class(est_rays: int, rays_per_s: float = 7e9) -> int:
    """Estimated service time class: < 1 ms -> 0, < 4 ms -> 1, < 16 ms -> 2, else 3."""
    t = est_rays / rays_per_s
    return 0 if t < 1e-3 else 1 if t < 4e-3 else 2 if t < 16e-3 else 3


def _light_levels(greatest: int, least: int) -> int:
    """How many of the device's stream priority levels the three short
    classes take under ``sjf_fifo`` (the rest rank the long requests): three
    when there are six or more levels, two with four or five (the two
    shortest classes share the top level), one otherwise."""
    n = least - greatest + 1
    return 3 if n >= 6 else (2 if n >= 4 else 1)


def fifo_light_level(cls: int, greatest: int, least: int) -> int:
    """Stream priority of a short request (size class 0..2) under ``sjf_fifo``."""
    k = _light_levels(greatest, least)
    return greatest + max(0, cls - (3 - k))


def fifo_heavy_level(heavy_inflight_levels, greatest: int, least: int) -> int:
    """Stream priority of a new long request under ``sjf_fifo``: the levels
    below the short classes rank the long requests in flight by arrival — a
    new one takes the level after the youngest one running (the lowest level
    once they run out), so the oldest long request keeps the SMs the short
    ones leave, instead of every long request sharing them equally and all
    finishing late."""
    first = min(least, greatest + _light_levels(greatest, least))
    if not heavy_inflight_levels:
        return first
    return min(least, max(heavy_inflight_levels) + 1)


def priority_class(est_rays: int, rays_per_s: float = 7e9, policy: str = "sjf") -> int:
    """Stream priority (lower = sooner) from the estimated service time class
    c: < 1 ms -> 0, < 4 ms -> 1, < 16 ms -> 2, else 3.

    sjf (shortest job first): priority c - 3, so short requests overtake long
    ones; the tail is the long requests, starved while short ones keep coming.
    lsf (least slack first, for a common latency target): priority -c, so a
    long request, whose service time alone is closest to the target, takes the
    SMs first and short ones fill the CTA slots it leaves; the tail is the
    short requests that arrive behind a long one."""
    if policy not in POLICIES:
        raise ValueError("priority policy must be one of %s" % (POLICIES,))
    c = size_class(est_rays, rays_per_s)
    return -c if policy == "lsf" else c - 3


def lambda_split(n_spec: int) -> int:
    """Wavelength ranges per 32-sample item the library uses by default (about
    eight wavelengths per task: 31 -> 4, 16 -> 2, 8 -> 1)."""
    return max(1, min(int(n_spec), (int(n_spec) + 4) // 8))


STARBURST_PUPIL, STARBURST_FILL = 256, 0.30


class StarburstPlans:
    """Resident DFT matrices of the serving starburst layer: one split-BF16
    MdftPlan per (width, height, spectral table), shared by every lens (each
    lens brings its own unit-sum stop pupil).  The pattern is scaled like the
    anamorphic sweep's, so the 400 nm period spans the frame width, and is
    centred per request on the plan's own stream (set_center rebuilds the
    matrices), which orders the requests that share a plan.  The streams run
    at the highest priority (the GEMMs are short), and the GEMMs use `ctas`
    CTAs (a quarter of the SMs by default), so the ghost layers of the
    requests in flight keep the other SMs: measured at 200 req/s, 38 CTAs cut
    the p99 from 125 to 104 ms against one CTA per SM.  (Writing the pattern
    first, with the ghost flush adding onto it, and plans per priority level
    were measured too: p99 148 and 185 ms.)"""

    def __init__(self, device=None, ctas: Optional[int] = None):
        import torch
        self.torch = torch
        self.device = device
        if ctas is None:
            sms = torch.cuda.get_device_properties(device if device is not None else 0).multi_processor_count
            ctas = max(1, sms // 4)
        self.ctas = int(ctas)          # GEMM CTAs per plan (0: one per SM)
        lo, hi = torch.cuda.Stream.priority_range()
        self.priority = min(lo, hi)
        self.plans: Dict[tuple, tuple] = {}

    @staticmethod
    def chunks(width: int, height: int, n_spec: int) -> int:
        """Wavelength ranges a pattern is enqueued in: one below 2048^2; the
        larger patterns in ranges of about four (2048^2) or two (4096^2)
        wavelengths, so their GEMM CTAs give the SMs back between ranges and
        the smaller patterns behind them start within a fraction of a
        millisecond instead of after the whole pattern."""
        px = int(width) * int(height)
        per = 0 if px < 2048 * 2048 else (4 if px < 4096 * 4096 else 2)
        return 1 if per == 0 else max(1, -(-int(n_spec) // per))

    def get(self, width: int, height: int, spec: np.ndarray):
        from .starburst import MdftPlan
        spec = np.ascontiguousarray(spec, np.float32).reshape(-1, 4)
        key = (int(width), int(height), spec.tobytes())
        hit = self.plans.get(key)
        if hit is None:
            lam = spec[:, 0].astype(np.float64)
            s = lam.min() / lam
            # the smaller the pattern the higher its stream's priority
            px = int(width) * int(height)
            lower = 0 if px <= 1024 * 1024 else (1 if px <= 2048 * 2048 else 2)
            lo, hi = self.torch.cuda.Stream.priority_range()
            prio = self.priority + lower if self.priority < max(lo, hi) else self.priority
            prio = min(prio, max(lo, hi))
            st = self.torch.cuda.Stream(device=self.device, priority=prio)
            plan = MdftPlan(STARBURST_PUPIL, (int(width), int(height)), s / width, s / height,
                            spec[:, 1:4], "split_bf16", stream=st.cuda_stream)
            if self.ctas > 0:
                plan.set_launch(self.ctas)
            st.synchronize()
            hit = (plan, st)
            self.plans[key] = hit
        return hit

    def close(self):
        for plan, _ in self.plans.values():
            plan.close()
        self.plans = {}


class SpriteStarbursts:
    """The serving starburst layer by the reference's default SPRITE engine
    (render_starburst, starburst_render.cu:594-1073): per (lens, output size,
    wavelength count) the stop pupil's FFT is baked over the spectrum and
    box-summed toward the output pitch once, with the physical scale of the
    lens's first-order optics (sprite_geometry), and only the M x M x 3 sprite
    stays resident.  Each request splats it at its source's image point on
    the request's own stream (gl_sprite_splat_source: the source passed by
    value, nothing staged or shared), so requests that use one sprite run side
    by side.  The pupil is the plain stop, without the field-dependent
    cat's-eye, as for the matrix-DFT serving layer."""

    def __init__(self):
        self.sprites: Dict[tuple, tuple] = {}

    def get(self, lens_id: int, rl, width: int, height: int, n_spec: int):
        key = (int(lens_id), int(width), int(height), int(n_spec))
        hit = self.sprites.get(key)
        if hit is None:
            hit = self._bake(rl, int(width), int(height), int(n_spec))
            self.sprites[key] = hit
        return hit

    @staticmethod
    def config_for(rl, n_spec: int):
        from .config import DiffractionConfig
        cfg = dataclasses.replace(rl.config)
        cfg.spectral_samples = int(n_spec)
        cfg.diffraction = DiffractionConfig(starburst=True, spectral_samples=int(n_spec), use_survivor_mask=False)
        return cfg

    def _bake(self, rl, width: int, height: int, n_spec: int):
        import torch
        from .starburst import _PLAN_LOCK, _sprite_plan, build_pupil2, sprite_geometry, starburst_spectrum
        cfg = self.config_for(rl, n_spec)
        centre = np.array([[0.5 * width, 0.5 * height, 1.0, 1.0, 1.0]], np.float32)
        front_r = rl.lens.surfaces[0].semi_aperture if rl.lens.surfaces else 0.0
        g = sprite_geometry(rl.calibration, cfg, centre, width, height, rl.sensor_half_w, rl.sensor_half_h,
                            front_R=front_r)
        spec = starburst_spectrum(cfg)
        with _PLAN_LOCK:
            plan, baked = _sprite_plan(g["N"], spec)
            pupil = build_pupil2(rl.lens, g["N"], g["fill"], int(cfg.aperture_blades), float(cfg.aperture_rotation))
            plan.bake(pupil, g["ds"])
            _, sprite, _ = plan.read()
            baked.clear()                   # the shared plan no longer holds a frame render's bake
            torch.cuda.current_stream().synchronize()
        return sprite, int(sprite.shape[0]), g

    def device_bytes(self) -> int:
        return sum(int(sp.numel()) * 4 for sp, _, _ in self.sprites.values())

    def close(self):
        self.sprites = {}


def request_bytes(width: int, height: int, n_pairs: int, host_copy: bool = True) -> int:
    """HBM a request holds: RGBA accumulator + three output planes + tables."""
    px = int(width) * int(height)
    return px * 16 + px * 12 + 4 * max(1, n_pairs) + 16384


# ---------------------------------------------------------------------------
# resident lens
# ---------------------------------------------------------------------------
class ResidentLens:
    """gl_lens: a lens with its filtered ghost pairs kept on the device."""

    def __init__(self, lens, sensor_half_w: float, sensor_half_h: float, config, pairs=None, boosts=None,
                 calibration=None):
        from .flare import filter_ghosts_device
        self._lib = _native.load()
        self.lens = lens
        self._calibration = calibration
        self.sensor_half_w, self.sensor_half_h = float(sensor_half_w), float(sensor_half_h)
        self.config = config
        if pairs is None:
            fr = filter_ghosts_device(lens, sensor_half_w, sensor_half_h, config)
            pairs, boosts = fr.pairs, fr.boosts
        self.pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        self.boosts = np.ascontiguousarray(boosts, np.float32).reshape(-1)
        arr = lens.to_array()
        P = C.POINTER
        h = C.c_void_p()
        _native.check(self._lib.gl_lens_create(arr, len(arr), self.pairs.ctypes.data_as(P(gl_ghost_pair)),
                                               self.boosts.ctypes.data_as(P(C.c_float)), len(self.pairs),
                                               int(config.aperture_blades), float(config.aperture_rotation),
                                               C.byref(h)), "lens_create")
        self._h = h
        # host pre-pass cells and pupil grids of PSF atlases (psf_inputs'
        # cache): they depend only on this lens and the atlas's sources
        self.psf_cache: dict = {}

    @property
    def n_pairs(self) -> int:
        return len(self.pairs)

    @property
    def calibration(self):
        """The lens's calibration (calibrate_lens), computed on first use."""
        if self._calibration is None:
            from .calibration import calibrate_lens
            self._calibration = calibrate_lens(self.lens)
        return self._calibration

    def starburst_pupil(self):
        """The stop pupil the starburst layer transforms (STARBURST_PUPIL^2,
        4x4 supersampled on the device, fill STARBURST_FILL), scaled to unit
        sum so every lens's pattern has the same zero-order peak; built once."""
        if getattr(self, "_pupil", None) is None:
            from .starburst import build_pupil
            p = build_pupil(self.lens, STARBURST_PUPIL, STARBURST_FILL, int(self.config.aperture_blades),
                            float(self.config.aperture_rotation))
            amp = float(p.double().sum())
            self._pupil = p / amp if amp > 0 else p
            import torch
            torch.cuda.current_stream().synchronize()      # used on other streams from here on
        return self._pupil

    def image_point(self, field_deg: float, width: int, height: int):
        """Pixel of the paraxial image of a source at field_deg along x."""
        fx = float(getattr(self, "focal_x", 0.0) or 0.0)
        x = fx * math.tan(math.radians(field_deg))
        return (x / (2.0 * self.sensor_half_w) + 0.5) * width, 0.5 * height

    def prepare(self, ray_grid: int, spec: Optional[np.ndarray] = None):
        P = C.POINTER
        sp = None if spec is None else np.ascontiguousarray(spec, np.float32).reshape(-1, 4)
        _native.check(self._lib.gl_lens_prepare(self._h, int(ray_grid),
                                                None if sp is None else sp.ctypes.data_as(P(gl_spectral_sample)),
                                                0 if sp is None else len(sp)), "lens_prepare")

    def device_bytes(self) -> int:
        n, b = C.c_int(), C.c_longlong()
        _native.check(self._lib.gl_lens_info(self._h, C.byref(n), C.byref(b)), "lens_info")
        return int(b.value)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gl_lens_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_spec_cache: Dict[int, tuple] = {}


def _spectral(n_spec: int, config):
    from .flare import spectral_table
    key = (int(n_spec), int(config.output_cs))
    v = _spec_cache.get(key)
    if v is None:
        v = spectral_table(n_spec, int(config.output_cs), config.custom_xyz_to_output)
        _spec_cache[key] = v
    return v


def render_params(rl: ResidentLens, req: FlareRequest, correction, apply_correction: bool):
    prm = gl_ghost_render_params()
    prm.width, prm.height = int(req.width), int(req.height)
    prm.fmt_w, prm.fmt_h, prm.fmt_x0, prm.fmt_y0 = int(req.width), int(req.height), 0, 0
    prm.sensor_half_w, prm.sensor_half_h = rl.sensor_half_w, rl.sensor_half_h
    prm.flare_gain = float(req.gain)
    prm.apply_correction = int(bool(apply_correction))
    for k, v in enumerate(np.asarray(correction, np.float32).reshape(-1)):
        prm.correction[k] = float(v)
    prm.plain_per_pair = 0
    prm.cull_dead_pairs = int(bool(rl.config.cull_dead_pairs))
    prm.blades_override = int(rl.config.aperture_blades)
    prm.rotation_deg = float(rl.config.aperture_rotation)
    return prm


# ---------------------------------------------------------------------------
# CUDA executor
# ---------------------------------------------------------------------------
class _Running:
    __slots__ = ("req", "handle", "stream", "outs", "host", "event", "psf", "prep")


class CudaExecutor:
    """Creates, enqueues and completes requests through gl_request_*.  Each
    in-flight request owns a stream (one pool of streams per priority level);
    its result is copied into pinned host memory on that stream."""

    def __init__(self, lenses: Dict[int, ResidentLens], max_inflight: int, items_per_warp: int = 8,
                 host_output: bool = True, device=None, policy: str = "sjf", lambda_chunks: Optional[int] = None):
        import torch
        if policy not in POLICIES:
            raise ValueError("priority policy must be one of %s" % (POLICIES,))
        self.policy = policy
        self.lambda_chunks = lambda_chunks      # None: the library's default split per request
        self.torch = torch
        lo, hi = torch.cuda.Stream.priority_range()
        self.least, self.greatest = max(lo, hi), min(lo, hi)      # e.g. 0 and -5
        if policy == "sjf_fifo":
            self.LEVELS = tuple(range(self.least, self.greatest - 1, -1))
        else:
            self.LEVELS = tuple(lv for lv in (0, -1, -2, -3) if lv >= self.greatest)
        self._heavy: Dict[int, int] = {}         # id(run) -> level of a long request in flight
        # the starburst layer's engine: "sprite" (the reference's default:
        # resident baked sprites, one splat per request) or "mdft" (the
        # split-BF16 matrix DFT of the field over the whole frame)
        self.starburst_engine = "sprite"
        self.sprites = SpriteStarbursts()
        self.starburst: Optional[StarburstPlans] = None    # created on the first matrix-DFT starburst request
        self.starburst_ctas: Optional[int] = None            # None: a quarter of the SMs
        self._lib = _native.load()
        self.lenses = lenses
        self.items_per_warp = int(items_per_warp)
        self.host_output = bool(host_output)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.streams = {lv: [torch.cuda.Stream(device=self.device, priority=lv) for _ in range(max_inflight)]
                        for lv in self.LEVELS}
        self.free_streams = {lv: list(v) for lv, v in self.streams.items()}
        self._prep_pool = None                   # worker thread of the PSF host pre-passes
        self._pinned: Dict[tuple, list] = collections.defaultdict(list)

    def cta_items(self, req: FlareRequest) -> int:
        """Tasks per warp for this request's CTAs: about the same CTA lifetime
        for every request (a task costs ~ its wavelengths x surfaces; the
        library splits an item's wavelengths into lambda_split(n_spec)
        tasks), so the CTA scheduler can hand SMs to a higher-priority stream
        often."""
        if self.items_per_warp <= 0:
            return 0
        n_surf = len(self.lenses[req.lens_id].lens.surfaces)
        split = self.lambda_chunks if self.lambda_chunks is not None else lambda_split(req.n_spec)
        cost = max(1.0, (req.n_spec / min(split, req.n_spec)) * n_surf / 80.0)
        return max(1, int(round(self.items_per_warp / cost)))

    def estimate(self, req: FlareRequest) -> None:
        rl = self.lenses[req.lens_id]
        masked = 0.8 * req.ray_grid * req.ray_grid
        if req.kind == "psf":
            # primary rays only: the atlas's tiles x pupil samples x wavelengths
            req.est_rays = int(req.psf_grid * req.psf_grid * masked * req.n_spec)
            req.priority = max(self.greatest, priority_class(req.est_rays, policy="sjf" if self.policy != "lsf"
                                                             else "lsf"))
            req.device_bytes = 3 * 4 * req.width * req.height * 2 + (1 << 20)
            return
        req.est_rays = int(rl.n_pairs * masked * req.n_spec)
        if self.policy == "sjf_fifo":
            c = size_class(req.est_rays)
            req.priority = (fifo_light_level(c, self.greatest, self.least) if c < 3
                            else self.least)                                  # long: ranked at start()
        else:
            req.priority = max(self.greatest, priority_class(req.est_rays, policy=self.policy))
        req.device_bytes = request_bytes(req.width, req.height, rl.n_pairs)

    def _pinned_buf(self, shape):
        lst = self._pinned[shape]
        if lst:
            return lst.pop()
        return self.torch.empty(shape, dtype=self.torch.float32, pin_memory=True)

    def close(self):
        """Stop the PSF pre-pass worker (after the pre-passes it holds)."""
        if self._prep_pool is not None:
            self._prep_pool.shutdown(wait=True)
            self._prep_pool = None

    def recycle(self, host):
        if host is not None:
            self._pinned[tuple(host.shape)].append(host)

    def start(self, req: FlareRequest) -> _Running:
        torch = self.torch
        rl = self.lenses[req.lens_id]
        heavy = self.policy == "sjf_fifo" and size_class(req.est_rays) == 3
        if heavy:
            req.priority = fifo_heavy_level(list(self._heavy.values()), self.greatest, self.least)
        lv = req.priority if req.priority in self.free_streams else self.least
        pool = self.free_streams[lv]
        stream = pool.pop() if pool else torch.cuda.Stream(device=self.device, priority=lv)
        if req.kind == "psf":
            return self._start_psf(req, rl, lv, stream)
        spec, corr = _spectral(req.n_spec, rl.config)
        apply_corr = bool(rl.config.spectral_correction) and req.n_spec != 3
        prm = render_params(rl, req, corr, apply_corr)
        src = np.array([[math.radians(req.field_deg), 0.0, 1.0, 1.0, 1.0]], np.float32)
        P = C.POINTER
        st = stream.cuda_stream
        h = C.c_void_p()
        sp = np.ascontiguousarray(spec, np.float32)
        _native.check(self._lib.gl_request_create(rl._h, int(req.ray_grid), sp.ctypes.data_as(P(gl_spectral_sample)),
                                                  len(sp), src.ctypes.data_as(P(gl_flare_source)), 1, C.byref(prm),
                                                  st, C.byref(h)), "request_create")
        run = _Running()
        run.req, run.handle, run.stream, run.psf, run.prep = req, h, (lv, stream), None, None
        # the request renders into its own pool-allocated planes
        if self.lambda_chunks is not None:
            _native.check(self._lib.gl_request_set_lambda_split(h, min(int(self.lambda_chunks), req.n_spec)),
                          "request_set_lambda_split")
        _native.check(self._lib.gl_request_enqueue(h, None, None, None, self.cta_items(req), st), "request_enqueue")
        if req.starburst:
            req.starburst = self._add_starburst(req, rl, h, stream)
        run.host = None
        run.outs = None
        if self.host_output:
            run.host = self._pinned_buf((3, req.height, req.width))
            _native.check(self._lib.gl_request_copy_out(h, run.host.data_ptr(), st), "request_copy_out")
        else:
            # device result: copied out of the pool block into a torch tensor on the same stream
            with torch.cuda.stream(stream):
                run.outs = torch.empty((3, req.height, req.width), dtype=torch.float32, device=self.device)
                _native.check(self._lib.gl_request_copy_out(h, run.outs.data_ptr(), st), "request_copy_out")
        run.event = torch.cuda.Event()
        run.event.record(stream)
        if heavy:
            self._heavy[id(run)] = lv
        return run

    def psf_config(self, req: FlareRequest, rl: ResidentLens):
        """The PSFConfig of a PSF request (and its sources), as render_psf takes them."""
        from .config import PSFConfig
        cfg = PSFConfig(grid_nx=req.psf_grid, grid_ny=req.psf_grid, tile_w=req.psf_tile, tile_h=req.psf_tile,
                        tile_extent_mm=req.psf_extent_mm, spectral_samples=req.n_spec, ray_grid=req.ray_grid)
        cal = rl.calibration
        f = np.float32
        ax, ay = f(cal.max_half_angle_h) * f(req.psf_field_frac), f(cal.max_half_angle_v) * f(req.psf_field_frac)
        xs = np.linspace(-ax, ax, req.psf_grid, dtype=np.float32)
        ys = np.linspace(-ay, ay, req.psf_grid, dtype=np.float32)
        s2 = np.stack(np.meshgrid(xs, ys, indexing="xy"), -1).reshape(-1, 2)
        src = np.concatenate([s2, np.ones((len(s2), 3), np.float32)], 1)
        return cfg, src

    def _start_psf(self, req: FlareRequest, rl: ResidentLens, lv, stream) -> _Running:
        """A PSF request: the host pre-pass, then the atlas on the request's
        stream (gl_psf_render_async: scratch from the device pool, no wait)
        into a tensor allocated on that stream, copied out like a flare.

        The pre-pass (float32 host traces, up to ~70 ms on a 30-surface lens)
        is kept per resident lens and source grid.  One not yet kept runs on
        a worker thread, so the request loop goes on admitting and completing
        other requests meanwhile; done() launches the atlas once it is
        ready."""
        from .psf_grid import psf_inputs
        cfg, src = self.psf_config(req, rl)
        run = _Running()
        run.req, run.handle, run.stream = req, None, (lv, stream)
        run.psf = run.host = run.outs = run.event = None
        run.prep = None
        s7 = np.zeros((len(src), 7), np.float32)
        s7[:, :src.shape[1]] = src
        if ("cells", s7.tobytes(), int(getattr(cfg, "center_mode", 0))) in rl.psf_cache:
            self._launch_psf(run, psf_inputs(src, rl.lens, cfg, rl.psf_cache))
        else:
            if self._prep_pool is None:
                import concurrent.futures
                self._prep_pool = concurrent.futures.ThreadPoolExecutor(max_workers=1,
                                                                        thread_name_prefix="gl-psf-prepass")
            run.prep = self._prep_pool.submit(psf_inputs, src, rl.lens, cfg, rl.psf_cache)
        return run

    def _launch_psf(self, run: _Running, inp: dict):
        from .psf_grid import psf_launch
        torch = self.torch
        req = run.req
        stream = run.stream[1]
        with torch.cuda.stream(stream):
            run.psf = torch.zeros((3, inp["comp_h"], inp["comp_w"]), dtype=torch.float32, device=self.device)
            psf_launch(inp, run.psf, stream.cuda_stream, ordered=True)
            run.host, run.outs = None, None
            if self.host_output:
                run.host = self._pinned_buf(tuple(run.psf.shape))
                run.host.copy_(run.psf, non_blocking=True)
            else:
                run.outs = run.psf
        req.traced = int(inp["n"] * len(inp["grid"]) * len(inp["spec"]))
        run.event = torch.cuda.Event()
        run.event.record(stream)
        return run

    def _add_starburst(self, req: FlareRequest, rl: ResidentLens, h, stream) -> bool:
        """Accumulate the starburst layer into the request's planes once its
        ghost layer is written: on the plan's stream, joined back by events.
        A source whose image point lies more than a frame width outside the
        frame (a field beyond the lens's coverage) gets no starburst layer:
        False."""
        torch = self.torch
        cx, cy = rl.image_point(req.field_deg, req.width, req.height)
        if abs(cx - 0.5 * req.width) > 1.5 * req.width:
            return False
        if self.starburst_engine == "sprite":
            sprite, M, g = self.sprites.get(req.lens_id, rl, req.width, req.height, req.n_spec)
            d = C.c_void_p()
            _native.check(self._lib.gl_request_planes(h, C.byref(d)), "request_planes")
            base, npx = int(d.value), req.width * req.height
            _native.check(self._lib.gl_sprite_splat_source(
                C.c_void_p(sprite.data_ptr()), M, float(cx), float(cy), 1.0, 1.0, 1.0, g["sx_ds"], g["sy_ds"],
                g["px_mm_x"], g["px_mm_y"], g["rx"], g["ry"], g["gain"], C.c_void_p(base),
                C.c_void_p(base + 4 * npx), C.c_void_p(base + 8 * npx), req.width, req.height,
                C.c_void_p(stream.cuda_stream)), "starburst")
            return True
        if self.starburst is None:
            self.starburst = StarburstPlans(self.device, self.starburst_ctas)
        spec, _ = _spectral(req.n_spec, rl.config)
        plan, pst = self.starburst.get(req.width, req.height, spec)
        d = C.c_void_p()
        _native.check(self._lib.gl_request_planes(h, C.byref(d)), "request_planes")
        base, npx = int(d.value), req.width * req.height
        ghost_done = torch.cuda.Event()
        ghost_done.record(stream)
        pst.wait_event(ghost_done)
        plan.set_center(cx, cy, stream=pst.cuda_stream)
        k = StarburstPlans.chunks(req.width, req.height, req.n_spec)
        if k == 1:
            plan.execute_raw(rl.starburst_pupil().data_ptr(), base, base + 4 * npx, base + 8 * npx,
                             stream=pst.cuda_stream, accumulate=True)
        else:
            per = -(-req.n_spec // k)
            for l0 in range(0, req.n_spec, per):
                plan.set_lambda_range(l0, min(req.n_spec, l0 + per))
                plan.execute_raw(rl.starburst_pupil().data_ptr(), base, base + 4 * npx, base + 8 * npx,
                                 stream=pst.cuda_stream, accumulate=True)
            plan.set_lambda_range(0, -1)
        sb_done = torch.cuda.Event()
        sb_done.record(pst)
        stream.wait_event(sb_done)
        return True

    def prewarm_starburst(self, shapes, n_specs, config):
        """Bake the sprites of every (lens, size, wavelength count), or create
        the matrix-DFT plans of every (size, wavelength count)."""
        if self.starburst_engine == "sprite":
            for lid, rl in self.lenses.items():
                for (w, h) in shapes:
                    for ns in n_specs:
                        self.sprites.get(lid, rl, w, h, ns)
            return
        if self.starburst is None:
            self.starburst = StarburstPlans(self.device, self.starburst_ctas)
        for (w, h) in shapes:
            for ns in n_specs:
                self.starburst.get(w, h, _spectral(ns, config)[0])

    def prewarm(self, shapes, count: int):
        """Pinned host buffers for `count` results of each (width, height)."""
        for (w, h) in shapes:
            bufs = [self._pinned_buf((3, h, w)) for _ in range(count)]
            for b in bufs:
                self.recycle(b)

    def done(self, run: _Running) -> bool:
        if run.prep is not None:                  # a PSF pre-pass on the worker thread
            if not run.prep.done():
                return False
            inp = run.prep.result()
            run.prep = None
            self._launch_psf(run, inp)
            return False
        return run.event.query()

    def finish(self, run: _Running):
        """Release the request's device memory (stream-ordered) and stream;
        returns the host planes (or the device tensor)."""
        lv, stream = run.stream
        self._heavy.pop(id(run), None)
        if run.handle is not None:
            v = C.c_longlong()
            if self._lib.gl_request_traced(run.handle, C.byref(v), None) == 0:
                run.req.traced = int(v.value)          # the stream is idle: no wait
            self._lib.gl_request_destroy(run.handle, stream.cuda_stream)
            run.handle = None
        run.psf = None
        self.free_streams[lv].append(stream)
        out = run.host if run.host is not None else run.outs
        run.outs = None
        return out


class FlareServer:
    """Continuous-batching request loop over one GPU.

    Streams beyond the device's hardware work queues share queues and
    serialise; run the process with CUDA_DEVICE_MAX_CONNECTIONS=32 (set before
    CUDA starts) and at most 32 requests in flight."""

    def __init__(self, lenses: Dict[int, ResidentLens], budget_bytes: int = 120 * 10 ** 9,
                 max_inflight: int = 16, items_per_warp: int = 8, host_output: bool = True,
                 executor=None, clock: Callable[[], float] = time.perf_counter, policy: str = "sjf",
                 lambda_chunks: Optional[int] = None):
        self.lenses = lenses
        self.sched = Scheduler(budget_bytes, max_inflight)
        self.exec = executor if executor is not None else CudaExecutor(lenses, max_inflight, items_per_warp,
                                                                       host_output, policy=policy,
                                                                       lambda_chunks=lambda_chunks)
        self.clock = clock
        self.t0 = clock()
        self.running: list = []             # (request, executor handle)
        self.completed: List[FlareRequest] = []
        self.rejected: List[FlareRequest] = []
        self.on_result: Optional[Callable] = None

    def now(self) -> float:
        return self.clock() - self.t0

    def submit(self, req: FlareRequest):
        """Queue a request; one that needs more than the whole HBM budget is
        marked rejected and kept out of the queue."""
        self.exec.estimate(req)
        try:
            self.sched.submit(req)
        except ValueError:
            req.rejected = True
            self.rejected.append(req)

    def step(self) -> int:
        """Complete finished requests, then admit and start new ones.
        Returns the number of state changes."""
        changes = 0
        still = []
        for req, run in self.running:
            if self.exec.done(run):
                out = self.exec.finish(run)
                req.finish = self.now()
                self.sched.release(req)
                self.completed.append(req)
                if self.on_result is not None:
                    self.on_result(req, out)      # the host buffer is reused after this returns
                if hasattr(self.exec, "recycle"):
                    self.exec.recycle(out if getattr(self.exec, "host_output", False) else None)
                changes += 1
            else:
                still.append((req, run))
        self.running = still
        for req in self.sched.admit():
            req.start = self.now()
            self.running.append((req, self.exec.start(req)))
            changes += 1
        return changes

    def idle(self) -> bool:
        return not self.running and not self.sched.pending

    def close(self):
        """Release the executor's host workers (the resident lenses stay)."""
        if hasattr(self.exec, "close"):
            self.exec.close()

    def run_trace(self, requests: List[FlareRequest], poll_s: float = 2e-4) -> List[FlareRequest]:
        """Replay requests at their arrival times (seconds from now) and
        serve them; returns them with start/finish times filled."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        self.t0 = self.clock()
        i = 0
        while i < len(reqs) or not self.idle():
            now = self.now()
            while i < len(reqs) and reqs[i].arrival <= now:
                self.submit(reqs[i])
                i += 1
            if self.step() == 0:
                nxt = reqs[i].arrival - self.now() if i < len(reqs) else poll_s
                time.sleep(max(0.0, min(poll_s, nxt)))
        return reqs


def latency_stats(reqs: List[FlareRequest], where: Optional[Callable] = None) -> dict:
    sel = [r for r in reqs if not r.rejected and (where is None or where(r))]
    if not sel:
        return {"n": 0}
    lat = np.array([r.latency for r in sel]) * 1e3
    return {"n": len(sel), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max())}


def poisson_requests(rate_hz: float, duration_s: float, lens_ids, seed: int = 5,
                     sizes=((512, 512), (1024, 1024), (2048, 2048), (4096, 4096)),
                     n_specs=(8, 16, 31), grid_min: int = 32, grid_max: int = 256,
                     field_max_deg: float = 20.0, starburst: bool = False,
                     psf_frac: float = 0.0) -> List[FlareRequest]:
    """The serving mix: Poisson arrivals; per request a lens from the pool,
    an output size, a wavelength count, a pupil grid side (multiple of 16 in
    [grid_min, grid_max]) and a source field angle, all seeded; starburst
    adds the starburst layer to every flare request; a fraction psf_frac of
    the requests are PSF atlases (4 x 4 or 8 x 8 tiles of 64^2, the 64^2
    pupil grid of the reference's default render config) instead."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    lens_ids = list(lens_ids)
    grids = list(range(grid_min, grid_max + 1, 16))
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= duration_s:
            break
        w, h = sizes[int(rng.integers(len(sizes)))]
        req = FlareRequest(lens_id=lens_ids[int(rng.integers(len(lens_ids)))], width=w, height=h,
                           n_spec=int(n_specs[int(rng.integers(len(n_specs)))]),
                           ray_grid=int(grids[int(rng.integers(len(grids)))]),
                           field_deg=float(rng.uniform(0.0, field_max_deg)), rid=len(out), arrival=t,
                           starburst=bool(starburst))
        if psf_frac > 0.0 and rng.random() < psf_frac:
            req.kind, req.starburst = "psf", False
            req.psf_grid = 4 if rng.random() < 0.5 else 8
            req.ray_grid = 64
            req.width = req.height = req.psf_grid * req.psf_tile
        out.append(req)
    return out


def serving_lens(seed: int, n_surfaces: int, field_deg: float = 20.0):
    """(OpticalSystem, sensor_half_w, sensor_half_h) of one seeded serving
    lens: the random prescription with n_surfaces entries, and the sensor of
    its calibration (calibrate_lens: the covered field's landing per axis)."""
    from .calibration import calibrate_lens
    from .optics import OpticalSystem
    from .prescriptions import random_lens
    surfs = random_lens(seed, n_surfaces, field_deg=field_deg)
    lens = OpticalSystem.from_records(surfs, name="serve_%d_%d" % (seed, n_surfaces))
    cal = calibrate_lens(lens)
    lens.serving_focal_x = float(cal.focal_length_x)
    lens.serving_calibration = cal
    return lens, cal.sensor_half_w, cal.sensor_half_h


def serving_lens_pool(n_lenses: int, config, seed: int = 100, n_min: int = 8, n_max: int = 30):
    """Register n_lenses seeded lenses with n_min..n_max surfaces as resident
    lenses; returns {lens_id: ResidentLens}."""
    rng = np.random.default_rng(seed)
    pool = {}
    for i in range(n_lenses):
        n = int(rng.integers(n_min, n_max + 1))
        lens, hw, hh = serving_lens(seed + i, n)
        pool[i] = ResidentLens(lens, hw, hh, config, calibration=lens.serving_calibration)
        pool[i].focal_x = lens.serving_focal_x
    return pool

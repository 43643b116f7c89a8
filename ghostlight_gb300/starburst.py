"""Matrix-DFT starburst on the tensor cores (row d of the flare path).

Two forms of the per-wavelength triple product on the same GEMMs:

* the reference's own engine (ghostlight/src/mdft_render.cu:199-340), the
  exact pixel-box integral of the intensity through the compact pupil
  autocorrelation C: I_l = Re(P_y C P_x^T), P[k][m] = sinc(s_l m)
  exp(-2 pi i s_l m (k - c)) (``mdft_box_starburst_layer``, the MDFT engine
  of render_source_flare);
* the field form E_l = W_y A W_x^T, I_l = |E_l|^2, out_c = sum_l w_c(l) I_l,
  W[k][j] = exp(-2 pi i s_l (j - (n-1)/2)(k - c)): the pupil sampled at the
  pixel centres, without the box integral (``starburst_layer``,
  ``mdft_starburst_eform``).

Forms: ``"split_bf16"`` (three-term split-BF16 tcgen05 products, FP32
accumulation in tensor memory), ``"tf32"`` (tcgen05 kind::tf32) and ``"fp32"``
(FP32 on the CUDA cores).  The DFT matrices are built once per plan and stay
resident in HBM.
"""
from __future__ import annotations

import ctypes as C
import math
import threading

import numpy as np

from . import _native

FORMS = {"split_bf16": 0, "tf32": 1, "fp32": 2}

# algorithmic FLOPs of one wavelength (complex W x real A, then complex x
# complex), K = output side, n = pupil side
def flops_per_lambda(n: int, K: int) -> float:
    return 2.0 * (2.0 * n * n * K + 4.0 * n * K * K)


class MdftPlan:
    """K: output side, or (Kx, Ky) for a Kx-wide, Ky-high output."""

    def __init__(self, n: int, K, scale_x, scale_y, weights_rgb, form="split_bf16",
                 center_x=None, center_y=None, stream=None, box=False, red_center=None):
        import torch
        self._lib = _native.load()
        Kx, Ky = (int(K), int(K)) if np.isscalar(K) else (int(K[0]), int(K[1]))
        self.n, self.Kx, self.Ky = int(n), Kx, Ky
        self.K = Kx
        sx = np.ascontiguousarray(scale_x, np.float64)
        sy = np.ascontiguousarray(scale_y, np.float64)
        w = np.ascontiguousarray(weights_rgb, np.float32).reshape(-1, 3)
        if not (len(sx) == len(sy) == len(w)):
            raise ValueError("mdft: scale_x, scale_y and weights need one entry per wavelength")
        self.n_lambda = len(sx)
        self.form = form
        cx = self.Kx / 2.0 if center_x is None else float(center_x)
        cy = self.Ky / 2.0 if center_y is None else float(center_y)
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        D = C.c_double * self.n_lambda
        h = C.c_void_p()
        self.box = bool(box)
        rc = 0.5 * (self.n - 1) if red_center is None else float(red_center)
        _native.check(self._lib.gl_mdft_plan_create3(
            self.n, self.Kx, self.Ky, self.n_lambda, D(*sx), D(*sy), cx, cy,
            (C.c_float * w.size)(*w.reshape(-1)), FORMS[form], int(self.box), rc, st, C.byref(h)), "mdft")
        self._h = h

    def set_center(self, center_x: float, center_y: float, stream=None):
        """Enqueue the DFT-matrix rebuild for a new pattern centre."""
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _native.check(self._lib.gl_mdft_plan_set_center(self._h, float(center_x), float(center_y), st), "mdft")
        return _native.last_launch_count()

    def execute(self, pupil, out_r, out_g, out_b, stream=None, accumulate=False):
        import torch
        if not (pupil.is_cuda and pupil.dtype == torch.float32 and pupil.shape == (self.n, self.n)):
            raise ValueError("mdft: pupil must be a float32 CUDA (n, n) tensor")
        for t in (out_r, out_g, out_b):
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and t.numel() == self.Kx * self.Ky):
                raise ValueError("mdft: outputs must be contiguous float32 CUDA (Ky, Kx) tensors")
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _native.check(self._lib.gl_mdft_plan_execute2(self._h, pupil.contiguous().data_ptr(), out_r.data_ptr(),
                                                      out_g.data_ptr(), out_b.data_ptr(), int(bool(accumulate)), st),
                      "mdft")
        return _native.last_launch_count()

    def execute_window(self, operand, out_r, out_g, out_b, x0, y0, win_w, win_h, tint=None, stream=None,
                       accumulate=True):
        """execute into (H, W) planes: plan pixel (l, k) -> plane pixel
        (y0 + l, x0 + k) for l < win_h, k < win_w; ``tint`` (r, g, b) scales
        the weights of this launch."""
        import torch
        if not (operand.is_cuda and operand.dtype == torch.float32 and operand.shape == (self.n, self.n)):
            raise ValueError("mdft: operand must be a float32 CUDA (n, n) tensor")
        H, W = out_r.shape
        for t in (out_r, out_g, out_b):
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and tuple(t.shape) == (H, W)):
                raise ValueError("mdft: outputs must be three contiguous float32 CUDA (H, W) tensors")
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        tr = (C.c_float * 3)(*(tint if tint is not None else (1.0, 1.0, 1.0)))
        _native.check(self._lib.gl_mdft_plan_execute3(self._h, operand.contiguous().data_ptr(), out_r.data_ptr(),
                                                      out_g.data_ptr(), out_b.data_ptr(), int(bool(accumulate)),
                                                      int(W), int(H), int(x0), int(y0), int(win_w), int(win_h), tr,
                                                      st), "mdft")
        return _native.last_launch_count()

    def set_lambda_range(self, begin: int = 0, end: int = -1):
        """Restrict the next executes to wavelengths [begin, end) ((0, -1): all)."""
        _native.check(self._lib.gl_mdft_plan_set_lambda_range(self._h, int(begin), int(end)), "mdft")

    def set_launch(self, ctas=0, tile: int = 128):
        """GEMM grid of the tensor-core forms (0 = one CTA per SM) and the
        output tile width of their second GEMM (128 or 64 complex columns);
        ``ctas`` may also be a (ctas, tile) pair, as the autotuner passes it."""
        if isinstance(ctas, (tuple, list)):
            ctas, tile = ctas
        _native.check(self._lib.gl_mdft_plan_set_launch(self._h, int(ctas)), "mdft")
        _native.check(self._lib.gl_mdft_plan_set_tile(self._h, int(tile)), "mdft")
        self.launch = (int(ctas), int(tile))

    def execute_raw(self, pupil_ptr: int, r_ptr: int, g_ptr: int, b_ptr: int, stream=None, accumulate=False):
        """execute on raw device addresses (planes owned by another component,
        e.g. a serving request); the caller guarantees the sizes."""
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _native.check(self._lib.gl_mdft_plan_execute2(self._h, int(pupil_ptr), int(r_ptr), int(g_ptr), int(b_ptr),
                                                      int(bool(accumulate)), st), "mdft")
        return _native.last_launch_count()

    def status(self) -> int:
        v = C.c_int()
        _native.check(self._lib.gl_mdft_plan_status(self._h, C.byref(v)), "mdft")
        return int(v.value)

    def device_bytes(self) -> int:
        """HBM the plan holds: the two DFT matrices, the operand mask and the
        intermediate T' in the form's element type (split-BF16: three bf16
        terms per element along K)."""
        kp = 3 * self.n if self.form == "split_bf16" else self.n
        elem = 2 if self.form == "split_bf16" else 4
        nl = self.n_lambda
        return (nl * 2 * (self.Kx + self.Ky) * kp * elem + self.n * kp * elem +
                nl * (self.Kx // 128) * 3 * 128 * kp * elem + 32 * nl + 4)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gl_mdft_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build_pupil(lens, N: int, pupil_fill: float = 0.45, blades_override: int = 0, rotation_deg: float = 0.0,
                stream=None):
    """Stop-silhouette pupil amplitude (N, N) float32 CUDA tensor, 4 x 4
    supersampled on the device (build_pupil_kernel, starburst_render.cu:155)."""
    import torch
    lib = _native.load()
    arr = lens.to_array()
    out = torch.empty((N, N), dtype=torch.float32, device="cuda")
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    _native.check(lib.gl_build_pupil(arr, len(arr), int(N), float(pupil_fill), int(blades_override),
                                     float(rotation_deg), out.data_ptr(), st), "build_pupil")
    return out


def mdft_starburst_eform(pupil, K, scale_x, scale_y, weights_rgb, form="split_bf16"):
    """One-shot: returns (3, K, K) float32 CUDA tensor."""
    import torch
    plan = MdftPlan(pupil.shape[0], K, scale_x, scale_y, weights_rgb, form)
    out = torch.empty((3, plan.Ky, plan.Kx), dtype=torch.float32, device=pupil.device)
    plan.execute(pupil, out[0], out[1], out[2])
    torch.cuda.synchronize()
    code = plan.status()
    plan.close()
    if code:
        raise _native.GhostlightError("mdft: device pipeline wait timed out (code %d)" % code)
    return out


def _round128(x: int) -> int:
    return max(128, (int(x) + 127) // 128 * 128)


def starburst_layer(lens, calibration, config, sources_px, width: int, height: int, sensor_half_w: float,
                    sensor_half_h: float, form: str = "split_bf16"):
    """The starburst layer of a flare render: the Fraunhofer pattern |E|^2 of
    the stop pupil (built on the device) around each source's image point,
    summed over the config's wavelengths.

    Scale per axis (the reference sizes its pattern by first-order optics,
    render_config.h:128-150): pupil sample pitch 2 EP / (fill n), output
    pixel pitch 2 half / size, focal length f -> s = pitch_pupil pitch_px /
    (lambda f) cycles per sample per pixel, divided by scale_trim.  Brightness:
    starburst_gain x the source flux per wavelength (cmf-weighted) over one
    period of the pattern.  sources_px: (N, 5) [px, py, r, g, b].
    Returns {"starburst_r", "starburst_g", "starburst_b"} (H, W) tensors.
    """
    import torch
    from .flare import spectral_table
    dc = config.diffraction
    n = 256 if int(dc.starburst_grid) <= 1024 else 512
    fill = float(dc.pupil_fill) if 0.02 < float(dc.pupil_fill) < 0.9 else 0.30
    ns = int(dc.spectral_samples) if int(dc.spectral_samples) > 0 else int(config.spectral_samples)
    ns = max(3, ns)
    spec, _ = spectral_table(ns, int(config.output_cs), config.custom_xyz_to_output)
    lam_mm = spec[:, 0].astype(np.float64) * 1e-6
    trim = float(dc.scale_trim) if float(dc.scale_trim) > 0 else 1.0
    fx = float(calibration.focal_length_x) or 1.0
    fy = float(calibration.focal_length_y) or 1.0
    dxp = 2.0 * float(calibration.entrance_pupil_semi_x) / (fill * n)
    dyp = 2.0 * float(calibration.entrance_pupil_semi_y) / (fill * n)
    sx = dxp * (2.0 * sensor_half_w / width) / (lam_mm * fx) / trim
    sy = dyp * (2.0 * sensor_half_h / height) / (lam_mm * fy) / trim
    pupil = build_pupil(lens, n, fill, int(config.aperture_blades), float(config.aperture_rotation))
    amp2 = float((pupil.double() ** 2).sum())
    Kx, Ky = _round128(width), _round128(height)
    src = np.asarray(sources_px, np.float64).reshape(-1, 5)
    out = torch.zeros((3, Ky, Kx), dtype=torch.float32, device="cuda")
    if amp2 <= 0.0 or len(src) == 0:
        return {k: torch.zeros((height, width), dtype=torch.float32, device="cuda")
                for k in ("starburst_r", "starburst_g", "starburst_b")}
    plan = None
    for (px, py, r, g, b) in src:
        # one period of |E|^2 sums to (1 / (sx sy)) sum |A|^2: normalise it to gain x flux per wavelength
        w = spec[:, 1:4].astype(np.float64) * np.array([r, g, b])[None, :] * (sx * sy)[:, None] / amp2
        w *= float(dc.starburst_gain)
        if plan is None:
            plan = MdftPlan(n, (Kx, Ky), sx, sy, w.astype(np.float32), form, center_x=px, center_y=py)
        else:
            plan.close()
            plan = MdftPlan(n, (Kx, Ky), sx, sy, w.astype(np.float32), form, center_x=px, center_y=py)
        plan.execute(pupil, out[0], out[1], out[2], accumulate=True)
    torch.cuda.synchronize()
    code = plan.status()
    plan.close()
    if code:
        raise _native.GhostlightError("starburst: device pipeline wait timed out (code %d)" % code)
    return {"starburst_r": out[0, :height, :width].contiguous(), "starburst_g": out[1, :height, :width].contiguous(),
            "starburst_b": out[2, :height, :width].contiguous()}


# ---------------------------------------------------------------------------
# SPRITE engine (render_starburst's default path, starburst_render.cu:594-1073)
# ---------------------------------------------------------------------------
LAMBDA_REF_NM = 550.0       # wavelength of the one FFT
SPRITE_OVERSAMPLE = 3       # sprite texels kept per output pixel after the box sum
APERTURE_REF_FNUMBER = 2.8


class SpritePlan:
    """Resident sprite pipeline for one grid and spectral table: FFT of the
    pupil, PSF, wavelength bake + box sum, splat (gl_sprite_plan_*)."""

    def __init__(self, N: int, spec, lambda_ref: float = LAMBDA_REF_NM):
        from ._abi import gl_spectral_sample
        lib = _native.load()
        spec = np.ascontiguousarray(spec, np.float32).reshape(-1, 4)
        arr = (gl_spectral_sample * len(spec))()
        C.memmove(arr, spec.ctypes.data, spec.nbytes)
        h = C.c_void_p()
        _native.check(lib.gl_sprite_plan_create(int(N), arr, len(spec), float(lambda_ref), C.byref(h)),
                      "sprite_plan_create")
        self._h, self.N, self.M = h, int(N), 0

    def bake(self, pupil, ds: int, stream=None) -> None:
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        pupil = pupil.to(torch.float32).contiguous()
        if tuple(pupil.shape) != (self.N, self.N):
            raise ValueError("sprite: pupil must be (N, N)")
        self._pupil = pupil      # kept alive until the stream has read it
        _native.check(_native.load().gl_sprite_plan_bake(self._h, C.c_void_p(pupil.data_ptr()), int(ds),
                                                         C.c_void_p(st)), "sprite_bake")
        self.M = self.N // int(ds)

    def splat(self, sources, sx_ds, sy_ds, px_mm_x, px_mm_y, rx, ry, gain, out_r, out_g, out_b, stream=None):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        src = np.ascontiguousarray(sources, np.float32).reshape(-1, 5)
        H, W = out_r.shape
        _native.check(_native.load().gl_sprite_plan_splat(
            self._h, src.ctypes.data_as(C.POINTER(C.c_float)), len(src), float(sx_ds), float(sy_ds),
            float(px_mm_x), float(px_mm_y), int(rx), int(ry), float(gain), C.c_void_p(out_r.data_ptr()),
            C.c_void_p(out_g.data_ptr()), C.c_void_p(out_b.data_ptr()), int(W), int(H), C.c_void_p(st)),
            "sprite_splat")

    def autocorr(self, pupil, mc: int, out, stream=None) -> None:
        """The compact autocorrelation of the pupil at lags |l| <= mc into
        ``out`` (rows x cols float32 CUDA, rows, cols >= 2 mc + 1; zeroed
        first), scaled to one texel area per pattern period."""
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        pupil = pupil.to(torch.float32).contiguous()
        if tuple(pupil.shape) != (self.N, self.N):
            raise ValueError("autocorr: pupil must be (N, N)")
        if not (out.is_cuda and out.dtype == torch.float32 and out.is_contiguous() and out.dim() == 2):
            raise ValueError("autocorr: output must be a contiguous float32 CUDA matrix")
        self._pupil = pupil
        _native.check(_native.load().gl_sprite_plan_autocorr(self._h, C.c_void_p(pupil.data_ptr()), int(mc),
                                                             C.c_void_p(out.data_ptr()), int(out.shape[1]),
                                                             int(out.shape[0]), C.c_void_p(st)), "autocorr")
        self.M = 0

    def read(self):
        """(PSF (N, N) before normalisation, sprite (M, M, 3), PSF energy)."""
        import torch
        psf = torch.empty((self.N, self.N), dtype=torch.float32, device="cuda")
        spr = torch.empty((self.M, self.M, 3), dtype=torch.float32, device="cuda")
        e, m = C.c_double(), C.c_int()
        st = torch.cuda.current_stream().cuda_stream
        _native.check(_native.load().gl_sprite_plan_read(self._h, C.c_void_p(psf.data_ptr()),
                                                         C.c_void_p(spr.data_ptr()), C.byref(e), C.byref(m),
                                                         C.c_void_p(st)), "sprite_read")
        return psf, spr, float(e.value)

    def close(self):
        if self._h:
            _native.load().gl_sprite_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _po2_floor(x: float, hi: int) -> int:
    p = 1
    while p * 2 <= x and p * 2 <= hi:
        p *= 2
    return max(p, 1)


def starburst_spectrum(config):
    """The starburst's spectral table (render_starburst :712-736): the
    output-space CMF with the sample spacing premultiplied, each channel then
    normalised so a flat spectrum sums to one (white in, white out)."""
    from .flare import spectral_table
    dc = config.diffraction
    ns = int(dc.spectral_samples) if int(dc.spectral_samples) > 0 else int(config.spectral_samples)
    ns = max(3, ns)
    spec, _ = spectral_table(ns, int(config.output_cs), config.custom_xyz_to_output)
    f = np.float32
    d_lambda = f(f(700.0 - 400.0) / f(ns))
    spec = spec.copy()
    spec[:, 1:4] = (spec[:, 1:4] * d_lambda).astype(np.float32)
    sums = spec[:, 1:4].astype(np.float64).sum(0)
    for c in range(3):
        if sums[c] > 0.0:
            spec[:, 1 + c] = (spec[:, 1 + c] / np.float32(sums[c])).astype(np.float32)
    return spec


def sprite_geometry(calibration, config, sources_px, width: int, height: int, sensor_half_w: float,
                    sensor_half_h: float, fmt_w=None, fmt_h=None, front_R: float = 0.0):
    """The sprite path's scalars (render_starburst :620-711, :1003-1070) in
    the reference's float32: grid N (grown to cover the frame when the pattern
    is prominent or the sensor oversized), engine ('sprite' / 'mdft'), fine
    texel pitch, box-sum factor ds, M, footprint rx / ry and the gain."""
    f = np.float32
    dc = config.diffraction
    fmt_w = int(fmt_w or width)
    fmt_h = int(fmt_h or height)
    efl_x, efl_y = f(calibration.focal_length_x), f(calibration.focal_length_y)
    ep_x, ep_y = f(calibration.entrance_pupil_semi_x), f(calibration.entrance_pupil_semi_y)
    if efl_x <= 0 and calibration.max_half_angle_h > 0:
        efl_x = f(f(sensor_half_w) / f(np.tan(f(calibration.max_half_angle_h))))
    if efl_y <= 0 and calibration.max_half_angle_v > 0:
        efl_y = f(f(sensor_half_h) / f(np.tan(f(calibration.max_half_angle_v))))
    if ep_x <= 0:
        ep_x = f(front_R)
    if ep_y <= 0:
        ep_y = f(front_R)
    if efl_x <= 0 or efl_y <= 0 or ep_x <= 0 or ep_y <= 0:
        raise ValueError("render_starburst: degenerate first-order optics (no focal length / pupil)")
    fnum_x = f(efl_x / (f(2.0) * ep_x))
    fnum_y = f(efl_y / (f(2.0) * ep_y))
    N = int(dc.starburst_grid)
    if N < 256 or (N & (N - 1)) != 0:
        raise ValueError("starburst_grid must be a power of two >= 256")
    fill = f(dc.pupil_fill) if f(0.02) < f(dc.pupil_fill) < f(0.9) else f(0.30)
    lam_mm = f(f(LAMBDA_REF_NM) * f(1e-6))
    dx_fine_x = f(f(lam_mm * fnum_x) * fill)
    dx_fine_y = f(f(lam_mm * fnum_y) * fill)
    engine = "mdft" if int(dc.starburst_engine) == 1 else "sprite"
    trim0 = f(dc.scale_trim) if f(dc.scale_trim) > 0 else f(1.0)
    dx0_x, dx0_y = f(trim0 * dx_fine_x), f(trim0 * dx_fine_y)
    frame_w, frame_h = f(f(2.0) * f(sensor_half_w)), f(f(2.0) * f(sensor_half_h))
    frac = max(f(f(N) * dx0_x / frame_w) if frame_w > 0 else f(0.0),
               f(f(N) * dx0_y / frame_h) if frame_h > 0 else f(0.0))
    grid_cap = int(dc.starburst_grid_cap) if int(dc.starburst_grid_cap) >= 256 else 8192
    grid_cap = min(grid_cap, 16384)
    p = 256
    while (p << 1) <= grid_cap:
        p <<= 1
    grid_cap = max(p, N)
    circle_w = f(calibration.image_circle_semi_w) if calibration.image_circle_semi_w > 0 else f(calibration.sensor_half_w)
    circle_h = f(calibration.image_circle_semi_h) if calibration.image_circle_semi_h > 0 else f(calibration.sensor_half_h)
    oversized = ((circle_w > 0 and f(sensor_half_w) > f(1.5) * circle_w) or
                 (circle_h > 0 and f(sensor_half_h) > f(1.5) * circle_h))
    prominent = frac >= f(0.20)
    if prominent:
        engine = "sprite"
    src = np.asarray(sources_px, np.float32).reshape(-1, 5)
    if frac < 1.0 and (prominent or oversized) and len(src) and width > 0 and height > 0 and grid_cap > N:
        reach_x = reach_y = f(0.0)
        for (px, py, _r, _g, _b) in src:
            reach_x = max(reach_x, max(f(px), f(f(width) - f(px))))
            reach_y = max(reach_y, max(f(py), f(f(height) - f(py))))
        px_buf_x, px_buf_y = f(frame_w / f(width)), f(frame_h / f(height))
        covN = max(2.0 * float(reach_x) * float(px_buf_x) / float(dx0_x),
                   2.0 * float(reach_y) * float(px_buf_y) / float(dx0_y))
        want = int(np.ceil(covN)) if covN > N else N
        want = min(want, grid_cap)
        Ne = 256
        while Ne < want:
            Ne <<= 1
        if Ne > N:
            N, engine = Ne, "sprite"
    px_mm_x = f(f(f(2.0) * f(sensor_half_w)) / f(fmt_w))
    px_mm_y = f(f(f(2.0) * f(sensor_half_h)) / f(fmt_h))
    trim = trim0
    sx, sy = f(trim * dx_fine_x), f(trim * dx_fine_y)
    ds_target = min(float(px_mm_x) / float(f(sx * f(SPRITE_OVERSAMPLE))),
                    float(px_mm_y) / float(f(sy * f(SPRITE_OVERSAMPLE))))
    ds = _po2_floor(ds_target, N // 8)
    M = N // ds
    sx_ds, sy_ds = f(sx * f(ds)), f(sy * f(ds))
    aperture_scale = f(f(f(APERTURE_REF_FNUMBER) * f(APERTURE_REF_FNUMBER)) * f(calibration.pupil_area_frac)
                       / max(f(fnum_x * fnum_y), f(1e-6)))
    gain = f(f(f(dc.starburst_gain) * f(1.0)) * aperture_scale)     # pupil throughput T = 1 (plain stop)
    rx = int(np.ceil(0.5 * M * float(sx_ds) / float(px_mm_x))) + 1
    ry = int(np.ceil(0.5 * M * float(sy_ds) / float(px_mm_y))) + 1
    rx, ry = min(rx, width), min(ry, height)
    return dict(N=N, engine=engine, fill=float(fill), ep_x=float(ep_x), ep_y=float(ep_y), sx=float(sx), sy=float(sy),
                ds=ds, M=M, sx_ds=float(sx_ds),
                sy_ds=float(sy_ds), px_mm_x=float(px_mm_x), px_mm_y=float(px_mm_y), rx=rx, ry=ry,
                gain=float(gain), fnum_x=float(fnum_x), fnum_y=float(fnum_y), efl_x=float(efl_x),
                efl_y=float(efl_y))


def build_pupil2(lens, N: int, pupil_fill: float, blades_override: int = 0, rotation_deg: float = 0.0,
                 aspect_one: bool = True, envelope=None, stream=None):
    """The starburst's effective pupil (build_pupil_kernel,
    starburst_render.cu:155-191): the stop rasterised round (the aspect goes
    into the per-axis pitch) and, when given, weighted by the cat's-eye
    envelope (ME x ME host or device array over pupil [-1, 1]^2)."""
    import torch
    lib = _native.load()
    arr = lens.to_array()
    out = torch.empty((N, N), dtype=torch.float32, device="cuda")
    st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    env, me = None, 0
    if envelope is not None:
        env = torch.as_tensor(np.asarray(envelope, np.float32) if not hasattr(envelope, "is_cuda") else envelope,
                              dtype=torch.float32).cuda().contiguous()
        me = env.shape[0]
    _native.check(lib.gl_build_pupil2(arr, len(arr), int(N), float(pupil_fill), int(blades_override),
                                      float(rotation_deg), int(bool(aspect_one)),
                                      C.c_void_p(env.data_ptr()) if env is not None else None, int(me),
                                      C.c_void_p(out.data_ptr()), C.c_void_p(st)), "build_pupil")
    if env is not None:
        torch.cuda.current_stream().synchronize()
    return out


def effective_pupil_info(lens, config, g, field) -> dict:
    """The sprite's pupil, its throughput T and the survivor-centre launch
    offset (render_starburst :740-922): on axis, or with use_survivor_mask
    off, the plain stop, T = 1 and no offset; off axis, the stop weighted by
    the cat's-eye envelope centred on the surviving crescent, T = its energy
    over the plain stop's.  {"pupil", "T", "chief": (cx, cy), "survivors"};
    pupil is None only where no launch survives at this field."""
    dc = config.diffraction
    f = np.float32
    bo, rot = int(config.aperture_blades), float(config.aperture_rotation)
    ax, ay = (f(field[0]), f(field[1])) if field is not None else (f(0.0), f(0.0))
    off_axis = abs(float(ax)) > 1e-5 or abs(float(ay)) > 1e-5
    if not (bool(dc.use_survivor_mask) and off_axis):
        return {"pupil": build_pupil2(lens, g["N"], g["fill"], bo, rot), "T": 1.0, "chief": (0.0, 0.0),
                "survivors": True}
    cx, cy, any_surv = survivor_center(lens, float(ax), float(ay))
    if not any_surv:
        return {"pupil": None, "T": 0.0, "chief": (0.0, 0.0), "survivors": False}
    me = min(max(int(dc.survivor_grid), 16), 1024)
    env = survivor_envelope(lens, g["ep_x"], g["ep_y"], cx, cy, float(ax), float(ay), me)
    plain = build_pupil2(lens, g["N"], g["fill"], bo, rot)
    pupil = build_pupil2(lens, g["N"], g["fill"], bo, rot, envelope=env)
    s_ref = float((plain.double() ** 2).sum())
    s_eff = float((pupil.double() ** 2).sum())
    T = min(max(s_eff / s_ref, 0.0), 1.0) if s_ref > 0 else 1.0
    return {"pupil": pupil, "T": T, "chief": (cx, cy), "survivors": True}


def effective_pupil(lens, config, g, field):
    """(pupil, T) of effective_pupil_info, or (None, T) where the starburst is
    cut off: nothing survives, or T < 1e-3 (the field is past the lens's
    imaged circle)."""
    info = effective_pupil_info(lens, config, g, field)
    if info["pupil"] is None or info["T"] < 1e-3:
        return None, info["T"]
    return info["pupil"], info["T"]


def sprite_starburst_layer(lens, calibration, config, sources_px, width: int, height: int, sensor_half_w: float,
                           sensor_half_h: float, fmt_w=None, fmt_h=None, geometry=None, field=None):
    """The starburst layer by the reference's default SPRITE engine: one FFT
    of the device-built effective pupil at 550 nm, baked over the config's
    wavelengths, box-summed toward the output pitch and resampled
    area-weighted at every source (sources_px: (N, 5) px, py, r, g, b in
    buffer pixels; field: the mean source direction (radians), which sets the
    off-axis cat's-eye).  Returns {"starburst_r", "starburst_g",
    "starburst_b"}."""
    import torch
    g = geometry or sprite_geometry(calibration, config, sources_px, width, height, sensor_half_w, sensor_half_h,
                                    fmt_w, fmt_h, front_R=lens.surfaces[0].semi_aperture if lens.surfaces else 0.0)
    if g["N"] > 8192:
        raise ValueError("render_starburst: sprite grids above 8192 are not supported (starburst_grid_cap)")
    out = {k: torch.zeros((height, width), dtype=torch.float32, device="cuda")
           for k in ("starburst_r", "starburst_g", "starburst_b")}
    src = np.asarray(sources_px, np.float32).reshape(-1, 5)
    if len(src) == 0:
        return out
    spec = starburst_spectrum(config)
    with _PLAN_LOCK:
        return _sprite_layer_locked(lens, config, g, spec, src, field, out)


def _sprite_layer_locked(lens, config, g, spec, src, field, out):
    import torch
    plan, baked = _sprite_plan(g["N"], spec)
    ax, ay = (float(np.float32(field[0])), float(np.float32(field[1]))) if field is not None else (0.0, 0.0)
    off_axis = abs(ax) > 1e-5 or abs(ay) > 1e-5
    # the baked sprite depends on the stop, the grid, the box sum and (off
    # axis, with the cat's-eye) the field: an unchanged key reuses it
    key = (lens.state_key(), g["N"], g["fill"], g["ds"], int(config.aperture_blades),
           float(config.aperture_rotation), bool(config.diffraction.use_survivor_mask) and off_axis,
           (ax, ay, g["ep_x"], g["ep_y"], int(config.diffraction.survivor_grid))
           if bool(config.diffraction.use_survivor_mask) and off_axis else None)
    if baked.get("key") != key:
        pupil, T = effective_pupil(lens, config, g, field)
        if pupil is None:
            baked.clear()
            return out      # past the vignette edge: no starburst
        if not float(pupil.sum()) > 0.0:
            raise ValueError("render_starburst: degenerate pupil (zero energy)")
        plan.bake(pupil, g["ds"])
        baked.update(key=key, T=T, bakes=baked.get("bakes", 0) + 1)
    gain = float(np.float32(np.float32(g["gain"]) * np.float32(baked["T"])))
    plan.splat(src, g["sx_ds"], g["sy_ds"], g["px_mm_x"], g["px_mm_y"], g["rx"], g["ry"], gain,
               out["starburst_r"], out["starburst_g"], out["starburst_b"])
    torch.cuda.synchronize()
    return out


def mdft_box_starburst_layer(lens, calibration, config, sources_px, width: int, height: int, sensor_half_w: float,
                             sensor_half_h: float, geometry=None, field=None, form: str = "split_bf16"):
    """The starburst layer by the reference's matrix-DFT engine
    (render_starburst's MDFT fork, starburst_render.cu:926-967, and
    mdft_starburst, mdft_render.cu:199-340), on the tensor cores.

    The effective pupil, throughput, spectral table, texel pitch and gain are
    the sprite engine's (the reference shares them); C is the pupil's compact
    autocorrelation (four FFT passes on the device, gl_sprite_plan_autocorr);
    each source adds the exact pixel-box integral of the intensity over its
    window of half a pattern period, I_l = Re(P_y C P_x^T) per wavelength with
    cmf (lambda_ref / lambda)^2, times (px_x px_y) / (dx_x dx_y) x gain x the
    source colour.  ``form``: the GEMM form ("split_bf16", "tf32", "fp32").
    Returns {"starburst_r", "starburst_g", "starburst_b"} (H, W) tensors."""
    import torch
    f = np.float32
    g = geometry or sprite_geometry(calibration, config, sources_px, width, height, sensor_half_w, sensor_half_h,
                                    front_R=lens.surfaces[0].semi_aperture if lens.surfaces else 0.0)
    out = {k: torch.zeros((height, width), dtype=torch.float32, device="cuda")
           for k in ("starburst_r", "starburst_g", "starburst_b")}
    src = np.asarray(sources_px, np.float32).reshape(-1, 5)
    if len(src) == 0:
        return out
    pupil, T = effective_pupil(lens, config, g, field)
    if pupil is None:
        return out      # past the vignette edge: no starburst
    N = int(g["N"])
    mc = min(int(math.ceil(float(f(g["fill"])) * float(N))) + 4, N // 2 - 1)
    Mc = 2 * mc + 1
    n = _round128(Mc)
    spec = starburst_spectrum(config)
    with _PLAN_LOCK:
        ac = _autocorr_plan(N)
        Cm = torch.empty((n, n), dtype=torch.float32, device="cuda")
        ac.autocorr(pupil, mc, Cm)
    # the reference's float32 scalars (mdft_render.cu:226-283)
    dx_x, dx_y = f(g["sx"]), f(g["sy"])
    px_x, px_y = f(g["px_mm_x"]), f(g["px_mm_y"])
    Sx, Sy = f(f(N) * dx_x), f(f(N) * dx_y)
    half_x = max(1, int(math.floor(0.5 * float(Sx) / float(px_x))))
    half_y = max(1, int(math.floor(0.5 * float(Sy) / float(px_y))))
    gain = f(f(g["gain"]) * f(T))
    knorm_gain = f(f(f(px_x * px_y) / f(dx_x * dx_y)) * gain)
    lam = spec[:, 0].astype(np.float32)
    lam_scale = (lam / f(LAMBDA_REF_NM)).astype(np.float32)
    k2 = ((f(LAMBDA_REF_NM) / lam) * (f(LAMBDA_REF_NM) / lam)).astype(np.float32)
    s_x = float(px_x) / (Sx * lam_scale).astype(np.float32).astype(np.float64)
    s_y = float(px_y) / (Sy * lam_scale).astype(np.float32).astype(np.float64)
    w = (spec[:, 1:4] * k2[:, None]).astype(np.float32)
    Kx, Ky = _round128(min(width, 2 * half_x + 1)), _round128(min(height, 2 * half_y + 1))
    plan = MdftPlan(n, (Kx, Ky), s_x, s_y, w, form, center_x=0.0, center_y=0.0, box=True, red_center=float(mc))
    try:
        for (px, py, r, gg, b) in src:
            kx0, kx1 = max(0, int(math.floor(px)) - half_x), min(width, int(math.floor(px)) + half_x + 1)
            ky0, ky1 = max(0, int(math.floor(py)) - half_y), min(height, int(math.floor(py)) + half_y + 1)
            if kx1 <= kx0 or ky1 <= ky0:
                continue        # the source's window lies off the frame
            plan.set_center(float(px) - 0.5 - kx0, float(py) - 0.5 - ky0)
            tint = (float(knorm_gain * f(r)), float(knorm_gain * f(gg)), float(knorm_gain * f(b)))
            plan.execute_window(Cm, out["starburst_r"], out["starburst_g"], out["starburst_b"], kx0, ky0,
                                kx1 - kx0, ky1 - ky0, tint=tint)
        torch.cuda.synchronize()
        code = plan.status()
    finally:
        plan.close()
    if code:
        raise _native.GhostlightError("starburst: device pipeline wait timed out (code %d)" % code)
    return out


# resident sprite plans by (device, grid, spectrum), least recently used
# first; each keeps its last bake and the key it was baked for.  _PLAN_LOCK
# guards the caches and every bake / splat / autocorrelation on a cached plan
# (a plan evicted by one thread must not be in use by another).
_SPRITE_PLANS = {}
_SPRITE_PLAN_CAP = 4
_AUTOCORR_PLANS = {}
_PLAN_LOCK = threading.RLock()


def _autocorr_plan(N):
    """A resident FFT plan of grid N for the matrix-DFT autocorrelation
    (spectrum unused), one per (device, grid)."""
    import torch
    key = (torch.cuda.current_device(), int(N))
    p = _AUTOCORR_PLANS.get(key)
    if p is None:
        while len(_AUTOCORR_PLANS) >= _SPRITE_PLAN_CAP:
            _AUTOCORR_PLANS.pop(next(iter(_AUTOCORR_PLANS))).close()
        p = SpritePlan(N, np.array([[LAMBDA_REF_NM, 1.0, 1.0, 1.0]], np.float32))
        _AUTOCORR_PLANS[key] = p
    return p


def _sprite_plan(N, spec):
    import torch
    key = (torch.cuda.current_device(), int(N), np.ascontiguousarray(spec, np.float32).tobytes())
    hit = _SPRITE_PLANS.pop(key, None)
    if hit is None:
        while len(_SPRITE_PLANS) >= _SPRITE_PLAN_CAP:
            old = _SPRITE_PLANS.pop(next(iter(_SPRITE_PLANS)))
            old[0].close()
        hit = (SpritePlan(N, spec), {})
    _SPRITE_PLANS[key] = hit
    return hit


# ---------------------------------------------------------------------------
# Off-axis cat's-eye: survivor centre and envelope (starburst_render.cu:393-583)
# ---------------------------------------------------------------------------
SURVIVOR_EDGE_SS = 10      # envelope rim supersampling per side
SURVIVOR_CENTER_SS = 8     # centre-solve boundary supersampling per side
SURVIVOR_SCAN = 81         # centre-solve launch grid per side


def _launch_dir(ax: float, ay: float):
    """Vec3f(tan ax, tan ay, 1).normalized() in float32 (vec3.h:48-52)."""
    f = np.float32
    bx, by = f(np.tan(f(ax))), f(np.tan(f(ay)))
    ln = f(np.sqrt(f(f(bx * bx) + f(by * by)) + f(1.0)))
    inv = f(f(1.0) / ln)
    return bx, by, (f(bx * inv), f(by * inv), f(inv))


def _survives_device(lens, ox, oy, z, d, lam=LAMBDA_REF_NM):
    """Primary traces of launches (ox[k], oy[k], z) along d on the device:
    True where the ray reaches the sensor at a finite position."""
    import torch
    from .flare import trace_rays
    n = len(ox)
    if n == 0:
        return np.zeros(0, bool)
    rays = np.empty((n, 7), np.float32)
    rays[:, 0], rays[:, 1], rays[:, 2] = ox, oy, z
    rays[:, 3], rays[:, 4], rays[:, 5] = d
    rays[:, 6] = lam
    r = trace_rays(lens, torch.from_numpy(rays).cuda(), -1, -1).cpu().numpy()
    return (r[:, 4] == 0) & np.isfinite(r[:, 0]) & np.isfinite(r[:, 1])


def _boundary8(a, valid=None):
    """Cells with an 8-neighbour of the other class (among valid cells)."""
    S0, S1 = a.shape
    cls = a > 0.5
    ok = np.ones_like(cls) if valid is None else valid
    out = np.zeros_like(cls)
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            if not di and not dj:
                continue
            sh = np.zeros_like(cls)
            shv = np.zeros_like(cls)
            ys = slice(max(dj, 0), S0 + min(dj, 0))
            yd = slice(max(-dj, 0), S0 + min(-dj, 0))
            xs = slice(max(di, 0), S1 + min(di, 0))
            xd = slice(max(-di, 0), S1 + min(-di, 0))
            sh[yd, xd] = cls[ys, xs]
            shv[yd, xd] = ok[ys, xs]
            out |= shv & (sh != cls)
    return out & ok


def survivor_center(lens, ax: float, ay: float, survives=None):
    """Centroid of the spawn-plane launches whose ray reaches the sensor at
    field (ax, ay) (solve_survivor_center, starburst_render.cu:503-583):
    an 81 x 81 scan over the front element's reach, boundary cells
    supersampled 8 x 8.  Returns (cx, cy, any_survivor)."""
    f = np.float32
    survives = survives or (lambda x, y, z, d: _survives_device(lens, x, y, z, d))
    front_R = f(lens.surfaces[0].semi_aperture) if lens.surfaces else f(0.0)
    if front_R <= 0:
        return 0.0, 0.0, False
    z = f(f(lens.surfaces[0].z) - f(20.0))
    bx, by, d = _launch_dir(ax, ay)
    span_x = f(f(f(1.1) * front_R) + f(f(20.0) * f(abs(bx))))
    span_y = f(f(f(1.1) * front_R) + f(f(20.0) * f(abs(by))))
    S = SURVIVOR_SCAN
    t = (f(2.0) * np.arange(S, dtype=np.float32) / f(S - 1) - f(1.0)).astype(np.float32)
    lx = (span_x * t).astype(np.float32)
    ly = (span_y * t).astype(np.float32)
    gx, gy = np.meshgrid(lx, ly)
    surv = survives(gx.ravel(), gy.ravel(), z, d).reshape(S, S)
    bnd = _boundary8(surv.astype(np.float32))
    sx = float(np.sum(gx[surv & ~bnd], dtype=np.float64))
    sy = float(np.sum(gy[surv & ~bnd], dtype=np.float64))
    w = float(np.count_nonzero(surv & ~bnd))
    jb, ib = np.nonzero(bnd)
    if len(jb):
        K = SURVIVOR_CENTER_SS
        hx, hy = f(span_x / f(S - 1)), f(span_y / f(S - 1))
        off = ((f(2.0) * (np.arange(K, dtype=np.float32) + f(0.5)) / f(K)) - f(1.0)).astype(np.float32)
        llx = (lx[ib][:, None, None] + (hx * off)[None, None, :]).astype(np.float32)
        lly = (ly[jb][:, None, None] + (hy * off)[None, :, None]).astype(np.float32)
        llx, lly = np.broadcast_arrays(llx, lly)
        ok = survives(llx.ravel().copy(), lly.ravel().copy(), z, d)
        inv_k2 = float(f(1.0) / f(K * K))
        sx += float(np.sum(llx.ravel()[ok].astype(np.float64))) * inv_k2
        sy += float(np.sum(lly.ravel()[ok].astype(np.float64))) * inv_k2
        w += int(ok.sum()) * inv_k2
    if w > 0:
        return float(f(sx / w)), float(f(sy / w)), True
    return 0.0, 0.0, False


def survivor_envelope(lens, ep_x, ep_y, cx, cy, ax, ay, ME: int, survives=None, contains=None):
    """Cat's-eye rim-vignetting envelope over pupil [-1, 1]^2, ME x ME
    (build_survivor_envelope, starburst_render.cu:393-491): 1 where a primary
    ray launched at (cx + u ep_x, cy + v ep_y) survives, cells on the survive
    / clip boundary supersampled 10 x 10 to a coverage fraction, cells outside
    the stop filled by a radius-2 dilation from inside."""
    f = np.float32
    from ._abi import surface_array
    from . import _native
    survives = survives or (lambda x, y, z, d: _survives_device(lens, x, y, z, d))
    if contains is None:
        arr = surface_array(lens.records())

        def contains(uv):
            uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
            out = np.zeros(len(uv), np.uint8)
            _native.check(_native.load().gl_pupil_contains(
                arr, len(arr), 0, 0.0, 1, uv.ctypes.data_as(C.POINTER(C.c_float)), len(uv),
                out.ctypes.data_as(C.POINTER(C.c_uint8))), "pupil_contains")
            return out.astype(bool)
    if not lens.surfaces:
        return np.ones((ME, ME), np.float32)
    z = f(f(lens.surfaces[0].z) - f(20.0))
    _, _, d = _launch_dir(ax, ay)
    c = ((np.arange(ME, dtype=np.float32) + f(0.5)) / f(ME) * f(2.0) - f(1.0)).astype(np.float32)
    U, V = np.meshgrid(c, c)
    inside = contains(np.stack([U.ravel(), V.ravel()], 1)).reshape(ME, ME)
    env = np.full((ME, ME), -1.0, np.float32)
    ox = (f(cx) + U[inside] * f(ep_x)).astype(np.float32)
    oy = (f(cy) + V[inside] * f(ep_y)).astype(np.float32)
    env[inside] = survives(ox, oy, z, d).astype(np.float32)
    bnd = _boundary8(env, env >= 0)
    jb, ib = np.nonzero(bnd)
    if len(jb):
        K = SURVIVOR_EDGE_SS
        du = f(f(2.0) / f(ME))
        off = (du * ((np.arange(K, dtype=np.float32) + f(0.5)) / f(K) - f(0.5))).astype(np.float32)
        uu = (c[ib][:, None, None] + off[None, None, :]).astype(np.float32)
        vv = (c[jb][:, None, None] + off[None, :, None]).astype(np.float32)
        uu, vv = np.broadcast_arrays(uu, vv)
        uu, vv = uu.reshape(len(jb), -1), vv.reshape(len(jb), -1)
        ins = contains(np.stack([uu.ravel(), vv.ravel()], 1)).reshape(uu.shape)
        ok = np.zeros(uu.shape, bool)
        ox = (f(cx) + uu[ins] * f(ep_x)).astype(np.float32)
        oy = (f(cy) + vv[ins] * f(ep_y)).astype(np.float32)
        ok[ins] = survives(ox, oy, z, d)
        n_in = ins.sum(1)
        frac = np.where(n_in > 0, ok.sum(1).astype(np.float32) / np.maximum(n_in, 1).astype(np.float32),
                        env[jb, ib])
        env[jb, ib] = frac.astype(np.float32)
    # dilation of the survival into the outside band (radius 2)
    filled = env.copy()
    pad = np.pad(np.where(env >= 0, env, 0.0).astype(np.float32), 2, constant_values=0.0)
    best = np.zeros_like(env)
    for dj in range(5):
        for di in range(5):
            best = np.maximum(best, pad[dj:dj + ME, di:di + ME])
    filled[env < 0] = best[env < 0]
    return filled

"""Matrix-DFT starburst on the tensor cores (row d of the flare path).

Field form of the reference's per-wavelength triple product
(ghostlight/src/mdft_render.cu:137-173): E_l = W_y A W_x^T, I_l = |E_l|^2,
out_c = sum_l w_c(l) I_l, with
W[k][j] = exp(-2 pi i s_l (j - (n-1)/2)(k - c)).

Forms: ``"split_bf16"`` (three-term split-BF16 tcgen05 products, FP32
accumulation in tensor memory), ``"tf32"`` (tcgen05 kind::tf32) and ``"fp32"``
(FP32 on the CUDA cores).  The DFT matrices are built once per plan and stay
resident in HBM.
"""
from __future__ import annotations

import ctypes as C

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
                 center_x=None, center_y=None, stream=None):
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
        _native.check(self._lib.gl_mdft_plan_create2(
            self.n, self.Kx, self.Ky, self.n_lambda, D(*sx), D(*sy), cx, cy,
            (C.c_float * w.size)(*w.reshape(-1)), FORMS[form], st, C.byref(h)), "mdft")
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

    def set_launch(self, ctas: int = 0):
        """GEMM grid of the tensor-core forms (0 = one CTA per SM)."""
        _native.check(self._lib.gl_mdft_plan_set_launch(self._h, int(ctas)), "mdft")
        self.launch = int(ctas)

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

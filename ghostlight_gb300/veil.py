"""Veiling-glare layer (render_veil, veil_render.cu:243-414).

An achromatic glare-spread halo g(r) = (a^2 / (r^2 + a^2))^p around each
source (a = spread x sensor half-height, p = falloff), energy-normalised so
`gain` is the fraction of the source's flux it carries, area-resampled onto
the frame and tinted by the source colour.  The 1024^2 sprite is baked once
per falloff and stays resident in the plan.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from ._abi import gl_veil_params

VEIL_GRID = 1024      # side of the plan's resident sprite (gl_veil_plan_geometry reports it)


class VeilPlan:
    def __init__(self, falloff: float = 1.5, stream=None):
        import torch
        self._lib = _native.load()
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        h = C.c_void_p()
        _native.check(self._lib.gl_veil_plan_create(float(falloff), st, C.byref(h)), "veil")
        self._h = h
        self.falloff = float(falloff)

    def execute(self, sources, width: int, height: int, sensor_half_w: float, sensor_half_h: float,
                spread: float, gain: float, out_r, out_g, out_b, fmt=None, accumulate=False, stream=None):
        """sources: (N, 5) float32 [px, py, r, g, b] (buffer pixels, output-space
        colour) as a CUDA tensor (graph-capturable) or host array."""
        import torch
        src = sources if isinstance(sources, torch.Tensor) else torch.as_tensor(
            np.ascontiguousarray(sources, np.float32).reshape(-1, 5))
        if not src.is_cuda:
            src = src.to("cuda")
        src = src.contiguous()
        if src.dtype != torch.float32 or src.ndim != 2 or src.shape[1] != 5:
            raise ValueError("veil: sources must be (N, 5) float32 [px, py, r, g, b]")
        for t in (out_r, out_g, out_b):
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and t.numel() == width * height):
                raise ValueError("veil: outputs must be contiguous float32 CUDA (H, W) tensors")
        fw, fh = (width, height) if fmt is None else fmt
        prm = gl_veil_params(int(width), int(height), int(fw), int(fh), float(sensor_half_w), float(sensor_half_h),
                             float(spread), float(gain), int(bool(accumulate)))
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        self._src = src                       # keep alive until the enqueued work ran
        _native.check(self._lib.gl_veil_plan_execute(self._h, src.data_ptr(), int(src.shape[0]), C.byref(prm),
                                                     out_r.data_ptr(), out_g.data_ptr(), out_b.data_ptr(), st),
                      "veil")
        return _native.last_launch_count()

    def geometry(self, width: int, height: int, sensor_half_w: float, sensor_half_h: float, spread: float,
                 fmt=None) -> dict:
        """The scale an execute with these arguments uses: grid, ds, dx_mm
        (sensor mm per sprite texel), core_mm, falloff, core_texels."""
        from ._abi import gl_veil_geometry
        fw, fh = (width, height) if fmt is None else fmt
        prm = gl_veil_params(int(width), int(height), int(fw), int(fh), float(sensor_half_w), float(sensor_half_h),
                             float(spread), 0.0, 0)
        out = gl_veil_geometry()
        _native.check(self._lib.gl_veil_plan_geometry(self._h, C.byref(prm), C.byref(out)), "veil")
        return {k: getattr(out, k) for k, _ in gl_veil_geometry._fields_}

    def read(self, stream=None):
        """The resident unit-sum GSF sprite, (grid, grid) float32 CUDA tensor."""
        import torch
        out = torch.empty((VEIL_GRID, VEIL_GRID), dtype=torch.float32, device="cuda")
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _native.check(self._lib.gl_veil_plan_read(self._h, C.c_void_p(out.data_ptr()), C.c_void_p(st)), "veil")
        return out

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gl_veil_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_veil(sources, width: int, height: int, sensor_half_w: float, sensor_half_h: float,
                spread: float = 0.12, falloff: float = 1.5, gain: float = 0.03):
    """One-shot: {"veil_r", "veil_g", "veil_b"} float32 CUDA tensors."""
    import torch
    plan = VeilPlan(falloff)
    out = {k: torch.empty((height, width), dtype=torch.float32, device="cuda") for k in ("veil_r", "veil_g", "veil_b")}
    plan.execute(sources, width, height, sensor_half_w, sensor_half_h, spread, gain,
                 out["veil_r"], out["veil_g"], out["veil_b"])
    torch.cuda.synchronize()
    plan.close()
    return out

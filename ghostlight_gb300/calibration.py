"""Per-lens first-order setup: calibrate_lens (lens_calibration.cpp:344) and
the screen-position -> field-angle solve (source_map.cpp:182), both by
tracing the spawn disc (csrc/gl_setup.cpp).  ``precision="fp32"`` runs the
reference's float32 arithmetic, so the values equal the reference's bit for
bit; ``precision="fp64"`` runs the same measurement with double-precision
traces and solves."""
from __future__ import annotations

import ctypes as C
import dataclasses

from . import _native
from ._abi import gl_lens_calibration, gl_source_solve
from .config import LensCalibration

D_LINE_NM = 587.56

SOLVED, CONTINUED, FALLBACK = 0, 1, 2
PRECISIONS = {"fp32": 0, "fp64": 1}


def _precision(p) -> int:
    if p not in PRECISIONS:
        raise ValueError("precision must be 'fp32' or 'fp64'")
    return PRECISIONS[p]


def calibrate_lens(lens, d_line_nm: float = D_LINE_NM, precision: str = "fp32") -> LensCalibration:
    """Covered field, image circle, per-axis EFL, entrance pupil, f-number."""
    lib = _native.load()
    arr = lens.to_array()
    out = gl_lens_calibration()
    _native.check(lib.gl_calibrate_lens2(arr, len(arr), float(getattr(lens, "focal_length", 0.0) or 0.0),
                                         float(d_line_nm), _precision(precision), C.byref(out)), "calibrate_lens")
    return LensCalibration(**{k: float(getattr(out, k)) for k in LensCalibration.FIELDS})


@dataclasses.dataclass
class SourceMapSolve:
    """SourceMapSolve (source_map.h:21-47)."""
    angle_x: float
    angle_y: float
    status: int
    residual_mm: float
    anchor_ax: float
    anchor_ay: float
    anchor_x: float
    anchor_y: float
    J: tuple
    eff_half_w: float
    eff_half_h: float
    inv_tan_w: float
    inv_tan_h: float
    probe_evals: int
    _raw: object = dataclasses.field(default=None, repr=False)

    def screen(self, angle_x: float, angle_y: float):
        """Screen fraction (0..1) of a nearby field angle (source_map.cpp:456)."""
        lib = _native.load()
        sx, sy = C.c_float(), C.c_float()
        _native.check(lib.gl_source_map_screen(C.byref(self._raw), float(angle_x), float(angle_y),
                                               C.byref(sx), C.byref(sy)), "source_map_screen")
        return float(sx.value), float(sy.value)


def _calib_struct(calib) -> gl_lens_calibration:
    c = gl_lens_calibration()
    for k in LensCalibration.FIELDS:
        v = calib[k] if isinstance(calib, dict) else getattr(calib, k)
        setattr(c, k, float(v))
    c.field_crossed = 1
    return c


def solve_source_angle(lens, calib, ndc_x: float, ndc_y: float, eff_half_w: float,
                       eff_half_h: float, precision: str = "fp32") -> SourceMapSolve:
    """Field angle whose spawn-disc survivors land at (ndc_x, ndc_y) of a frame
    with half extents eff_half_w x eff_half_h mm."""
    lib = _native.load()
    arr = lens.to_array() if lens is not None else None
    out = gl_source_solve()
    c = _calib_struct(calib)
    _native.check(lib.gl_solve_source_angle2(arr, 0 if arr is None else len(arr), C.byref(c), float(ndc_x),
                                             float(ndc_y), float(eff_half_w), float(eff_half_h),
                                             _precision(precision), C.byref(out)), "solve_source_angle")
    return SourceMapSolve(out.angle_x, out.angle_y, int(out.status), out.residual_mm, out.anchor_ax, out.anchor_ay,
                          out.anchor_x, out.anchor_y, tuple(out.J), out.eff_half_w, out.eff_half_h, out.inv_tan_w,
                          out.inv_tan_h, int(out.probe_evals), out)

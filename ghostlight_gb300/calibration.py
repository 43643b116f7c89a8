"""Per-lens first-order setup: calibrate_lens (lens_calibration.cpp:344) and
the screen-position -> field-angle solve (source_map.cpp:182)."""
from __future__ import annotations

from .config import LensCalibration


def calibrate_lens(lens, d_line_nm: float = 587.56) -> LensCalibration:
    raise NotImplementedError("calibrate_lens: pass calibration= explicitly")


def solve_source_angle(lens, calib, ndc_x, ndc_y, eff_half_w, eff_half_h):
    raise NotImplementedError("solve_source_angle: pass source_angle= explicitly")

"""ctypes mirror of the plain-C data formats in include/ghostlight_gb300.h.

Every struct here has exactly the field order and 4-byte field types of its C
counterpart, so an array of them can be handed to the C-ABI as a pointer.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

GL_OK = 0
GL_ERR_INVALID = -1
GL_ERR_OOM = -2
GL_ERR_CUDA = -3
GL_ERR_TIMEOUT = -4
GL_ERR_BUDGET = -5
GL_ERR_NO_DEVICE = -6
GL_ERR_UNSUPPORTED = -7


class gl_surface(C.Structure):
    _fields_ = [
        ("radius", C.c_float), ("thickness", C.c_float), ("ior", C.c_float),
        ("abbe_v", C.c_float), ("semi_aperture", C.c_float), ("z", C.c_float),
        ("is_stop", C.c_int32), ("is_active", C.c_int32),
        ("aperture_shape", C.c_int32), ("aperture_blades", C.c_int32),
        ("aperture_rotation_rad", C.c_float), ("aperture_aspect", C.c_float),
        ("aperture_curvature", C.c_float), ("aperture_twist", C.c_float),
        ("aperture_notch_rad", C.c_float), ("aperture_notch_angle_rad", C.c_float),
        ("decenter_x", C.c_float), ("decenter_y", C.c_float),
        ("rot", C.c_float * 9),
        ("form", C.c_int32), ("conic_k", C.c_float),
        ("asphere_terms", C.c_float * 8), ("n_asphere_terms", C.c_int32),
        ("cyl_axis", C.c_int32), ("disp_model", C.c_int32),
        ("sellmeier_B", C.c_float * 3), ("sellmeier_C", C.c_float * 3),
        ("coating_model", C.c_int32), ("ar_layers", C.c_int32),
        ("tint_r", C.c_float), ("tint_g", C.c_float), ("tint_b", C.c_float),
        ("tint_strength", C.c_float),
        ("gauss_sigma", C.c_float), ("gauss_background", C.c_float),
        ("gauss_peak", C.c_float), ("gauss_decenter_x", C.c_float),
        ("gauss_decenter_y", C.c_float),
    ]


class gl_spectral_sample(C.Structure):
    _fields_ = [("lambda_", C.c_float), ("cmf_r", C.c_float),
                ("cmf_g", C.c_float), ("cmf_b", C.c_float)]


class gl_pupil_sample(C.Structure):
    _fields_ = [("u", C.c_float), ("v", C.c_float)]


class gl_ghost_pair(C.Structure):
    _fields_ = [("surf_a", C.c_int32), ("surf_b", C.c_int32)]


class gl_flare_source(C.Structure):
    _fields_ = [("angle_x", C.c_float), ("angle_y", C.c_float),
                ("r", C.c_float), ("g", C.c_float), ("b", C.c_float)]


class gl_sampler_params(C.Structure):
    _fields_ = [("ray_grid", C.c_int32), ("pupil_jitter", C.c_int32),
                ("jitter_seed", C.c_int32), ("blades_override", C.c_int32),
                ("rotation_deg", C.c_float)]


class gl_filter_params(C.Structure):
    _fields_ = [("min_ghost_intensity", C.c_float), ("ghost_normalize", C.c_int32),
                ("max_area_boost", C.c_float)]


class gl_ghost_render_params(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("fmt_w", C.c_int32), ("fmt_h", C.c_int32),
                ("fmt_x0", C.c_int32), ("fmt_y0", C.c_int32),
                ("sensor_half_w", C.c_float), ("sensor_half_h", C.c_float),
                ("flare_gain", C.c_float), ("apply_correction", C.c_int32),
                ("correction", C.c_float * 9), ("plain_per_pair", C.c_int32),
                ("splat_mode", C.c_int32), ("cull_dead_pairs", C.c_int32),
                ("blades_override", C.c_int32), ("rotation_deg", C.c_float)]


CALIBRATION_FIELDS = ["sensor_half_w", "sensor_half_h", "max_half_angle_h", "max_half_angle_v",
                      "image_circle_semi_w", "image_circle_semi_h", "focal_length_x", "focal_length_y",
                      "entrance_pupil_semi_x", "entrance_pupil_semi_y", "f_number_x", "f_number_y",
                      "pupil_area_frac"]


class gl_lens_calibration(C.Structure):
    _fields_ = [(n, C.c_float) for n in CALIBRATION_FIELDS] + [("field_crossed", C.c_int32)]


class gl_source_solve(C.Structure):
    _fields_ = [("angle_x", C.c_float), ("angle_y", C.c_float), ("status", C.c_int32),
                ("residual_mm", C.c_float), ("anchor_ax", C.c_float), ("anchor_ay", C.c_float),
                ("anchor_x", C.c_float), ("anchor_y", C.c_float), ("J", C.c_float * 4),
                ("eff_half_w", C.c_float), ("eff_half_h", C.c_float), ("inv_tan_w", C.c_float),
                ("inv_tan_h", C.c_float), ("probe_evals", C.c_int32)]


class gl_veil_params(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("fmt_w", C.c_int32), ("fmt_h", C.c_int32),
                ("sensor_half_w", C.c_float), ("sensor_half_h", C.c_float), ("spread", C.c_float),
                ("gain", C.c_float), ("accumulate", C.c_int32)]


class gl_veil_geometry(C.Structure):
    _fields_ = [("grid", C.c_int32), ("ds", C.c_int32), ("dx_mm", C.c_float), ("core_mm", C.c_float),
                ("falloff", C.c_float), ("core_texels", C.c_float)]


class gl_psf_cell(C.Structure):
    _fields_ = [("beam_ax", C.c_float), ("beam_ay", C.c_float), ("chief_x_mm", C.c_float),
                ("chief_y_mm", C.c_float), ("status", C.c_int32), ("pupil_fraction", C.c_float),
                ("aim_residual_mm", C.c_float)]


class gl_psf_source(C.Structure):
    _fields_ = [("angle_x", C.c_float), ("angle_y", C.c_float), ("r", C.c_float), ("g", C.c_float),
                ("b", C.c_float), ("chief_x_mm", C.c_float), ("chief_y_mm", C.c_float),
                ("tile_x0", C.c_int32), ("tile_y0", C.c_int32)]


SURFACE_DTYPE = np.dtype([(name, np.float32 if t in (C.c_float,) else np.int32)
                          if not hasattr(t, "_length_") else
                          (name, np.float32, (t._length_,))
                          for name, t in gl_surface._fields_])
assert SURFACE_DTYPE.itemsize == C.sizeof(gl_surface)


def surface_array(surfaces) -> "C.Array[gl_surface]":
    """Pack a sequence of gl_surface into a contiguous ctypes array."""
    arr = (gl_surface * len(surfaces))()
    for i, s in enumerate(surfaces):
        arr[i] = s
    return arr


def default_surface() -> gl_surface:
    """A Surface with the reference defaults (optical_system.h:157-249)."""
    s = gl_surface()
    s.ior = 1.0
    s.is_active = 1
    s.aperture_aspect = 1.0
    s.rot[0] = s.rot[4] = s.rot[8] = 1.0
    s.tint_r = s.tint_g = s.tint_b = 1.0
    s.tint_strength = 0.04
    return s

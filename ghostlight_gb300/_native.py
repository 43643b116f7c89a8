"""Loader of libghostlight_gb300.so, the C-ABI of include/ghostlight_gb300.h.

There is no fallback: if the shared library is missing or fails to load, every
entry point raises.  ``load()`` builds it in-tree first when the sources are
newer (nvcc cross-compiles without a GPU).
"""
from __future__ import annotations

import ctypes as C
import threading

from . import _abi
from ._abi import (gl_filter_params, gl_flare_source, gl_ghost_pair, gl_ghost_render_params,
                   gl_lens_calibration, gl_pupil_sample, gl_sampler_params, gl_source_solve,
                   gl_spectral_sample, gl_surface, gl_veil_params, gl_veil_geometry, gl_psf_cell, gl_psf_source)

_lock = threading.Lock()
_lib = None


class GhostlightError(RuntimeError):
    """A CUDA / device failure reported by the C-ABI."""


def _declare(lib):
    P = C.POINTER
    i, f, vp = C.c_int, C.c_float, C.c_void_p
    lib.gl_last_error.restype = C.c_char_p
    lib.gl_version.restype = i
    lib.gl_last_launch_count.restype = i
    lib.gl_finalize_z.argtypes = [P(gl_surface), i]
    lib.gl_euler_rotation.argtypes = [C.c_float, C.c_float, C.c_float, P(C.c_float)]
    fp = P(C.c_float)
    vp_ = C.c_void_p
    lib.gl_build_pupil2.argtypes = [P(gl_surface), i, i, C.c_float, i, C.c_float, i, vp_, i, vp_, vp_]
    lib.gl_pupil_contains.argtypes = [P(gl_surface), i, i, C.c_float, i, fp, i, P(C.c_uint8)]
    lib.gl_ghost_plan_stats.argtypes = [vp_, P(C.c_ulonglong), vp_]
    lib.gl_sprite_plan_create.argtypes = [i, P(gl_spectral_sample), i, C.c_float, P(vp_)]
    lib.gl_sprite_plan_bake.argtypes = [vp_, vp_, i, vp_]
    lib.gl_sprite_plan_splat.argtypes = [vp_, fp, i, C.c_float, C.c_float, C.c_float, C.c_float, i, i, C.c_float,
                                         vp_, vp_, vp_, i, i, vp_]
    lib.gl_sprite_plan_read.argtypes = [vp_, vp_, vp_, P(C.c_double), P(i), vp_]
    lib.gl_sprite_plan_destroy.argtypes = [vp_]
    lib.gl_sprite_splat_source.argtypes = [vp_, i, f, f, f, f, f, f, f, f, f, i, i, f, vp_, vp_, vp_, i, i, vp_]
    lib.gl_coating_table_create.argtypes = [i, fp, i, fp, i, fp, C.c_float, i, P(i)]
    lib.gl_coating_table_info.argtypes = [i, P(i), P(i), P(i), fp, P(i)]
    lib.gl_coating_table_read.argtypes = [i, fp, fp, fp]
    lib.gl_aperture_image_create.argtypes = [i, i, fp, C.c_float, P(i)]
    lib.gl_coating_table_prepare.argtypes = [i]
    lib.gl_coating_bake_layers.argtypes = [P(gl_surface), i, i, i, fp, P(i), fp, fp, fp, P(i)]
    lib.gl_blade_radius.argtypes = [i, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, P(C.c_float), i,
                                    P(C.c_float)]
    lib.gl_enumerate_ghost_pairs.argtypes = [P(gl_surface), i, P(gl_ghost_pair), i, P(i)]
    lib.gl_build_aperture_samples.argtypes = [P(gl_surface), i, P(gl_sampler_params),
                                              P(gl_pupil_sample), i, P(i)]
    lib.gl_build_spectral_table.argtypes = [i, i, P(f), P(gl_spectral_sample), P(f)]
    lib.gl_color_matrices.argtypes = [i, P(f), i, P(f), P(f), P(f)]
    lib.gl_filter_ghost_pairs.argtypes = [P(gl_surface), i, f, f, P(gl_filter_params),
                                          P(gl_ghost_pair), P(f), P(f), i, P(i), P(i)]
    lib.gl_trace_rays.argtypes = [P(gl_surface), i, i, i, vp, i, vp, vp]
    lib.gl_trace_rays_noalloc.argtypes = [P(gl_surface), i, i, i, vp, i, vp, vp]
    render_args = [P(gl_surface), i, P(gl_ghost_pair), P(f), P(C.c_int32), i,
                   P(gl_flare_source), i, P(gl_pupil_sample), P(C.c_int32), i,
                   P(gl_spectral_sample), i, P(gl_ghost_render_params)]
    lib.gl_render_ghosts.argtypes = render_args + [vp, vp, vp, vp]
    lib.gl_ghost_plan_create.argtypes = render_args + [P(vp)]
    lib.gl_ghost_plan_execute.argtypes = [vp, vp, vp, vp, vp]
    lib.gl_ghost_plan_info.argtypes = [vp, P(C.c_longlong), P(i), P(i)]
    lib.gl_ghost_plan_destroy.argtypes = [vp]
    lib.gl_ghost_plan_pair_hits.argtypes = [vp, P(C.c_int32), i]
    lib.gl_ghost_plan_traced.argtypes = [vp, P(C.c_longlong)]
    lib.gl_ghost_plan_traced_split.argtypes = [vp, P(C.c_longlong), P(C.c_longlong)]
    lib.gl_ghost_plan_set_timing.argtypes = [vp, vp, vp, vp]
    lib.gl_morton_order.argtypes = [P(gl_pupil_sample), i, P(gl_pupil_sample)]
    lib.gl_ghost_plan_set_launch.argtypes = [vp, i, i]
    lib.gl_ghost_plan_set_lambda_split.argtypes = [vp, i]
    lib.gl_gemm_bf16_tc.argtypes = [vp, vp, vp, i, i, i, vp]
    d = C.c_double
    lib.gl_mdft_plan_create.argtypes = [i, i, i, P(d), P(d), d, d, P(f), i, vp, P(vp)]
    lib.gl_mdft_plan_execute.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.gl_mdft_plan_status.argtypes = [vp, P(i)]
    lib.gl_mdft_plan_destroy.argtypes = [vp]
    lib.gl_mdft_plan_create2.argtypes = [i, i, i, i, P(d), P(d), d, d, P(f), i, vp, P(vp)]
    lib.gl_mdft_plan_set_center.argtypes = [vp, d, d, vp]
    lib.gl_mdft_plan_create3.argtypes = [i, i, i, i, P(d), P(d), d, d, P(f), i, i, f, vp, P(vp)]
    lib.gl_mdft_plan_execute3.argtypes = [vp, vp, vp, vp, vp, i, i, i, i, i, i, i, P(f), vp]
    lib.gl_sprite_plan_autocorr.argtypes = [vp, vp, i, vp, i, i, vp]
    lib.gl_mdft_plan_set_launch.argtypes = [vp, i]
    lib.gl_mdft_plan_set_tile.argtypes = [vp, i]
    lib.gl_mdft_plan_set_lambda_range.argtypes = [vp, i, i]
    lib.gl_mdft_plan_execute2.argtypes = [vp, vp, vp, vp, vp, i, vp]
    lib.gl_build_pupil.argtypes = [P(gl_surface), i, i, f, i, f, vp, vp]
    lib.gl_conv2d_plan_create.argtypes = [i, i, P(f), i, i, vp, P(vp)]
    lib.gl_conv2d_plan_execute.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    lib.gl_conv2d_plan_execute2.argtypes = [vp] + [vp] * 9 + [vp]
    lib.gl_conv2d_plan_info.argtypes = [vp, P(i), P(i)]
    lib.gl_conv2d_plan_destroy.argtypes = [vp]
    ll = C.c_longlong
    lib.gl_lens_create.argtypes = [P(gl_surface), i, P(gl_ghost_pair), P(f), i, i, f, P(vp)]
    lib.gl_lens_prepare.argtypes = [vp, i, P(gl_spectral_sample), i]
    lib.gl_lens_info.argtypes = [vp, P(i), P(ll)]
    lib.gl_lens_destroy.argtypes = [vp]
    lib.gl_request_create.argtypes = [vp, i, P(gl_spectral_sample), i, P(gl_flare_source), i,
                                      P(gl_ghost_render_params), vp, P(vp)]
    lib.gl_request_enqueue.argtypes = [vp, vp, vp, vp, i, vp]
    lib.gl_request_set_lambda_split.argtypes = [vp, i]
    lib.gl_request_planes.argtypes = [vp, P(vp)]
    lib.gl_request_copy_out.argtypes = [vp, vp, vp]
    lib.gl_request_info.argtypes = [vp, P(ll), P(ll), P(i)]
    lib.gl_request_traced.argtypes = [vp, P(ll), vp]
    lib.gl_request_destroy.argtypes = [vp, vp]
    lib.gl_pool_info.argtypes = [P(ll), P(ll)]
    lib.gl_pool_trim.argtypes = [ll]
    lib.gl_psf_prepass.argtypes = [P(gl_surface), i, P(f), i, i, P(gl_psf_cell)]
    lib.gl_psf_render.argtypes = [P(gl_surface), i, P(gl_psf_source), i, P(gl_pupil_sample), i,
                                  P(gl_spectral_sample), i, i, i, i, i, f, i, f, i, vp, vp, vp, vp]
    lib.gl_psf_render_async.argtypes = lib.gl_psf_render.argtypes
    lib.gl_veil_plan_create.argtypes = [f, vp, P(vp)]
    lib.gl_veil_plan_execute.argtypes = [vp, vp, i, P(gl_veil_params), vp, vp, vp, vp]
    lib.gl_veil_plan_destroy.argtypes = [vp]
    lib.gl_veil_plan_geometry.argtypes = [vp, P(gl_veil_params), P(gl_veil_geometry)]
    lib.gl_veil_plan_read.argtypes = [vp, vp, vp]
    lib.gl_calibrate_lens.argtypes = [P(gl_surface), i, f, f, P(gl_lens_calibration)]
    lib.gl_calibrate_lens2.argtypes = [P(gl_surface), i, f, f, i, P(gl_lens_calibration)]
    lib.gl_solve_source_angle2.argtypes = [P(gl_surface), i, P(gl_lens_calibration), f, f, f, f, i,
                                           P(gl_source_solve)]
    lib.gl_solve_source_angle.argtypes = [P(gl_surface), i, P(gl_lens_calibration), f, f, f, f,
                                          P(gl_source_solve)]
    lib.gl_source_map_screen.argtypes = [P(gl_source_solve), f, f, P(f), P(f)]
    return lib


def load():
    """Return the loaded library, building it first if it is stale."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            from . import build as _build
            path = _build.build()
            _lib = _declare(C.CDLL(str(path)))
    return _lib


def lib_path():
    from . import build as _build
    return _build.LIB


def check(rc: int, what: str = "") -> None:
    """Map a GL_* status to the reference's exception types."""
    if rc == _abi.GL_OK:
        return
    msg = (_lib.gl_last_error() or b"").decode(errors="replace") if _lib is not None else ""
    if what and not msg.startswith(what):
        msg = "%s: %s" % (what, msg)
    if rc in (_abi.GL_ERR_INVALID, _abi.GL_ERR_UNSUPPORTED):
        raise ValueError(msg)
    raise GhostlightError(msg)


def last_launch_count() -> int:
    return int(load().gl_last_launch_count())

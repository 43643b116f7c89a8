"""ghostlight_gb300 — the Ghostlight flare hot path on GB300 (sm_103a).

The call surface mirrors the reference Python package (ghostlight): lens
model, ghost-pair enumeration and filter, ray traces, and the flare renders,
all executed by hand-written CUDA kernels in libghostlight_gb300.so.
"""
from .config import (DiffractionConfig, FlareConfig, GhostAovMode, GhostFilter, GhostFilterMode,
                     InputColorSpace, LensCalibration, OutputColorSpace, PointFlareConfig, PSFConfig,
                     RenderConfig, StarburstEngine)
from .optics import (ApertureShape, Coating, CoatingModel, CylinderAxis, DispersionModel,
                     OpticalSystem, Ray, Surface, SurfaceForm, TraceResult, TraceStatus, Vec3f)
from .flare import (GhostPair, GhostRenderPlan, enumerate_ghost_pairs, filter_ghost_pairs,
                    prepare_ghost_render, pupil_grid, render_ghosts, render_point_flare,
                    render_source_flare, spectral_table, trace_ghost_ray, trace_primary_ray,
                    trace_rays)
from .calibration import calibrate_lens, solve_source_angle
from .starburst import MdftPlan, mdft_starburst_eform
from .psf import ConvPlan, convolve_psf, synthetic_psf_kernel
from .apertures import curved_blade_mask
from .psf_grid import render_psf
from .veil import render_veil
from .lensfile import lens_format_version, load_lens, save_lens
from .debug import _render_starburst_debug, _render_veil_debug

__version__ = "0.1.0"


def _cuda_available() -> bool:
    try:
        import torch
        return bool(torch.cuda.is_available())
    except Exception:
        return False

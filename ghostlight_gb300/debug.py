"""Validation captures of the diffraction layers: the reference's
_render_starburst_debug and _render_veil_debug (bind_renderers.cpp:194-286).

Each renders one source placed as render_point_flare places it (the
production source-angle solve of config.source_x / source_y, the colour
through input_cs -> XYZ -> output_cs; make_debug_source,
bind_renderers.cpp:45-79) and returns the layer together with the
intermediates the reference's StarburstDebug / VeilDebug capture
(diffraction.h:22-40, veil_render.h:31-40), as host numpy arrays under the
reference's keys.  The layers come from the same device pipeline as the
frame render; the intermediates are read back from it.
"""
from __future__ import annotations

import numpy as np

from .config import LensCalibration, PointFlareConfig
from .optics import OpticalSystem


def _debug_source(width: int, height: int, lens: OpticalSystem, calibration: LensCalibration,
                  config: PointFlareConfig):
    """(eff_half_w, eff_half_h, field angle, (1, 5) [px, py, r, g, b])."""
    from .calibration import solve_source_angle
    from .flare import _eff_half, source_rgb
    if width <= 0 or height <= 0:
        raise ValueError("width and height must be positive")
    if lens.num_surfaces() <= 0:
        raise ValueError("lens has no surfaces")
    hw, hh = _eff_half(config, calibration)
    f = np.float32
    smap = solve_source_angle(lens, calibration, float((f(config.source_x) - f(0.5)) * f(2.0)),
                              float((f(config.source_y) - f(0.5)) * f(2.0)), hw, hh,
                              precision=getattr(config, "setup_precision", "fp32"))
    r, g, b = source_rgb(config, config.source_r, config.source_g, config.source_b)
    sx, sy = smap.screen(smap.angle_x, smap.angle_y)
    pos = np.array([[f(sx) * f(width), f(sy) * f(height), r, g, b]], np.float32)
    return hw, hh, (float(f(smap.angle_x)), float(f(smap.angle_y))), pos


def _host(planes, keys):
    return {k: planes[k].cpu().numpy() for k in keys}


def _render_starburst_debug(width: int, height: int, lens: OpticalSystem, calibration: LensCalibration,
                            config: PointFlareConfig) -> dict:
    """The starburst layer of one source with its PSF (grid^2, DC-centred,
    unit sum, at 550 nm), RGB sprite (grid^2 x 3, baked over the config's
    wavelengths at full resolution), effective pupil, texel pitch, first-order
    optics, field angle, throughput and survivor-centre offset.  The
    matrix-DFT engine has no sprite: psf and sprite_rgb are zeros, as in the
    reference.  With diffraction.starburst off the layer is black and the
    capture empty (grid 0)."""
    import torch
    from .flare import starburst_layer_for
    from .starburst import LAMBDA_REF_NM, SpritePlan, effective_pupil_info, starburst_spectrum
    hw, hh, field, pos = _debug_source(width, height, lens, calibration, config)
    keys = ("starburst_r", "starburst_g", "starburst_b")
    d = {"width": int(width), "height": int(height), "grid": 0}
    z2 = np.zeros((0, 0), np.float32)
    scal = dict(dx_mm_x=0.0, dx_mm_y=0.0, f_number_x=0.0, f_number_y=0.0, focal_length_x=0.0, focal_length_y=0.0,
                entrance_pupil_semi_x=0.0, entrance_pupil_semi_y=0.0, lambda_ref_nm=0.0, field_angle_x=0.0,
                field_angle_y=0.0, throughput=1.0, chief_offset_x=0.0, chief_offset_y=0.0)
    if not bool(config.diffraction.starburst):
        d.update({k: np.zeros((height, width), np.float32) for k in keys})
        d.update(psf=z2, sprite_rgb=np.zeros((0, 0, 3), np.float32), pupil=z2, **scal)
        d.update(source_px=float(pos[0, 0]), source_py=float(pos[0, 1]))
        return d
    layer, geo = starburst_layer_for(lens, calibration, config, pos, width, height, hw, hh, field)
    torch.cuda.synchronize()
    d.update(_host(layer, keys))
    N = int(geo["N"])
    info = effective_pupil_info(lens, config, geo, field)
    d["grid"] = N
    pupil = info["pupil"]
    d["pupil"] = pupil.cpu().numpy() if pupil is not None else np.zeros((N, N), np.float32)
    psf = np.zeros((N, N), np.float32)
    sprite = np.zeros((N, N, 3), np.float32)
    live = pupil is not None and info["T"] >= 1e-3
    if live and geo["engine"] == "sprite":
        plan = SpritePlan(N, starburst_spectrum(config))
        try:
            plan.bake(pupil, 1)
            raw, spr, e = plan.read()
            torch.cuda.synchronize()
        finally:
            plan.close()
        k = np.float32(1.0 / e) if e > 0 else np.float32(0.0)
        psf = (raw.cpu().numpy() * k).astype(np.float32)
        sprite = spr.cpu().numpy()
    f = np.float32
    d.update(psf=psf, sprite_rgb=sprite)
    d.update(dx_mm_x=float(f(geo["sx"])), dx_mm_y=float(f(geo["sy"])), f_number_x=geo["fnum_x"],
             f_number_y=geo["fnum_y"], focal_length_x=geo["efl_x"], focal_length_y=geo["efl_y"],
             entrance_pupil_semi_x=geo["ep_x"], entrance_pupil_semi_y=geo["ep_y"], lambda_ref_nm=LAMBDA_REF_NM,
             field_angle_x=field[0], field_angle_y=field[1], throughput=float(f(info["T"])),
             chief_offset_x=float(f(info["chief"][0])), chief_offset_y=float(f(info["chief"][1])))
    d.update(source_px=float(pos[0, 0]), source_py=float(pos[0, 1]))
    return d


def _render_veil_debug(width: int, height: int, lens: OpticalSystem, calibration: LensCalibration,
                       config: PointFlareConfig) -> dict:
    """The veil layer of one source with its unit-sum glare-spread function
    (grid^2, DC-centred), the neutral RGB sprite the reference replicates it
    into, the texel pitch, core radius (mm and texels) and falloff used.
    With diffraction.veil off the layer is black and the capture empty."""
    import torch
    from .veil import VeilPlan
    hw, hh, _field, pos = _debug_source(width, height, lens, calibration, config)
    dc = config.diffraction
    keys = ("veil_r", "veil_g", "veil_b")
    d = {"width": int(width), "height": int(height), "grid": 0}
    if not bool(dc.veil):
        d.update({k: np.zeros((height, width), np.float32) for k in keys})
        d.update(dx_mm_x=0.0, dx_mm_y=0.0, core_mm=0.0, falloff=0.0, core_texels=0.0,
                 source_px=float(pos[0, 0]), source_py=float(pos[0, 1]))
        return d
    plan = VeilPlan(dc.veil_falloff)
    try:
        layer = {k: torch.empty((height, width), dtype=torch.float32, device="cuda") for k in keys}
        plan.execute(pos, width, height, hw, hh, dc.veil_spread, dc.veil_gain, *(layer[k] for k in keys))
        geo = plan.geometry(width, height, hw, hh, dc.veil_spread)
        ref = plan.read()
        torch.cuda.synchronize()
    finally:
        plan.close()
    d.update(_host(layer, keys))
    gsf = ref.cpu().numpy()
    d.update(grid=int(geo["grid"]), reference=gsf, sprite_rgb=np.repeat(gsf[:, :, None], 3, axis=2),
             dx_mm_x=geo["dx_mm"], dx_mm_y=geo["dx_mm"], core_mm=geo["core_mm"], falloff=geo["falloff"],
             core_texels=geo["core_texels"], source_px=float(pos[0, 0]), source_py=float(pos[0, 1]))
    return d

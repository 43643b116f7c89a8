"""Pin the FP64 restatement of the reference's matrix-DFT engine
(oracle/mdft_box_oracle.py) to the reference's own GPU goldens
(validation/goldens/aperture_baseline/*__starburst_mdft.npy, packed in
tests/golden/ref_goldens.npz) on all five lenses.

The restatement takes the stop amplitude built from the oracle's pinned
PupilMask::contains, the starburst's first-order scalars and spectral table
from the product's host code (themselves pinned bit for bit elsewhere) and
evaluates mdft_render.cu:199-340 in float64.  The goldens carry the
reference GPU's float32 rounding, so the bar is 1e-4 relative L2 (measured
5e-6 to 7e-6).
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

_META = json.loads((GOLDEN / "ref_goldens.json").read_text())
LENSES = ["double_gauss", "sirui", "hex_stop", "hex_rot30", "blade_shape"]


def unpack(b, shape):
    return np.ascontiguousarray(b.T).reshape(-1).view(np.float32).reshape(shape).copy()


@pytest.mark.parametrize("name", LENSES)
def test_mdft_box_oracle_matches_reference_golden(name):
    import ghostlight_gb300 as gl
    from ghostlight_gb300._abi import gl_surface
    from ghostlight_gb300.calibration import solve_source_angle
    from ghostlight_gb300.flare import source_rgb
    from ghostlight_gb300.starburst import sprite_geometry, starburst_spectrum
    from oracle import mdft_box_oracle as MB
    from oracle import oracle as O
    packed = np.load(GOLDEN / "ref_goldens.npz")
    key = "ab/%s__starburst_mdft" % name
    g = _META["goldens"][key]
    raw = packed["lens/" + name]
    recs = list((gl_surface * raw.shape[0]).from_buffer_copy(raw.tobytes()))
    lens = gl.OpticalSystem.from_records(recs, focal_length=_META["lenses"][name]["focal_length"])
    cal = gl.LensCalibration.from_dict(_META["lenses"][name]["calibration"])
    cfg = gl.PointFlareConfig(spectral_samples=g["spectral_samples"], source_x=0.5, source_y=0.5)
    cfg.diffraction.starburst = True
    cfg.diffraction.starburst_engine = gl.StarburstEngine.MDFT
    cfg.diffraction.starburst_grid = g["starburst_grid"]
    cfg.diffraction.pupil_fill = g["pupil_fill"]
    cfg.diffraction.scale_trim = g["scale_trim"]
    cfg.diffraction.spectral_samples = g["sb_spectral_samples"]
    hw, hh = cal.sensor_half_w, cal.sensor_half_h
    sm = solve_source_angle(lens, cal, 0.0, 0.0, hw, hh)
    sx, sy = sm.screen(sm.angle_x, sm.angle_y)
    r, gg, b = source_rgb(cfg, g["source_rgb"], g["source_rgb"], g["source_rgb"])
    W, H = g["W"], g["H"]
    pos = np.array([[sx * W, sy * H, r, gg, b]], np.float32)
    geo = sprite_geometry(cal, cfg, pos, W, H, hw, hh, front_R=recs[0].semi_aperture)
    assert geo["engine"] == "mdft"
    A = MB.pupil(lambda uv: O.pupil_contains(recs, uv, 0, 0.0, aspect_one=True), geo["N"], geo["fill"])
    img = MB.render(A, g["pupil_fill"], starburst_spectrum(cfg), 550.0, geo["sx"], geo["sy"], geo["px_mm_x"],
                    geo["px_mm_y"], pos, geo["gain"], W, H)
    want = unpack(packed["img/" + key], tuple(g["shape"])).transpose(2, 0, 1)
    assert rel_l2(img, want) < 1e-4

"""Veiling glare against the FP64 restatement, and its energy."""
import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,hw,hh,spread,falloff", [(256, 192, 12.0, 9.0, 0.12, 1.5),
                                                      (512, 512, 18.0, 18.0, 0.05, 2.2),
                                                      (300, 200, 6.0, 4.0, 0.4, 1.0)])
def test_veil_matches_fp64(W, H, hw, hh, spread, falloff):
    from ghostlight_gb300.veil import render_veil
    from oracle import veil_oracle as VO
    src = np.array([[W * 0.4 + 0.3, H * 0.55 - 0.2, 1.0, 0.7, 0.4],
                    [W * 0.9, H * 0.1 + 0.5, 0.2, 0.5, 1.0]], np.float32)
    out = render_veil(src, W, H, hw, hh, spread, falloff, 0.03)
    got = np.stack([out[k].cpu().numpy() for k in ("veil_r", "veil_g", "veil_b")]).astype(np.float64)
    want = VO.render(src, W, H, hw, hh, spread, falloff, 0.03)
    # float32 texel coordinates reach M/2 = 512, so a pixel's overlap widths carry
    # ~1e-4 relative rounding in the reference's own formulation
    assert rel_l2(got, want) < 1e-4


def test_veil_energy_is_gain_times_flux():
    """A small halo well inside the frame carries gain x source flux."""
    from ghostlight_gb300.veil import render_veil
    W = H = 512
    out = render_veil(np.array([[256.0, 256.0, 2.0, 1.0, 0.5]], np.float32), W, H, 18.0, 18.0,
                      spread=0.02, falloff=2.5, gain=0.05)
    for k, flux in (("veil_r", 2.0), ("veil_g", 1.0), ("veil_b", 0.5)):
        assert abs(out[k].double().sum().item() - 0.05 * flux) < 1e-3 * 0.05 * flux


def test_point_flare_with_veil_layer(pins, meta):
    """render_point_flare with the veil switched on returns veil_r/g/b centred on
    the solved source image point."""
    import ghostlight_gb300 as gl
    from conftest import lens_from_pins
    lens = gl.OpticalSystem.from_records(lens_from_pins(pins, "cfg1_double_gauss_12"))
    cal = gl.LensCalibration.from_dict(meta["cfg1_double_gauss_12"]["calibration"])
    cfg = gl.PointFlareConfig(ray_grid=32, spectral_samples=8, source_x=0.7, source_y=0.4)
    cfg.diffraction.veil = True
    cfg.diffraction.veil_spread = 0.05
    out = gl.render_point_flare(256, 256, lens, cal, cfg)
    assert {"ghost_r", "veil_r", "veil_g", "veil_b"} <= set(out)
    v = out["veil_g"].cpu().numpy()
    y, x = np.unravel_index(np.argmax(v), v.shape)
    assert abs(x - 0.7 * 256) <= 3 and abs(y - 0.4 * 256) <= 3


def test_point_flare_with_starburst_layer(pins, meta):
    """render_point_flare with the starburst switched on returns starburst_r/g/b:
    the pattern peaks on the source's image point and carries at most
    starburst_gain x the source flux (one period of the pattern)."""
    import ghostlight_gb300 as gl
    from conftest import lens_from_pins
    lens = gl.OpticalSystem.from_records(lens_from_pins(pins, "cfg1_double_gauss_12"))
    cal = gl.LensCalibration.from_dict(meta["cfg1_double_gauss_12"]["calibration"])
    cfg = gl.PointFlareConfig(ray_grid=32, spectral_samples=8, source_x=0.6, source_y=0.45)
    cfg.diffraction.starburst = True
    cfg.diffraction.scale_trim = 200.0         # enlarge: one period of the pattern spans the frame
    out = gl.render_point_flare(250, 200, lens, cal, cfg)
    assert {"ghost_r", "starburst_r", "starburst_g", "starburst_b"} <= set(out)
    g = out["starburst_g"].cpu().numpy()
    assert g.shape == (200, 250) and np.isfinite(g).all() and g.max() > 0
    y, x = np.unravel_index(np.argmax(g), g.shape)
    assert abs(x - 0.6 * 250) <= 2 and abs(y - 0.45 * 200) <= 2

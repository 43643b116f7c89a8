"""SPRITE starburst engine on the host: the setup scalars of
render_starburst (starburst_render.cu:620-711, :1003-1070) — engine choice,
grid growth, box-sum factor, footprint, gain — and the FP64 restatement's
own invariants (unit-energy PSF, energy-conserving splat)."""
import numpy as np
import pytest

from ghostlight_gb300.config import LensCalibration, PointFlareConfig, StarburstEngine
from ghostlight_gb300.starburst import _po2_floor, sprite_geometry, starburst_spectrum
from oracle import sprite_oracle as SO


def _cal(**kw):
    c = LensCalibration()
    c.sensor_half_w, c.sensor_half_h = 18.0, 12.0
    c.focal_length_x = c.focal_length_y = 50.0
    c.entrance_pupil_semi_x = c.entrance_pupil_semi_y = 12.5     # f/2
    c.image_circle_semi_w, c.image_circle_semi_h = 20.0, 14.0
    c.pupil_area_frac = 0.9
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _cfg(trim=1.0, engine=StarburstEngine.SPRITE, grid=1024):
    cfg = PointFlareConfig(spectral_samples=16)
    cfg.diffraction.starburst = True
    cfg.diffraction.scale_trim = trim
    cfg.diffraction.starburst_engine = engine
    cfg.diffraction.starburst_grid = grid
    return cfg


SRC = np.array([[960.0, 540.0, 1, 1, 1]], np.float32)


def test_po2_floor():
    assert [_po2_floor(x, 128) for x in (0.3, 1.0, 1.9, 2.0, 7.9, 8.0, 1000.0)] == [1, 1, 1, 2, 4, 8, 128]


def test_plain_geometry():
    g = sprite_geometry(_cal(), _cfg(), SRC, 1920, 1080, 18.0, 12.0)
    f = np.float32
    dx = f(f(f(550.0) * f(1e-6)) * f(2.0)) * f(0.3)
    assert g["engine"] == "sprite" and g["N"] == 1024
    assert g["sx"] == pytest.approx(float(dx), rel=1e-7)
    px = 36.0 / 1920
    ds = _po2_floor(px / (float(dx) * 3), 1024 // 8)
    assert g["ds"] == ds and g["M"] == 1024 // ds
    assert g["rx"] == int(np.ceil(0.5 * g["M"] * g["sx_ds"] / g["px_mm_x"])) + 1
    assert g["gain"] == pytest.approx(2.8 * 2.8 * 0.9 / 4.0, rel=1e-6)


def test_mdft_engine_kept_when_small_forced_sprite_when_prominent():
    assert sprite_geometry(_cal(), _cfg(engine=StarburstEngine.MDFT), SRC, 1920, 1080, 18.0, 12.0)["engine"] == "mdft"
    g = sprite_geometry(_cal(), _cfg(trim=30.0, engine=StarburstEngine.MDFT), SRC, 1920, 1080, 18.0, 12.0)
    assert g["engine"] == "sprite"


def test_grid_grows_to_cover_the_frame():
    """A prominent pattern (N dx / frame >= 0.2) that does not span the frame
    grows to the smallest power of two covering the farthest edge."""
    g = sprite_geometry(_cal(), _cfg(trim=30.0), SRC, 1920, 1080, 18.0, 12.0)
    dx0 = 30.0 * 550e-6 * 2.0 * 0.3
    cov = 2 * 960 * (36.0 / 1920) / dx0
    want = 256
    while want < min(np.ceil(cov), 8192):
        want *= 2
    assert g["N"] == max(1024, want) and g["N"] > 1024


def test_oversized_sensor_grows_grid():
    cal = _cal(image_circle_semi_w=10.0, image_circle_semi_h=8.0)
    g = sprite_geometry(cal, _cfg(), SRC, 1920, 1080, 18.0, 12.0)
    assert g["N"] > 1024


def test_degenerate_optics_rejected():
    with pytest.raises(ValueError, match="degenerate"):
        sprite_geometry(_cal(focal_length_x=0.0, max_half_angle_h=0.0), _cfg(), SRC, 1920, 1080, 18.0, 12.0)
    with pytest.raises(ValueError, match="power of two"):
        sprite_geometry(_cal(), _cfg(grid=1000), SRC, 1920, 1080, 18.0, 12.0)


def test_spectrum_white_balanced():
    spec = starburst_spectrum(_cfg())
    np.testing.assert_allclose(spec[:, 1:4].astype(np.float64).sum(0), 1.0, rtol=1e-6)


def test_oracle_energy():
    """The restatement's sprite carries about the PSF's unit energy per
    channel (the bilinear rescale by lambda_ref / lambda is exact only in
    the continuum: a few percent at this small grid) and its splat keeps the
    sprite's energy for a source far from the frame edges."""
    N = 256
    yy, xx = np.mgrid[:N, :N] - N / 2
    pupil = ((xx ** 2 + yy ** 2) < (0.3 * N / 2) ** 2).astype(np.float64)
    spec = starburst_spectrum(_cfg())
    spr = SO.sprite(pupil, spec, 2)
    tot = spr.reshape(-1, 3).sum(0)
    assert np.all(np.abs(tot - 1.0) < 0.08)
    img = SO.splat(spr, [[100.2, 90.7, 1.0, 1.0, 1.0]], 0.01, 0.01, 0.02, 0.02, 80, 80, 1.0, 200, 180)
    np.testing.assert_allclose(img.reshape(3, -1).sum(1), tot, rtol=1e-9)


@pytest.mark.parametrize("field_deg", [(15.0, 5.0), (-22.0, 0.0), (3.0, -18.0)])
def test_survivor_structure_matches_restatement(field_deg):
    """The product's vectorised cat's-eye centre and envelope against the
    oracle's loop-by-loop restatement of solve_survivor_center /
    build_survivor_envelope, both fed the oracle's float host trace: the
    same launches, boundary cells, supersamples and dilation give the same
    numbers bit for bit."""
    import math
    from ghostlight_gb300 import prescriptions as P
    from ghostlight_gb300.optics import OpticalSystem
    from ghostlight_gb300.starburst import survivor_center, survivor_envelope
    lens = OpticalSystem.from_records(P.double_gauss_12(seed=1))
    surfs = lens.records()
    ax, ay = (math.radians(a) for a in field_deg)

    def host_survives(x, y, z, d):
        return SO._survive(surfs, np.stack([x, y], 1), z, d)

    got = survivor_center(lens, ax, ay, survives=host_survives)
    want = SO.survivor_center(surfs, ax, ay)
    assert got[2] == want[2]
    assert np.float32(got[0]) == np.float32(want[0]) and np.float32(got[1]) == np.float32(want[1])
    if not want[2]:
        return
    cal = lens.calibration()
    ep_x, ep_y = cal.entrance_pupil_semi_x, cal.entrance_pupil_semi_y
    env = survivor_envelope(lens, ep_x, ep_y, got[0], got[1], ax, ay, 40, survives=host_survives)
    ref = SO.survivor_envelope(surfs, ep_x, ep_y, want[0], want[1], ax, ay, 40)
    np.testing.assert_array_equal(env, ref)
    assert 0.0 < env.mean() < 1.0 and ((env > 0) & (env < 1)).any()

"""The SPRITE starburst engine on the GPU against its FP64 restatement
(oracle/sprite_oracle.py, render_starburst's sprite path): the PSF, the
wavelength-baked and box-summed sprite, the area-weighted splat, and the
layer through render_point_flare."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import sprite_oracle as SO

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _lens():
    from ghostlight_gb300 import prescriptions as P
    from ghostlight_gb300.optics import OpticalSystem
    lens = OpticalSystem.from_records(P.double_gauss_12(seed=1))
    for s in lens.surfaces:
        if s.is_stop:
            s.aperture_shape, s.aperture_blades = 1, 9
            s.aperture_rotation_rad = 0.2
            s.aperture_curvature = 0.3
    return lens


def _config(ns=16):
    import ghostlight_gb300 as gl
    cfg = gl.PointFlareConfig(ray_grid=32, spectral_samples=ns)
    cfg.diffraction.starburst = True
    return cfg


@pytest.mark.parametrize("N,ds", [(512, 1), (512, 4), (1024, 2)])
def test_sprite_matches_oracle(N, ds):
    from ghostlight_gb300.starburst import SpritePlan, build_pupil, starburst_spectrum
    spec = starburst_spectrum(_config())
    pupil = build_pupil(_lens(), N, 0.3)
    plan = SpritePlan(N, spec)
    plan.bake(pupil, ds)
    psf, spr, energy = plan.read()
    torch.cuda.synchronize()
    plan.close()
    p_ref = SO.psf(pupil.cpu().numpy())
    assert energy == pytest.approx(p_ref.sum(), rel=1e-5)
    assert rel_l2(psf.cpu().numpy(), p_ref) < 1e-5
    s_ref = SO.sprite(pupil.cpu().numpy(), spec, ds)
    got = spr.cpu().numpy()
    assert got.shape == (N // ds, N // ds, 3)
    assert rel_l2(got, s_ref) < 1e-4
    # white in, white out: each channel of the sprite carries about unit
    # energy (the bilinear wavelength rescale is exact only in the continuum)
    tot = got.reshape(-1, 3).sum(0)
    assert np.all(np.abs(tot - 1.0) < 0.08)


@pytest.mark.parametrize("N", [4096, 8192])
def test_large_grids_psf(N):
    """The 2- and 1-column FFT groups of the large grids: the PSF is the
    pupil's |FFT|^2 (checked against numpy at 4096), its energy the pupil's
    by Parseval, and centro-symmetric for the real pupil."""
    from ghostlight_gb300.starburst import SpritePlan, build_pupil, starburst_spectrum
    spec = starburst_spectrum(_config(8))
    pupil = build_pupil(_lens(), N, 0.3)
    plan = SpritePlan(N, spec)
    plan.bake(pupil, 8)
    psf, spr, energy = plan.read()
    torch.cuda.synchronize()
    plan.close()
    a2 = float((pupil.double() ** 2).sum())
    assert energy == pytest.approx(N * N * a2, rel=1e-4)
    p = psf.cpu().numpy()
    c = N // 2
    assert p[c, c] == p.max()
    np.testing.assert_allclose(p[1:, 1:], p[1:, 1:][::-1, ::-1], rtol=2e-3, atol=p.max() * 1e-5)
    if N == 4096:
        assert rel_l2(p, SO.psf(pupil.cpu().numpy())) < 1e-5
    assert np.isfinite(spr.cpu().numpy()).all()


def test_splat_matches_oracle():
    from ghostlight_gb300.starburst import SpritePlan, build_pupil, starburst_spectrum
    N, ds, W, H = 512, 2, 300, 220
    spec = starburst_spectrum(_config())
    pupil = build_pupil(_lens(), N, 0.3)
    plan = SpritePlan(N, spec)
    plan.bake(pupil, ds)
    _, spr, _ = plan.read()
    src = np.array([[150.3, 100.7, 1.0, 0.8, 0.6], [12.5, 210.2, 0.5, 1.0, 1.0], [299.9, 3.1, 2.0, 2.0, 2.0]],
                   np.float32)
    args = (0.011, 0.012, 0.02, 0.02, 140, 140, 1.7)
    out = [torch.zeros((H, W), dtype=torch.float32, device="cuda") for _ in range(3)]
    plan.splat(src, *args, *out)
    torch.cuda.synchronize()
    plan.close()
    got = np.stack([o.cpu().numpy() for o in out])
    want = SO.splat(spr.cpu().numpy().astype(np.float64), src, *args, W, H)
    assert want.sum() > 0
    assert rel_l2(got, want) < 1e-5


def test_stateless_splat_matches_plan_splat():
    """gl_sprite_splat_source (one source by value, the caller's copy of the
    sprite, no staging) adds what the plan's splat adds, source by source,
    on and off the frame, into planes that already hold an image."""
    import ctypes as C
    from ghostlight_gb300 import _native
    from ghostlight_gb300.starburst import SpritePlan, build_pupil, starburst_spectrum
    N, ds, W, H = 512, 2, 300, 220
    plan = SpritePlan(N, starburst_spectrum(_config()))
    plan.bake(build_pupil(_lens(), N, 0.3), ds)
    _, spr, _ = plan.read()
    M = spr.shape[0]
    args = (0.011, 0.012, 0.02, 0.02, 140, 140, 1.7)
    lib = _native.load()
    base = torch.rand((3, H, W), device="cuda")
    for src in ([150.3, 100.7, 1.0, 0.8, 0.6], [-40.0, 210.2, 0.5, 1.0, 1.0], [299.9, 3.1, 2.0, 2.0, 2.0]):
        a = base.clone()
        b = base.clone()
        plan.splat(np.array([src], np.float32), *args, a[0], a[1], a[2])
        _native.check(lib.gl_sprite_splat_source(C.c_void_p(spr.data_ptr()), M, *[float(v) for v in src],
                                                 *[float(v) for v in args[:4]], args[4], args[5], float(args[6]),
                                                 C.c_void_p(b[0].data_ptr()), C.c_void_p(b[1].data_ptr()),
                                                 C.c_void_p(b[2].data_ptr()), W, H,
                                                 C.c_void_p(torch.cuda.current_stream().cuda_stream)), "splat")
        torch.cuda.synchronize()
        assert (a - base).abs().sum() > 0
        torch.testing.assert_close(b, a, rtol=0, atol=0)
    plan.close()


def test_layer_through_point_flare():
    """render_point_flare's starburst by the default SPRITE engine: against
    the oracle pipeline on the same geometry; the brightest pixel is the
    source's image point and the layer carries gain x colour of energy."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300.starburst import build_pupil, sprite_geometry, starburst_spectrum
    lens = _lens()
    cal = lens.calibration()
    cfg = _config(12)
    cfg.source_x, cfg.source_y = 0.55, 0.45
    cfg.diffraction.scale_trim = 5.0
    W, H = 320, 240
    out = gl.render_point_flare(W, H, lens, cal, cfg)
    got = np.stack([out["starburst_%s" % c].cpu().numpy() for c in "rgb"])
    assert got.shape == (3, H, W) and got.max() > 0
    y, x = np.unravel_index(np.argmax(got[1]), got[1].shape)
    assert abs(x - 0.55 * W) <= 2 and abs(y - 0.45 * H) <= 2
    # the same layer from the oracle, on the geometry the render used
    hw, hh = cal.sensor_half_w, cal.sensor_half_h
    pos = np.array([[x + 0.5, y + 0.5, 1, 1, 1]], np.float32)
    geo = sprite_geometry(cal, cfg, pos, W, H, hw, hh, front_R=lens.surfaces[0].semi_aperture)
    assert geo["engine"] == "sprite"
    spec = starburst_spectrum(cfg)
    pupil = build_pupil(lens, geo["N"], geo["fill"]).cpu().numpy()
    spr = SO.sprite(pupil, spec, geo["ds"])
    # total energy: the sprite's per-channel sum x gain x the source colour,
    # less what falls off the frame
    from ghostlight_gb300.flare import source_rgb
    rgb = source_rgb(cfg, cfg.source_r, cfg.source_g, cfg.source_b)
    for c in range(3):
        full = spr[..., c].sum() * geo["gain"] * float(rgb[c])
        assert 0.5 * full < got[c].sum() <= full * 1.001, c


def test_mdft_engine_still_selectable():
    import ghostlight_gb300 as gl
    from ghostlight_gb300.config import StarburstEngine
    lens = _lens()
    cal = lens.calibration()
    cfg = _config(8)
    cfg.source_x, cfg.source_y = 0.5, 0.5
    cfg.diffraction.starburst_engine = StarburstEngine.MDFT
    out = gl.render_point_flare(256, 192, lens, cal, cfg)
    g = out["starburst_g"].cpu().numpy()
    y, x = np.unravel_index(np.argmax(g), g.shape)
    assert abs(x - 128) <= 2 and abs(y - 96) <= 2


@pytest.mark.parametrize("field_deg", [(15.0, 5.0), (-12.0, 3.0), (-22.0, 0.0)])
def test_cats_eye_device_matches_oracle(field_deg):
    """The cat's-eye centre and envelope from device traces against the
    oracle's float host traces: launches that straddle an aperture edge
    within rounding may land on either side, so the envelopes agree up to a
    few rim cells and the centres to a small fraction of the pupil."""
    import math
    from ghostlight_gb300.starburst import survivor_center, survivor_envelope
    lens = _lens()
    surfs = lens.records()
    ax, ay = (math.radians(a) for a in field_deg)
    got = survivor_center(lens, ax, ay)
    want = SO.survivor_center(surfs, ax, ay)
    assert got[2] == want[2]
    if not want[2]:         # past this lens's vignette edge
        return
    ep = lens.calibration().entrance_pupil_semi_x
    assert abs(got[0] - want[0]) < 1e-3 * ep and abs(got[1] - want[1]) < 1e-3 * ep
    env = survivor_envelope(lens, ep, ep, want[0], want[1], ax, ay, 64)
    ref = SO.survivor_envelope(surfs, ep, ep, want[0], want[1], ax, ay, 64)
    assert np.abs(env - ref).mean() < 2e-3 and (env != ref).mean() < 0.01
    assert 0.0 < ref.mean() < 1.0


def test_off_axis_sprite_uses_the_cats_eye():
    """Off axis the sprite's pupil is the stop weighted by the envelope: it
    never exceeds the plain stop, its throughput T < 1 scales the gain, and
    switching use_survivor_mask off restores the plain stop."""
    import math
    from ghostlight_gb300.starburst import build_pupil2, effective_pupil, sprite_geometry
    lens = _lens()
    cal = lens.calibration()
    cfg = _config(8)
    g = sprite_geometry(cal, cfg, np.array([[100, 100, 1, 1, 1]], np.float32), 320, 240, cal.sensor_half_w,
                        cal.sensor_half_h, front_R=lens.surfaces[0].semi_aperture)
    field = (math.radians(18.0), math.radians(4.0))
    pupil, T = effective_pupil(lens, cfg, g, field)
    plain = build_pupil2(lens, g["N"], g["fill"])
    assert pupil is not None and 0.01 < T < 0.999
    p, q = pupil.cpu().numpy(), plain.cpu().numpy()
    assert np.all(p <= q + 1e-6)
    assert float((pupil.double() ** 2).sum() / (plain.double() ** 2).sum()) == pytest.approx(T, rel=1e-9)
    cfg.diffraction.use_survivor_mask = False
    p2, T2 = effective_pupil(lens, cfg, g, field)
    assert T2 == 1.0 and torch.equal(p2, plain)
    # far past the vignette edge nothing survives: no starburst
    cfg.diffraction.use_survivor_mask = True
    assert effective_pupil(lens, cfg, g, (math.radians(80.0), 0.0))[0] is None


def test_resident_sprite_is_reused():
    """A second render of the same lens, grid and spectrum splats the
    resident sprite without baking again, with the same image; another field
    off axis (cat's-eye) bakes anew."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300 import starburst as SB
    lens = _lens()
    cal = lens.calibration()
    cfg = _config(8)
    cfg.diffraction.scale_trim = 5.0
    cfg.diffraction.use_survivor_mask = False
    a = gl.render_point_flare(200, 150, lens, cal, cfg)["starburst_g"].cpu().numpy()
    bakes = [v[1].get("bakes", 0) for v in SB._SPRITE_PLANS.values()]
    b = gl.render_point_flare(200, 150, lens, cal, cfg)["starburst_g"].cpu().numpy()
    assert [v[1].get("bakes", 0) for v in SB._SPRITE_PLANS.values()] == bakes
    np.testing.assert_array_equal(a, b)
    cfg.diffraction.use_survivor_mask = True
    cfg.source_x = 0.8
    gl.render_point_flare(200, 150, lens, cal, cfg)
    assert sum(v[1].get("bakes", 0) for v in SB._SPRITE_PLANS.values()) > sum(bakes)

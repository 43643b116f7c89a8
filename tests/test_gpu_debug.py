"""The validation captures _render_starburst_debug / _render_veil_debug
(bind_renderers.cpp:194-286) on the double Gauss 58 mm f/2.

The starburst cases restate the reference's own engine tests, which run
through the same debug entry (bindings/python/tests/test_starburst.py:44-200):
flux parity of the two engines, spectral-sample invariance, the sub-pixel
stability of the matrix-DFT window against a supersampled truth built from the
captured pupil, source tracking, the off-frame reach, determinism.  Each
capture's layer must also equal the frame render's layer for the same config,
and its intermediates must hold their definitions (unit-sum PSF and GSF centred
on the grid, the sprite's scale, the reference's scalars)."""
import json

import numpy as np
import pytest

from conftest import GOLDEN

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_META = json.loads((GOLDEN / "ref_goldens.json").read_text())


@pytest.fixture(scope="module")
def psf_lens():
    import ghostlight_gb300 as gl
    from ghostlight_gb300._abi import gl_surface
    raw = np.load(GOLDEN / "ref_goldens.npz")["lens/double_gauss"]
    recs = list((gl_surface * raw.shape[0]).from_buffer_copy(raw.tobytes()))
    return gl.OpticalSystem.from_records(recs, name="double_gauss",
                                         focal_length=_META["lenses"]["double_gauss"]["focal_length"])


def _cfg(engine, sx=0.5, sy=0.5, ns=6, grid=1024, trim=8.0, blades=0):
    import ghostlight_gb300 as gl
    c = gl.PointFlareConfig()
    c.source_x, c.source_y = sx, sy
    c.source_r = c.source_g = c.source_b = 1.0
    c.spectral_samples = ns
    c.aperture_blades = blades
    c.diffraction.starburst = True
    c.diffraction.starburst_engine = gl.StarburstEngine(engine)
    c.diffraction.starburst_grid = grid
    c.diffraction.pupil_fill = 0.30
    c.diffraction.scale_trim = trim
    c.diffraction.spectral_samples = ns
    return c


SPRITE, MDFT = 0, 1


def _lum(d):
    return (np.asarray(d["starburst_r"]) + np.asarray(d["starburst_g"]) + np.asarray(d["starburst_b"])).astype(np.float64)


def _render(lens, engine, w=192, **kw):
    import ghostlight_gb300 as gl
    return gl._render_starburst_debug(w, w, lens, lens.calibration(), _cfg(engine, **kw))


def test_mdft_renders_finite_nonzero(psf_lens):
    lum = _lum(_render(psf_lens, MDFT))
    assert np.isfinite(lum).all() and lum.sum() > 0.0 and (lum < 0.0).sum() == 0


def test_mdft_flux_matches_sprite(psf_lens):
    sp = _lum(_render(psf_lens, SPRITE)).sum()
    md = _lum(_render(psf_lens, MDFT)).sum()
    assert abs(md / sp - 1.0) < 0.06


def test_mdft_flux_is_spectral_sample_invariant(psf_lens):
    sums = [_lum(_render(psf_lens, MDFT, ns=n)).sum() for n in (3, 6, 12)]
    assert max(sums) / min(sums) < 1.005


def test_mdft_error_is_stable_sprite_flickers(psf_lens):
    """Against a supersampled truth from the captured pupil, the matrix-DFT
    window's shape error stays flat as the source scrubs sub-pixel; the
    sprite's swings."""
    import ghostlight_gb300 as gl
    cal = psf_lens.calibration()
    w = 256
    px = 2.0 * float(cal.sensor_half_w) / w

    def err_vs_truth(engine, sx):
        d = gl._render_starburst_debug(w, w, psf_lens, cal, _cfg(engine, sx=sx, sy=0.5, ns=6))
        A = np.asarray(d["pupil"], np.float64)
        N = int(d["grid"])
        dx = float(d["dx_mm_x"])
        P2 = np.zeros((2 * N, 2 * N), np.complex64)
        P2[N // 2:N // 2 + N, N // 2:N // 2 + N] = A
        I2 = (np.abs(np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(P2)))) ** 2).astype(np.float64)
        I2 /= I2.sum()
        dx2, N2 = dx / 2.0, 2 * N
        spx, spy = float(d["source_px"]), float(d["source_py"])
        K = 40
        kx0, ky0 = int(np.floor(spx)) - K // 2, int(np.floor(spy)) - K // 2

        def ov(k0, pos, n, tex):
            lo = ((k0 + np.arange(K) - pos) * px) / tex + 0.5 * n
            hi = lo + px / tex
            ii = np.arange(n)
            return np.clip(np.minimum(hi[:, None], ii[None, :] + 1) - np.maximum(lo[:, None], ii[None, :]), 0.0, None)

        truth = ov(ky0, spy, N2, dx2) @ I2 @ ov(kx0, spx, N2, dx2).T
        win = _lum(d)[ky0:ky0 + K, kx0:kx0 + K]
        a = win / max(win.sum(), 1e-30)
        b = truth / max(truth.sum(), 1e-30)
        return float(np.abs(a - b).sum() / 2)

    xs = [0.820 + i * 0.0015 for i in range(12)]
    md = np.array([err_vs_truth(MDFT, x) for x in xs])
    sp = np.array([err_vs_truth(SPRITE, x) for x in xs])
    assert md.std() < sp.std() * 0.35, (md.std(), sp.std())
    assert md.max() < sp.max() and md.mean() < 0.10, (md, sp)


def test_mdft_source_position_tracks(psf_lens):
    w = 192
    ys, xs = np.mgrid[0:w, 0:w]

    def centroid(sx):
        lum = _lum(_render(psf_lens, MDFT, w=w, sx=sx))
        return float((xs * lum).sum() / lum.sum())

    assert centroid(0.60) > centroid(0.40) + 10


def test_offframe_reach_matches_sprite(psf_lens):
    near_sp = _lum(_render(psf_lens, SPRITE, sx=0.98)).sum()
    near_md = _lum(_render(psf_lens, MDFT, sx=0.98)).sum()
    assert near_md > 0 and near_sp > 0 and abs(near_md / near_sp - 1.0) < 0.08
    assert _lum(_render(psf_lens, SPRITE, sx=1.15)).sum() == 0.0
    assert _lum(_render(psf_lens, MDFT, sx=1.15)).sum() == 0.0


def test_sprite_engine_deterministic(psf_lens):
    assert np.array_equal(_lum(_render(psf_lens, SPRITE)), _lum(_render(psf_lens, SPRITE)))


def test_six_blade_mdft_finite(psf_lens):
    lum = _lum(_render(psf_lens, MDFT, blades=6))
    assert np.isfinite(lum).all() and lum.sum() > 0


@pytest.mark.parametrize("engine,sx", [(SPRITE, 0.5), (SPRITE, 0.8), (MDFT, 0.5)])
def test_starburst_capture_matches_frame_render(psf_lens, engine, sx):
    """The captured layer is the frame render's starburst layer; the PSF is
    unit-sum and DC-centred; the sprite carries the baked spectrum; the scalars
    are the lens's first-order optics."""
    import ghostlight_gb300 as gl
    cal = psf_lens.calibration()
    cfg = _cfg(engine, sx=sx)
    d = gl._render_starburst_debug(192, 192, psf_lens, cal, cfg)
    out = gl.render_point_flare(192, 192, psf_lens, cal, cfg)
    for c in "rgb":
        want = out["starburst_" + c].cpu().numpy()
        if engine == SPRITE:
            np.testing.assert_array_equal(d["starburst_" + c], want)
        else:
            # the window accumulates wavelengths with float atomics: order noise
            np.testing.assert_allclose(d["starburst_" + c], want, rtol=1e-5, atol=1e-6 * float(want.max()))
    N = d["grid"]
    assert N >= 1024 and d["pupil"].shape == (N, N) and d["psf"].shape == (N, N)
    assert d["sprite_rgb"].shape == (N, N, 3)
    assert 0.0 <= d["pupil"].min() and d["pupil"].max() <= 1.0 + 1e-6
    assert d["lambda_ref_nm"] == 550.0
    assert d["f_number_x"] == pytest.approx(cal.f_number_x, rel=1e-5)
    assert d["focal_length_x"] == pytest.approx(cal.focal_length_x, rel=1e-6)
    assert d["entrance_pupil_semi_x"] == pytest.approx(cal.entrance_pupil_semi_x, rel=1e-6)
    f = np.float32
    dx = f(f(f(f(550.0) * f(1e-6)) * f(d["f_number_x"])) * f(0.30)) * f(8.0)
    assert d["dx_mm_x"] == pytest.approx(float(dx), rel=1e-6)
    if engine == MDFT:
        assert not d["psf"].any() and not d["sprite_rgb"].any()
        return
    assert float(d["psf"].sum(dtype=np.float64)) == pytest.approx(1.0, abs=1e-4)
    assert np.unravel_index(np.argmax(d["psf"]), d["psf"].shape) == (N // 2, N // 2)
    # each wavelength's scaled copy of the unit-sum PSF keeps (nearly) unit sum,
    # so a channel sums to its colour-matching weights over the spectrum (the
    # weights go negative in places, so can single texels)
    from ghostlight_gb300.starburst import starburst_spectrum
    spec = starburst_spectrum(cfg)
    sums = d["sprite_rgb"].sum(axis=(0, 1), dtype=np.float64)
    expect = spec[:, 1:4].astype(np.float64).sum(0)
    np.testing.assert_allclose(sums, expect, rtol=0.05, atol=0.02 * float(np.abs(expect).max()))
    if sx == 0.5:
        assert d["throughput"] == 1.0 and d["chief_offset_x"] == 0.0
    else:
        assert 0.0 < d["throughput"] <= 1.0 and d["field_angle_x"] > 0.0


def test_starburst_capture_off_is_empty(psf_lens):
    import ghostlight_gb300 as gl
    cfg = _cfg(SPRITE)
    cfg.diffraction.starburst = False
    d = gl._render_starburst_debug(64, 48, psf_lens, psf_lens.calibration(), cfg)
    assert d["grid"] == 0 and d["psf"].shape == (0, 0) and d["starburst_r"].shape == (48, 64)
    assert not d["starburst_r"].any()


@pytest.mark.parametrize("falloff,spread", [(1.5, 0.12), (0.5, 0.3), (4.0, 0.05)])
def test_veil_capture(psf_lens, falloff, spread):
    """The veil capture: its layer is the frame render's veil layer, the GSF is
    unit-sum, centred and radially decreasing, the sprite is the neutral
    replica, the scale follows spread x sensor half-height over N / 32 texels
    and the falloff is clamped to [1, 3]."""
    import ghostlight_gb300 as gl
    cal = psf_lens.calibration()
    cfg = gl.PointFlareConfig(source_x=0.3, source_y=0.6, source_r=2.0, source_g=1.0, source_b=0.5)
    cfg.diffraction.veil = True
    cfg.diffraction.veil_falloff = falloff
    cfg.diffraction.veil_spread = spread
    d = gl._render_veil_debug(160, 120, psf_lens, cal, cfg)
    out = gl.render_point_flare(160, 120, psf_lens, cal, cfg)
    for c in "rgb":
        np.testing.assert_array_equal(d["veil_" + c], out["veil_" + c].cpu().numpy())
    N = d["grid"]
    ref = d["reference"]
    assert N == 1024 and ref.shape == (N, N) and d["sprite_rgb"].shape == (N, N, 3)
    assert float(ref.sum(dtype=np.float64)) == pytest.approx(1.0, abs=1e-5)
    assert np.unravel_index(np.argmax(ref), ref.shape) == (N // 2, N // 2)
    assert ref[N // 2, N // 2 + 10] < ref[N // 2, N // 2 + 1]
    np.testing.assert_array_equal(d["sprite_rgb"][..., 1], ref)
    assert d["falloff"] == min(max(falloff, 1.0), 3.0)
    assert d["core_texels"] == N / 32
    f = np.float32
    assert d["core_mm"] == pytest.approx(float(f(spread) * f(cal.sensor_half_h)), rel=1e-6)
    assert d["dx_mm_x"] == pytest.approx(d["core_mm"] / d["core_texels"], rel=1e-6)
    assert 0.0 <= d["source_px"] <= 160 and 0.0 <= d["source_py"] <= 120


def test_veil_capture_off_has_no_sprite(psf_lens):
    import ghostlight_gb300 as gl
    d = gl._render_veil_debug(32, 32, psf_lens, psf_lens.calibration(), gl.PointFlareConfig())
    assert d["grid"] == 0 and "reference" not in d and not d["veil_r"].any()

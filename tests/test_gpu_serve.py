"""Serving path on the GPU: a request equals the plan render of the same
inputs, the two work modes agree, and every result is the same alone and in
a concurrent mix."""
import math

import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pool():
    import ghostlight_gb300 as gl
    from ghostlight_gb300.serve import serving_lens_pool
    cfg = gl.FlareConfig(min_ghost_intensity=1e-6)
    p = serving_lens_pool(3, cfg, seed=200, n_min=8, n_max=16)
    yield p, cfg
    for rl in p.values():
        rl.close()


def _run_server(pool, reqs, **kw):
    from ghostlight_gb300.serve import FlareServer
    results = {}
    engine = kw.pop("starburst_engine", "sprite")
    srv = FlareServer(pool, max_inflight=kw.pop("max_inflight", 8), **kw)
    srv.exec.starburst_engine = engine
    srv.on_result = lambda r, out: results.__setitem__(r.rid, out.clone())
    srv.run_trace(reqs)
    torch.cuda.synchronize()
    return results


def _reqs():
    from ghostlight_gb300.serve import FlareRequest
    shapes = [(256, 256, 8, 48, 3.0), (512, 512, 16, 64, 12.0), (384, 256, 8, 96, 18.0),
              (512, 512, 31, 48, 7.0), (256, 256, 16, 80, 0.0), (512, 384, 8, 64, 15.0)]
    out = []
    for i, (w, h, ns, g, f) in enumerate(shapes):
        out.append(FlareRequest(lens_id=i % 3, width=w, height=h, n_spec=ns, ray_grid=g, field_deg=f, rid=i))
    return out


def test_request_matches_plan_render(pool):
    from ghostlight_gb300.flare import GhostRenderPlan, pupil_grid
    from ghostlight_gb300.serve import _spectral
    p, cfg = pool
    for req in _reqs()[:3]:
        rl = p[req.lens_id]
        got = _run_server(p, [req])[req.rid]
        spec, corr = _spectral(req.n_spec, cfg)
        grid = pupil_grid(rl.lens, req.ray_grid, 0, 0, 0, 0.0)
        src = np.array([[math.radians(req.field_deg), 0.0, 1.0, 1.0, 1.0]], np.float32)
        plan = GhostRenderPlan(rl.lens, rl.pairs, rl.boosts, src, [grid], np.zeros(len(rl.pairs), np.int32), spec,
                               corr, req.width, req.height, rl.sensor_half_w, rl.sensor_half_h, req.gain,
                               apply_correction=True, cull_dead_pairs=True)
        outs = [torch.zeros((req.height, req.width), device="cuda") for _ in range(3)]
        plan.execute(*outs)
        torch.cuda.synchronize()
        want = torch.stack(outs).cpu().numpy()
        plan.close()
        assert np.abs(want).sum() > 0
        assert rel_l2(got.numpy(), want) < 1e-5


@pytest.mark.parametrize("ipw", [0, 2])
def test_work_modes_agree(pool, ipw):
    p, _ = pool
    reqs = _reqs()[3:5]
    a = _run_server(p, [r for r in reqs], items_per_warp=8)
    for r in reqs:
        r.start = r.finish = 0.0
    b = _run_server(p, reqs, items_per_warp=ipw)
    for r in reqs:
        assert rel_l2(b[r.rid].numpy(), a[r.rid].numpy()) < 1e-5


def test_wavelength_split_agrees(pool):
    """A request split into wavelength ranges (the default: 31 -> 4, 16 -> 2)
    renders the image of the unsplit request."""
    p, _ = pool
    reqs = _reqs()[1:4]
    a = _run_server(p, reqs, lambda_chunks=1)
    for r in reqs:
        r.start = r.finish = 0.0
    b = _run_server(p, reqs)
    for r in reqs:
        r.start = r.finish = 0.0
    c = _run_server(p, reqs, lambda_chunks=3)
    for r in reqs:
        assert rel_l2(b[r.rid].numpy(), a[r.rid].numpy()) < 1e-5
        assert rel_l2(c[r.rid].numpy(), a[r.rid].numpy()) < 1e-5


@pytest.mark.parametrize("engine", ["sprite", "mdft"])
def test_request_starburst_layer(pool, engine):
    """A request with the starburst layer = its ghost layer + the lens's
    starburst at the source's image point: with the SPRITE engine the frame
    render's sprite layer of the same geometry (plain stop, T = 1), with the
    matrix-DFT engine the resident plan's pattern of the lens's stop pupil."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300.serve import STARBURST_PUPIL, SpriteStarbursts, _spectral
    from ghostlight_gb300.starburst import sprite_starburst_layer
    p, cfg = pool
    base = _reqs()[3]                                  # 512^2, 31 wavelengths
    ghost = _run_server(p, [base])[base.rid].numpy()
    base.start = base.finish = 0.0
    base.starburst = True
    both = _run_server(p, [base], starburst_engine=engine)[base.rid].numpy()
    rl = p[base.lens_id]
    cx, cy = rl.image_point(base.field_deg, base.width, base.height)
    if engine == "sprite":
        scfg = SpriteStarbursts.config_for(rl, base.n_spec)
        _, _, g = SpriteStarbursts()._bake(rl, base.width, base.height, base.n_spec)
        layer = sprite_starburst_layer(rl.lens, rl.calibration, scfg, np.array([[cx, cy, 1.0, 1.0, 1.0]], np.float32),
                                       base.width, base.height, rl.sensor_half_w, rl.sensor_half_h, geometry=g)
        want = np.stack([layer["starburst_" + c].cpu().numpy() for c in "rgb"])
    else:
        spec, _ = _spectral(base.n_spec, cfg)
        lam = spec[:, 0].astype(np.float64)
        sc = lam.min() / lam
        plan = gl.MdftPlan(STARBURST_PUPIL, (base.width, base.height), sc / base.width, sc / base.height,
                           spec[:, 1:4], "split_bf16", center_x=cx, center_y=cy)
        out = [torch.zeros((base.height, base.width), device="cuda") for _ in range(3)]
        plan.execute(rl.starburst_pupil(), *out)
        torch.cuda.synchronize()
        want = torch.stack(out).cpu().numpy()
        plan.close()
    assert want.max() > 0.0
    assert rel_l2(both - ghost, want) < 1e-4


def test_alone_and_in_the_mix_agree(pool):
    p, _ = pool
    reqs = _reqs()
    for r in reqs[::2]:
        r.starburst = True
    alone = {}
    for r in reqs:
        alone.update(_run_server(p, [r]))
    for r in reqs:
        r.arrival = 0.0
    mix = _run_server(p, reqs, max_inflight=6)
    assert set(mix) == set(alone)
    for r in reqs:
        a, m = alone[r.rid].numpy(), mix[r.rid].numpy()
        assert np.isfinite(m).all()
        assert rel_l2(m, a) < 1e-5, r


def test_served_lens_with_tables_and_bitmaps():
    """A resident lens with table coatings and bitmap apertures serves the
    same image as the plan render of the same pairs (the tables and bitmaps
    resolve to device-resident store entries in both)."""
    import warnings
    import ghostlight_gb300 as gl
    from ghostlight_gb300 import load_lens
    from ghostlight_gb300.flare import GhostRenderPlan, pupil_grid
    from ghostlight_gb300.serve import FlareRequest, ResidentLens, _spectral
    from test_coatings import LENS as COATED
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lens = load_lens(COATED)
    lens.set_aperture_image(0, np.where(np.hypot(*np.mgrid[-1:1:64j, -1:1:64j]) < 0.9, 1.0, 0.0),
                            lens.surfaces[0].semi_aperture * 1.05)
    cal = lens.calibration()
    cfg = gl.FlareConfig(min_ghost_intensity=1e-6)
    rl = ResidentLens(lens, cal.sensor_half_w, cal.sensor_half_h, cfg)
    try:
        req = FlareRequest(lens_id=0, width=256, height=256, n_spec=16, ray_grid=48, field_deg=6.0, rid=0)
        got = _run_server({0: rl}, [req])[0].numpy()
        spec, corr = _spectral(16, cfg)
        grid = pupil_grid(lens, 48, 0, 0, 0, 0.0)
        src = np.array([[math.radians(6.0), 0.0, 1.0, 1.0, 1.0]], np.float32)
        plan = GhostRenderPlan(lens, rl.pairs, rl.boosts, src, [grid], np.zeros(len(rl.pairs), np.int32), spec,
                               corr, 256, 256, rl.sensor_half_w, rl.sensor_half_h, req.gain,
                               apply_correction=True, cull_dead_pairs=True)
        outs = [torch.zeros((256, 256), device="cuda") for _ in range(3)]
        plan.execute(*outs)
        torch.cuda.synchronize()
        want = torch.stack(outs).cpu().numpy()
        plan.close()
        assert np.abs(want).sum() > 0
        assert rel_l2(got, want) < 1e-5
    finally:
        rl.close()


def test_psf_request_matches_render_psf(pool):
    """A PSF request (render_psf, PSFRenderer.cpp:260, as a served request:
    the pre-pass on the host, the atlas stream-ordered on the request's own
    stream) equals render_psf of the same configuration, alone and in a mix
    with flare requests."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300.serve import CudaExecutor, FlareRequest
    p, _ = pool
    reqs = []
    for i, (g, ns, grid) in enumerate(((4, 8, 48), (8, 16, 32))):
        r = FlareRequest(lens_id=i % len(p), width=0, height=0, n_spec=ns, ray_grid=grid, field_deg=0.0,
                         rid=100 + i, kind="psf", psf_grid=g)
        r.width = r.height = g * r.psf_tile
        reqs.append(r)
    ex = CudaExecutor(p, 4)
    wants = {}
    for r in reqs:
        cfg, src = ex.psf_config(r, p[r.lens_id])
        out = gl.render_psf(src, p[r.lens_id].lens, cfg)
        torch.cuda.synchronize()
        wants[r.rid] = np.stack([out[c].cpu().numpy() for c in "rgb"])
        assert wants[r.rid].sum() > 0
    alone = {}
    for r in reqs:
        alone.update(_run_server(p, [r]))
    mix_reqs = _reqs()[:4] + reqs
    for r in mix_reqs:
        r.arrival, r.start, r.finish = 0.0, 0.0, 0.0
    mix = _run_server(p, mix_reqs, max_inflight=6)
    for r in reqs:
        assert alone[r.rid].shape == (3, r.height, r.width)
        assert rel_l2(alone[r.rid].numpy(), wants[r.rid]) < 1e-6
        assert rel_l2(mix[r.rid].numpy(), wants[r.rid]) < 1e-6
        assert r.traced > 0


def test_served_requests_match_fp64_oracle(pool):
    """Every flare request of a concurrent mix (three lenses, several sizes,
    wavelength counts, grids and fields, off-sensor cull on) against the FP64
    oracle's render of the same pairs, grid, source and spectrum, colour
    correction applied: relative L2 below 1e-3."""
    from oracle import oracle as O
    from ghostlight_gb300.flare import pupil_grid
    from ghostlight_gb300.serve import _spectral
    p, cfg = pool
    reqs = _reqs()
    got = _run_server(p, reqs)
    for req in reqs:
        rl = p[req.lens_id]
        spec, corr = _spectral(req.n_spec, cfg)
        grid = pupil_grid(rl.lens, req.ray_grid, 0, 0, 0, 0.0)
        src = np.array([[math.radians(req.field_deg), 0.0, 1.0, 1.0, 1.0]], np.float32)
        want = O.render(rl.lens.records(), rl.pairs, rl.boosts, src, [grid], spec, rl.sensor_half_w,
                        rl.sensor_half_h, req.width, req.height, req.gain, fp64=True)
        want = np.einsum("ij,jhw->ihw", corr.astype(np.float64), want)
        assert np.abs(want).sum() > 0
        assert rel_l2(got[req.rid].numpy(), want) < 1e-3, req

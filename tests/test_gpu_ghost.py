"""GPU parity of the flare path: device culler, device trace, batched
render, against the reference's recorded outputs and the FP64 oracle.

Tolerances (the flare path's parity bar): ghost set and pupil mask
bit-exact; FP32 images within 1e-3 relative L2 of the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import LENS_NAMES, lens_from_pins, rel_l2
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

IMG_TOL = 1e-3


def _lens(pins, name):
    from ghostlight_gb300.optics import OpticalSystem
    return OpticalSystem.from_records(lens_from_pins(pins, name))


@pytest.mark.parametrize("name", LENS_NAMES)
def test_device_trace_matches_reference_rays(pins, name):
    import ghostlight_gb300 as gl
    lens = _lens(pins, name)
    k = 0
    while "%s/rays_%d/ab" % (name, k) in pins:
        a, b = (int(x) for x in pins["%s/rays_%d/ab" % (name, k)])
        rays = torch.from_numpy(pins["%s/rays_%d/in" % (name, k)]).cuda()
        want = pins["%s/rays_%d/out" % (name, k)]
        got = gl.trace_rays(lens, rays, a, b).cpu().numpy()
        # every ray's status equals the reference's (none of these rays meets
        # a clear aperture within float rounding of its edge: their FP64
        # statuses do not change when every clear radius grows or shrinks by
        # 1e-5); landings within 5e-4 mm (measured at most 1.5e-4 mm, the
        # float32 rounding of a walk in another operation order)
        np.testing.assert_array_equal(got[:, 4], want[:, 4], err_msg="%s rays_%d status" % (name, k))
        ok = (got[:, 4] == 0) & (want[:, 4] == 0)
        if ok.any():
            d = np.abs(got[ok, :2].astype(np.float64) - want[ok, :2])
            assert np.median(d) < 1e-4 and d.max() < 5e-4, (name, k, np.median(d), d.max())
            rw = np.abs(got[ok, 3] - want[ok, 3]) / np.maximum(np.abs(want[ok, 3]), 1e-30)
            assert np.median(rw) < 1e-4
        k += 1


@pytest.mark.parametrize("name", LENS_NAMES)
@pytest.mark.parametrize("thr", ["1e-7", "1e-6", "1e-4", "0"])
def test_device_culler_ghost_set_bit_exact(pins, meta, name, thr):
    from ghostlight_gb300 import FlareConfig
    from ghostlight_gb300.flare import filter_ghosts_device
    lens = _lens(pins, name)
    cal = meta[name]["calibration"]
    cfg = FlareConfig(min_ghost_intensity=float(thr))
    r = filter_ghosts_device(lens, cal["sensor_half_w"], cal["sensor_half_h"], cfg)
    np.testing.assert_array_equal(r.pairs, pins["%s/filter_%s/pairs" % (name, thr)])
    want_b = pins["%s/filter_%s/boosts" % (name, thr)]
    np.testing.assert_allclose(r.boosts, want_b, rtol=1e-5)


def _plan_vs_oracle(lens, cal, pairs, boosts, grids, pair_grid, spec, W, H, src, gain=1000.0,
                    plain=False, correction=False):
    from ghostlight_gb300.flare import GhostRenderPlan, spectral_table
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    _, corr = spectral_table(len(spec))
    plan = GhostRenderPlan(lens, pairs, boosts, src, grids, pair_grid, spec, corr, W, H, hw, hh, gain,
                           apply_correction=correction, plain_per_pair=plain)
    out = [torch.zeros((H, W), dtype=torch.float32, device="cuda") for _ in range(3)]
    plan.execute(*out)
    torch.cuda.synchronize()
    got = np.stack([o.cpu().numpy() for o in out])
    want = O.render(lens.records(), pairs, boosts, src, grids, spec, hw, hh, W, H, gain,
                    pair_grid=pair_grid, fp64=True)
    if correction:
        want = np.einsum("ij,jhw->ihw", corr.astype(np.float64), want)
    plan.close()
    return got, want


def test_render_cfg1_matches_fp64_oracle(pins, meta, ref_images):
    """Configuration 1 (12-surface double Gauss, 30 non-crossing pairs, 8
    wavelengths, 10 deg source) at 128^2 pupil samples, 512^2 output."""
    lens = _lens(pins, "cfg1_double_gauss_12")
    cal = meta["cfg1_double_gauss_12"]["calibration"]
    pairs, boosts = ref_images["cfg1_small/pairs"], ref_images["cfg1_small/boosts"]
    spec = ref_images["cfg1_small/spec"]
    grid = O.aperture_samples(lens.records(), 128, 0)
    src = ref_images["cfg1_small/source"]
    got, want = _plan_vs_oracle(lens, cal, pairs, boosts, [grid], np.zeros(len(pairs), np.int32), spec,
                                512, 512, src)
    assert want.sum() > 0
    assert rel_l2(got, want) < IMG_TOL


def test_render_correction_and_plain_mode(pins, meta, ref_images):
    lens = _lens(pins, "cfg1_double_gauss_12")
    cal = meta["cfg1_double_gauss_12"]["calibration"]
    pairs, boosts = ref_images["cfg1_small/pairs"], ref_images["cfg1_small/boosts"]
    spec = ref_images["cfg1_small/spec"]
    grid = O.aperture_samples(lens.records(), 96, 1, 3)
    src = np.array([[0.12, -0.05, 1.0, 0.7, 0.4]], np.float32)
    got_c, want_c = _plan_vs_oracle(lens, cal, pairs, boosts, [grid], np.zeros(len(pairs), np.int32), spec,
                                    301, 203, src, correction=True)
    assert rel_l2(got_c, want_c) < IMG_TOL
    got_p, want_p = _plan_vs_oracle(lens, cal, pairs, boosts, [grid], np.zeros(len(pairs), np.int32), spec,
                                    301, 203, src, correction=True, plain=True)
    assert rel_l2(got_p, got_c) < 1e-5


def test_render_adaptive_grids_cfg2_matches_oracle(pins, meta):
    """Configuration 2 lens (24 surfaces, two aspheres) with uneven per-pair
    pupil grids in one persistent launch."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300.flare import filter_ghosts_device, pupil_grid, spectral_table
    lens = _lens(pins, "cfg2_wide_angle_24")
    cal = meta["cfg2_wide_angle_24"]["calibration"]
    cfg = gl.FlareConfig(min_ghost_intensity=1e-6)
    fr = filter_ghosts_device(lens, cal["sensor_half_w"], cal["sensor_half_h"], cfg)
    pairs, boosts = fr.pairs[::5], fr.boosts[::5]
    sizes = [16, 32, 48, 64]
    grids = [pupil_grid(lens, g) for g in sizes]
    pair_grid = np.arange(len(pairs), dtype=np.int32) % len(sizes)
    spec, _ = spectral_table(31)
    src = np.array([[np.radians(15.0), 0.0, 1.0, 1.0, 1.0]], np.float32)
    got, want = _plan_vs_oracle(lens, cal, pairs, boosts, grids, pair_grid, spec, 256, 256, src)
    assert want.sum() > 0
    assert rel_l2(got, want) < IMG_TOL


@pytest.mark.parametrize("golden", ["refgpu_pfs_dg_axial_c0", "refgpu_pfs_dg_axial_c1", "refgpu_ab_dg_axial",
                                    "refgpu_ab_hex_axial"])
def test_render_matches_reference_gpu_golden(pins, meta, ref_images, golden):
    """Against the reference renderer's own GPU output (validation/goldens,
    concentration off): same lens, sampling, spectral table and gain."""
    import ghostlight_gb300 as gl
    m = meta[golden]
    lens = _lens(pins, m["lens"])
    cal = gl.LensCalibration.from_dict(meta[m["lens"]]["calibration"])
    cfg = gl.PointFlareConfig(ray_grid=m["ray_grid"], spectral_samples=m["spectral_samples"],
                              pupil_jitter=m["pupil_jitter"], jitter_seed=m["jitter_seed"],
                              flare_gain=m["flare_gain"], min_ghost_intensity=m["min_ghost_intensity"],
                              source_r=m["source_rgb"], source_g=m["source_rgb"], source_b=m["source_rgb"],
                              cull_dead_pairs=bool(m.get("cull", False)))
    if m["sensor_half"] != "calib":
        cfg.sensor_half_w = cfg.sensor_half_h = float(m["sensor_half"])
    else:
        cfg.sensor_half_w, cfg.sensor_half_h = cal.sensor_half_w, cal.sensor_half_h
    out = gl.render_point_flare(m["W"], m["H"], lens, cal, cfg, source_angle=(0.0, 0.0))
    got = np.stack([out[k].cpu().numpy() for k in ("ghost_r", "ghost_g", "ghost_b")], -1)
    want = ref_images[golden + "/image"]
    assert got.shape == want.shape
    assert rel_l2(got, want) < IMG_TOL


@pytest.mark.parametrize("golden", ["refgpu_pfs_dg_axial_c1", "refgpu_ab_hex_axial"])
def test_drop_in_point_flare_calibrates_and_solves(pins, meta, ref_images, golden):
    """The reference call shape with nothing precomputed: the lens calibrates
    itself (calibrate_lens) and the source position is solved to a field
    angle (solve_source_angle) before the render."""
    import ghostlight_gb300 as gl
    m = meta[golden]
    lens = gl.OpticalSystem.from_records(lens_from_pins(pins, m["lens"]),
                                         focal_length=meta[m["lens"]]["focal_length"])
    cfg = gl.PointFlareConfig(ray_grid=m["ray_grid"], spectral_samples=m["spectral_samples"],
                              pupil_jitter=m["pupil_jitter"], jitter_seed=m["jitter_seed"],
                              flare_gain=m["flare_gain"], min_ghost_intensity=m["min_ghost_intensity"],
                              source_r=m["source_rgb"], source_g=m["source_rgb"], source_b=m["source_rgb"],
                              source_x=m["source_xy"][0], source_y=m["source_xy"][1],
                              cull_dead_pairs=bool(m.get("cull", False)))
    if m["sensor_half"] != "calib":
        cfg.sensor_half_w = cfg.sensor_half_h = float(m["sensor_half"])
    out = lens.render_point_flare(m["W"], m["H"], cfg)
    got = np.stack([out[k].cpu().numpy() for k in ("ghost_r", "ghost_g", "ghost_b")], -1)
    assert rel_l2(got, ref_images[golden + "/image"]) < IMG_TOL


def test_graph_capture_replays_plan(pins, meta, ref_images):
    from ghostlight_gb300.flare import GhostRenderPlan
    lens = _lens(pins, "cfg1_double_gauss_12")
    cal = meta["cfg1_double_gauss_12"]["calibration"]
    pairs, boosts = ref_images["cfg1_small/pairs"], ref_images["cfg1_small/boosts"]
    spec, corr = ref_images["cfg1_small/spec"], ref_images["cfg1_small/corr"]
    grid = O.aperture_samples(lens.records(), 64, 0)
    src = ref_images["cfg1_small/source"]
    plan = GhostRenderPlan(lens, pairs, boosts, src, [grid], None, spec, corr, 256, 256,
                           cal["sensor_half_w"], cal["sensor_half_h"], 1000.0)
    eager = [torch.zeros((256, 256), device="cuda") for _ in range(3)]
    plan.execute(*eager)
    torch.cuda.synchronize()
    outs = [torch.zeros((256, 256), device="cuda") for _ in range(3)]
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        plan.execute(*outs, stream=s.cuda_stream)   # warm on the capture stream
        s.synchronize()
        with torch.cuda.graph(g, stream=s):
            plan.execute(*outs, stream=s.cuda_stream)
    for o in outs:
        o.zero_()
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip(eager, outs):
        assert rel_l2(b.cpu().numpy(), a.cpu().numpy()) < 1e-5
    plan.close()


def test_edge_cases(pins, meta, ref_images):
    from ghostlight_gb300.flare import GhostRenderPlan
    lens = _lens(pins, "cfg1_double_gauss_12")
    cal = meta["cfg1_double_gauss_12"]["calibration"]
    spec, corr = ref_images["cfg1_small/spec"], ref_images["cfg1_small/corr"]
    pairs, boosts = ref_images["cfg1_small/pairs"], ref_images["cfg1_small/boosts"]
    grid = O.aperture_samples(lens.records(), 16, 0)
    # no pairs -> black image, no launch of the trace kernel
    plan = GhostRenderPlan(lens, np.zeros((0, 2), np.int32), np.zeros(0, np.float32),
                           ref_images["cfg1_small/source"], [grid], None, spec, corr, 7, 5,
                           cal["sensor_half_w"], cal["sensor_half_h"], 1000.0)
    out = [torch.full((5, 7), 3.0, device="cuda") for _ in range(3)]
    plan.execute(*out)
    torch.cuda.synchronize()
    assert all(float(o.abs().max()) == 0.0 for o in out)
    plan.close()
    # 1x1 image and a source far outside the field: finite, non-negative
    for W, H, ang in ((1, 1, 0.0), (37, 23, 1.2)):
        src = np.array([[ang, 0.0, 1.0, 1.0, 1.0]], np.float32)
        plan = GhostRenderPlan(lens, pairs, boosts, src, [grid], None, spec, corr, W, H,
                               cal["sensor_half_w"], cal["sensor_half_h"], 1000.0)
        out = [torch.zeros((H, W), device="cuda") for _ in range(3)]
        plan.execute(*out)
        torch.cuda.synchronize()
        img = np.stack([o.cpu().numpy() for o in out])
        assert np.isfinite(img).all()
        plan.close()
    # bad arguments raise ValueError before any device work
    with pytest.raises(ValueError):
        GhostRenderPlan(lens, np.array([[3, 3]], np.int32), np.ones(1, np.float32),
                        ref_images["cfg1_small/source"], [grid], None, spec, corr, 8, 8,
                        cal["sensor_half_w"], cal["sensor_half_h"], 1000.0)
    with pytest.raises(ValueError):
        GhostRenderPlan(lens, pairs, boosts, ref_images["cfg1_small/source"], [grid], None, spec, corr,
                        0, 8, cal["sensor_half_w"], cal["sensor_half_h"], 1000.0)


def test_off_sensor_cull_keeps_the_image(pins, meta):
    """The device probe cull (three 40^2 wang-jittered passes, 1.25 margin)
    drops pairs without changing the frame: configuration 2 at 15 deg."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300.flare import filter_ghosts_device, prepare_ghost_render
    lens = _lens(pins, "cfg2_wide_angle_24")
    cal = meta["cfg2_wide_angle_24"]["calibration"]
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    src = np.array([[np.radians(15.0), 0.0, 1.0, 1.0, 1.0]], np.float32)
    imgs = {}
    for cull in (False, True):
        cfg = gl.FlareConfig(min_ghost_intensity=1e-6, spectral_samples=16, ray_grid=112,
                             cull_dead_pairs=cull)
        fr = filter_ghosts_device(lens, hw, hh, cfg)
        plan = prepare_ghost_render(lens, src, 384, 384, cfg, hw, hh, filter_result=fr)
        out = [torch.zeros((384, 384), device="cuda") for _ in range(3)]
        plan.execute(*out)
        torch.cuda.synchronize()
        imgs[cull] = np.stack([o.cpu().numpy() for o in out])
        if cull:
            hits = plan.pair_hits()
            assert (hits == 0).sum() > len(hits) // 4      # most pairs are off-sensor here
        plan.close()
    assert imgs[False].sum() > 0
    assert rel_l2(imgs[True], imgs[False]) < 1e-4


@pytest.mark.parametrize("deg", [0.0, 9.0, 15.0, 24.0])
def test_probe_cull_independent_of_wavelength_split(pins, meta, deg):
    """The pairs the off-sensor probe keeps, and the frame, do not depend on
    how an item's wavelengths are split into tasks: one wavelength per task,
    all of them in one task, and splits between."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300.flare import filter_ghosts_device, prepare_ghost_render
    lens = _lens(pins, "cfg2_wide_angle_24")
    cal = meta["cfg2_wide_angle_24"]["calibration"]
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    src = np.array([[np.radians(deg), np.radians(0.3 * deg), 1.0, 1.0, 1.0]], np.float32)
    cfg = gl.FlareConfig(min_ghost_intensity=1e-6, spectral_samples=31, ray_grid=64, cull_dead_pairs=True)
    fr = filter_ghosts_device(lens, hw, hh, cfg)
    plan = prepare_ghost_render(lens, src, 256, 256, cfg, hw, hh, filter_result=fr)
    kept, imgs = {}, {}
    for chunks in (31, 1, 4, 2):
        plan.set_launch(0, 0, chunks)
        out = [torch.zeros((256, 256), device="cuda") for _ in range(3)]
        plan.execute(*out)
        torch.cuda.synchronize()
        kept[chunks] = plan.pair_hits() > 0
        imgs[chunks] = np.stack([o.cpu().numpy() for o in out])
    plan.close()
    assert kept[31].sum() > 0
    for chunks in (1, 4, 2):
        np.testing.assert_array_equal(kept[chunks], kept[31])
        assert rel_l2(imgs[chunks], imgs[31]) < 1e-5


def test_autotuned_launch_shapes_give_the_same_image(pins, meta, ref_images, tmp_path):
    from ghostlight_gb300.autotune import Tuner, tune_ghost_plan
    from ghostlight_gb300.flare import GhostRenderPlan
    lens = _lens(pins, "cfg1_double_gauss_12")
    cal = meta["cfg1_double_gauss_12"]["calibration"]
    pairs, boosts = ref_images["cfg1_small/pairs"], ref_images["cfg1_small/boosts"]
    spec, corr = ref_images["cfg1_small/spec"], ref_images["cfg1_small/corr"]
    grid = O.aperture_samples(lens.records(), 96, 0)
    plan = GhostRenderPlan(lens, pairs, boosts, ref_images["cfg1_small/source"], [grid], None, spec, corr,
                           256, 256, cal["sensor_half_w"], cal["sensor_half_h"], 1000.0)
    ref = [torch.zeros((256, 256), device="cuda") for _ in range(3)]
    plan.execute(*ref)
    torch.cuda.synchronize()
    want = torch.stack(ref).cpu().numpy()
    for shape in ((0, 4), (1, 0), (8, 0), (0, 0, 4), (2, 0, 3), (0, 0, 8)):
        plan.set_launch(*shape)
        outs = [torch.zeros((256, 256), device="cuda") for _ in range(3)]
        plan.execute(*outs)
        torch.cuda.synchronize()
        assert rel_l2(torch.stack(outs).cpu().numpy(), want) < 1e-6
    t = Tuner(cache_path=str(tmp_path / "t.json"), reps=2)
    choice = tune_ghost_plan(plan, ref, tuner=t)
    assert tuple(choice) in [tuple(c) for c in __import__("ghostlight_gb300.autotune").autotune.GHOST_CANDIDATES]
    plan.close()


def test_aov_per_pair_layers():
    """GhostAovMode.PER_PAIR: one ghost_s{a}_s{b} triplet per active pair
    (the first aov_max_pairs of them), each the render of that pair alone,
    and the combined planes their sum."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300 import prescriptions as P
    from ghostlight_gb300.flare import render_ghosts
    lens = gl.OpticalSystem.from_records(P.double_gauss_12(seed=1))
    cal = lens.calibration()
    cfg = gl.FlareConfig(ray_grid=24, spectral_samples=8)
    src = np.array([[0.05, 0.02, 1.0, 1.0, 1.0]], np.float32)
    full = render_ghosts(lens, src, 96, 80, cfg, cal.sensor_half_w, cal.sensor_half_h)
    cfg.aov_mode = gl.GhostAovMode.PER_PAIR
    cfg.aov_max_pairs = 5
    aov = render_ghosts(lens, src, 96, 80, cfg, cal.sensor_half_w, cal.sensor_half_h)
    keys = sorted(k for k in aov if k.startswith("ghost_s"))
    assert len(keys) == 15
    tot = sum(aov[k].cpu().numpy() for k in keys if k.endswith("_g"))
    np.testing.assert_allclose(aov["ghost_g"].cpu().numpy(), tot, rtol=1e-5, atol=1e-9)
    assert float(aov["ghost_g"].sum()) <= float(full["ghost_g"].sum()) * (1 + 1e-4)
    # one layer equals the include-filtered render of that pair alone
    name = keys[0]
    a, b = int(name.split("_")[1][1:]), int(name.split("_")[2][1:])
    cfg1 = gl.FlareConfig(ray_grid=24, spectral_samples=8, cull_dead_pairs=False)
    cfg1.ghost_filter.mode = gl.GhostFilterMode.INCLUDE
    cfg1.ghost_filter.pairs = [(a, b)]
    one = render_ghosts(lens, src, 96, 80, cfg1, cal.sensor_half_w, cal.sensor_half_h)
    np.testing.assert_allclose(aov["ghost_s%d_s%d_g" % (a, b)].cpu().numpy(), one["ghost_g"].cpu().numpy(),
                               rtol=1e-5, atol=1e-9)


def test_collect_stats_counts_match_oracle():
    """collect_stats: the diagnostic pass's per-pair counters against the
    oracle's float trace of the same rays (traces exact; survived and
    on-sensor within the rays that graze an edge within rounding)."""
    import ghostlight_gb300 as gl
    from ghostlight_gb300 import prescriptions as P
    from ghostlight_gb300.flare import render_ghosts, pupil_grid, spectral_table
    lens = gl.OpticalSystem.from_records(P.double_gauss_12(seed=1))
    cal = lens.calibration()
    cfg = gl.FlareConfig(ray_grid=24, spectral_samples=8, collect_stats=True)
    src = np.array([[0.0, 0.0, 1.0, 1.0, 1.0]], np.float32)      # on axis: launches straight down z
    out = render_ghosts(lens, src, 96, 80, cfg, cal.sensor_half_w, cal.sensor_half_h)
    st = out["stats"]
    assert st["n_pairs"] == len(st["pair_traces"]) > 0 and st["n_spec"] == 8
    grid = pupil_grid(lens, 24)
    assert st["pair_traces"][0] == len(grid) * 8
    assert st["traces_total"] == sum(st["pair_traces"]) >= st["traces_survived"] >= st["traces_on_sensor"] > 0
    spec, _ = spectral_table(8)
    surfs = lens.records()
    for i in range(min(4, st["n_pairs"])):
        a, b = st["pair_surf_a"][i], st["pair_surf_b"][i]
        n = len(grid)
        rays = np.zeros((n * 8, 7), np.float32)
        d = np.array([0.0, 0.0, 1.0], np.float32)
        for k, lam in enumerate(spec[:, 0]):
            rays[k * n:(k + 1) * n, 0] = grid[:, 0] * surfs[0].semi_aperture
            rays[k * n:(k + 1) * n, 1] = grid[:, 1] * surfs[0].semi_aperture
            rays[k * n:(k + 1) * n, 2] = surfs[0].z - 20.0
            rays[k * n:(k + 1) * n, 3:6] = d
            rays[k * n:(k + 1) * n, 6] = lam
        r = O.trace(surfs, a, b, rays, fp64=False)
        ok = (r[:, 4] == 0) & np.isfinite(r[:, 0]) & np.isfinite(r[:, 1])
        assert abs(int(ok.sum()) - st["pair_survived"][i]) <= max(2, 0.01 * ok.sum()), (a, b)

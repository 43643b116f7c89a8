"""Source sweep as one CUDA graph: replay equals direct enqueue, each frame's
ghost layer equals a plan render of its source and the FP64 oracle's render,
and the starburst lands on the source's image point."""
import math

import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _setup(with_starburst):
    import ghostlight_gb300 as gl
    from ghostlight_gb300.serve import ResidentLens, serving_lens, _spectral
    from ghostlight_gb300.starburst import build_pupil
    from ghostlight_gb300.sweep import SourceSweep, diagonal_sources, paraxial_centers
    cfg = gl.FlareConfig(min_ghost_intensity=1e-6)
    lens, hw, hh = serving_lens(301, 12)
    rl = ResidentLens(lens, hw, hh, cfg)
    W, H, L, G = 256, 128, 8, 48
    src = diagonal_sources(4, 15.0, hw, hh, 50.0, 50.0)
    sb = None
    if with_starburst:
        spec, _ = _spectral(L, cfg)
        lam = spec[:, 0].astype(np.float64)
        sx = (400.0 / lam) / 256.0
        sy = sx * 1.3
        w = (spec[:, 1:4] / 1e4).astype(np.float32)
        plan = gl.MdftPlan(128, (W, H), sx, sy, w, "split_bf16")
        cent = paraxial_centers(src, 50.0, 50.0, hw, hh, W, H)
        sb = dict(plan=plan, pupil=build_pupil(lens, 128, 0.3), centers=cent)
    return rl, cfg, SourceSweep(rl, src, W, H, L, G, starburst=sb), src, sb


def test_graph_replay_equals_direct_enqueue():
    rl, cfg, sw, src, sb = _setup(True)
    sw.run()
    direct = [sw.frame(k).cpu().numpy() for k in range(sw.n_frames)]
    sw.capture()
    sw.replay()
    torch.cuda.synchronize()
    assert sb["plan"].status() == 0
    for k in range(sw.n_frames):
        got = sw.frame(k).cpu().numpy()
        assert np.abs(got).sum() > 0
        assert rel_l2(got, direct[k]) < 1e-5
    assert sw.traced() > 0
    sw.close(); sb["plan"].close(); rl.close()


def test_frames_equal_plan_renders_and_starburst_is_centred():
    from ghostlight_gb300.flare import GhostRenderPlan, pupil_grid
    from ghostlight_gb300.serve import _spectral
    rl, cfg, sw, src, _ = _setup(False)
    sw.capture()
    sw.replay()
    torch.cuda.synchronize()
    spec, corr = _spectral(sw.n_spec, cfg)
    grid = pupil_grid(rl.lens, sw.ray_grid, 0, 0, 0, 0.0)
    for k in range(sw.n_frames):
        s = np.array([[src[k, 0], src[k, 1], 1.0, 1.0, 1.0]], np.float32)
        plan = GhostRenderPlan(rl.lens, rl.pairs, rl.boosts, s, [grid], np.zeros(len(rl.pairs), np.int32), spec,
                               corr, sw.width, sw.height, rl.sensor_half_w, rl.sensor_half_h, 1000.0,
                               apply_correction=True, cull_dead_pairs=True)
        outs = [torch.zeros((sw.height, sw.width), device="cuda") for _ in range(3)]
        plan.execute(*outs)
        torch.cuda.synchronize()
        want = torch.stack(outs).cpu().numpy()
        plan.close()
        assert rel_l2(sw.frame(k).cpu().numpy(), want) < 1e-5
    sw.close(); rl.close()
    # starburst alone: its brightest pixel sits at the paraxial centre
    rl, cfg, sw, src, sb = _setup(True)
    planes = torch.zeros((3, sw.height, sw.width), device="cuda")
    cx, cy = 0.3 * sw.width + 0.37, 0.6 * sw.height - 0.21
    sb["plan"].set_center(cx, cy)
    sb["plan"].execute(sb["pupil"], planes[0], planes[1], planes[2])
    torch.cuda.synchronize()
    g = planes[1].cpu().numpy()
    y, x = np.unravel_index(np.argmax(g), g.shape)
    assert abs(x - cx) <= 1.0 and abs(y - cy) <= 1.0
    sw.close(); sb["plan"].close(); rl.close()


def test_sweep_frames_match_fp64_oracle():
    """Each replayed frame's ghost layer against the FP64 oracle's render of
    the same lens, pairs, grid, spectrum and source (colour correction
    applied): relative L2 below 1e-3."""
    from oracle import oracle as O
    from ghostlight_gb300.flare import pupil_grid
    from ghostlight_gb300.serve import _spectral
    rl, cfg, sw, src, _ = _setup(False)
    sw.capture()
    sw.replay()
    torch.cuda.synchronize()
    spec, corr = _spectral(sw.n_spec, cfg)
    grid = pupil_grid(rl.lens, sw.ray_grid, 0, 0, 0, 0.0)
    for k in range(sw.n_frames):
        s = np.array([[src[k, 0], src[k, 1], 1.0, 1.0, 1.0]], np.float32)
        want = O.render(rl.lens.records(), rl.pairs, rl.boosts, s, [grid], spec, rl.sensor_half_w,
                        rl.sensor_half_h, sw.width, sw.height, 1000.0, fp64=True)
        want = np.einsum("ij,jhw->ihw", corr.astype(np.float64), want)
        assert np.abs(want).sum() > 0, k
        assert rel_l2(sw.frame(k).cpu().numpy(), want) < 1e-3, k
    sw.close(); rl.close()

"""Bitmap (IMAGE) apertures on the GPU: the device culler's ghost set
against the reference's (tests/golden/image_pins.npz), the batched render
within 1e-3 relative L2 of the FP64 oracle and of the reference's own host
render, and the device trace against the oracle (nearest-pixel sampling on
both sides: decisions differ only for hits within rounding of a pixel
boundary)."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as O
from test_aperture_images import image_lens, meta, pins, register_oracle  # noqa: F401

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_device_culler(pins, meta):
    import ghostlight_gb300 as gl
    from ghostlight_gb300.flare import filter_ghosts_device
    cal = meta["calibration"]
    r = filter_ghosts_device(image_lens(), cal["sensor_half_w"], cal["sensor_half_h"],
                             gl.FlareConfig(min_ghost_intensity=1e-7))
    np.testing.assert_array_equal(r.pairs, pins["pairs"])
    np.testing.assert_allclose(r.boosts, pins["boosts"], rtol=1e-5)


def test_render_matches_oracle_and_reference(pins, meta):
    from ghostlight_gb300.flare import GhostRenderPlan, pupil_grid, spectral_table
    lens = image_lens()
    register_oracle(lens)
    cal = meta["calibration"]
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    pairs, boosts, src = pins["pairs"], pins["boosts"], pins["source"]
    spec, corr = spectral_table(8)
    grid = pupil_grid(lens, 48)
    W = H = 128
    plan = GhostRenderPlan(lens, pairs, boosts, src, [grid], np.zeros(len(pairs), np.int32), spec, corr,
                           W, H, hw, hh, 1000.0, apply_correction=False)
    out = [torch.zeros((H, W), dtype=torch.float32, device="cuda") for _ in range(3)]
    plan.execute(*out)
    torch.cuda.synchronize()
    got = np.stack([o.cpu().numpy() for o in out])
    plan.close()
    want = O.render(lens.records(), pairs, boosts, src, [grid], spec, hw, hh, W, H, 1000.0, fp64=True)
    assert want.sum() > 0
    assert rel_l2(got, want) < 1e-3
    assert rel_l2(got, pins["image"]) < 2e-3


def test_device_trace_matches_oracle():
    import ghostlight_gb300 as gl
    lens = image_lens()
    register_oracle(lens)
    surfs = lens.records()
    rng = np.random.default_rng(5)
    n = 16384
    R0 = surfs[0].semi_aperture
    ang = rng.uniform(-0.2, 0.2, (n, 2))
    rays = np.stack([rng.uniform(-1, 1, n) * R0, rng.uniform(-1, 1, n) * R0, np.full(n, surfs[0].z - 20.0),
                     np.sin(ang[:, 0]), np.sin(ang[:, 1]), np.ones(n), rng.uniform(400, 700, n)], 1)
    rays[:, 3:6] /= np.linalg.norm(rays[:, 3:6], axis=1, keepdims=True)
    rays = rays.astype(np.float32)
    for a, b in ((-1, -1), (2, 5), (1, 8)):
        got = gl.trace_rays(lens, torch.from_numpy(rays).cuda(), a, b).cpu().numpy()
        want = O.trace(surfs, a, b, rays, fp64=False)
        assert (got[:, 4] == want[:, 4]).mean() >= 0.995
        ok = (got[:, 4] == 0) & (want[:, 4] == 0)
        assert ok.mean() > 0.02
        rw = np.abs(got[ok, 3] - want[ok, 3]) / np.maximum(want[ok, 3], 1e-30)
        assert np.median(rw) < 1e-4

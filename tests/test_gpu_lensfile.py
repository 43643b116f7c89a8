"""A lens loaded from a ghostlight-optical file, end to end on the GPU: the
device culler's ghost set bit-exact against the oracle's, the batched render
within 1e-3 relative L2 of the FP64 oracle.  The rig fixture has tilted and
pivoted elements, so the trace runs its general (transformed) surface path."""
import warnings

import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

LENSES = __import__("pathlib").Path(__file__).resolve().parent / "golden" / "lenses"


@pytest.mark.parametrize("name", ["fixture_rig", "fixture_minimal"])
def test_lens_file_flare_matches_oracle(name):
    import ghostlight_gb300 as gl
    from ghostlight_gb300.flare import GhostRenderPlan, filter_ghosts_device, pupil_grid, spectral_table
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lens = gl.load_lens(LENSES / (name + ".lens"))
    cal = lens.calibration()
    hw, hh = cal.sensor_half_w, cal.sensor_half_h
    cfg = gl.FlareConfig(min_ghost_intensity=1e-7)
    fr = filter_ghosts_device(lens, hw, hh, cfg)
    want_pairs, want_boosts = O.filter_pairs(lens.records(), hw, hh, 1e-7)
    np.testing.assert_array_equal(fr.pairs, want_pairs)
    np.testing.assert_allclose(fr.boosts, want_boosts, rtol=1e-5)
    grids = [pupil_grid(lens, 48)]
    pair_grid = np.zeros(len(fr.pairs), np.int32)
    spec, corr = spectral_table(8)
    src = np.array([[np.radians(8.0), np.radians(3.0), 1.0, 1.0, 1.0]], np.float32)
    W = H = 128
    plan = GhostRenderPlan(lens, fr.pairs, fr.boosts, src, grids, pair_grid, spec, corr, W, H, hw, hh, 1000.0,
                           apply_correction=False)
    out = [torch.zeros((H, W), dtype=torch.float32, device="cuda") for _ in range(3)]
    plan.execute(*out)
    torch.cuda.synchronize()
    got = np.stack([o.cpu().numpy() for o in out])
    plan.close()
    want = O.render(lens.records(), fr.pairs, fr.boosts, src, grids, spec, hw, hh, W, H, 1000.0,
                    pair_grid=pair_grid, fp64=True)
    assert want.sum() > 0
    assert rel_l2(got, want) < 1e-3

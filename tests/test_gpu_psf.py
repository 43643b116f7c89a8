"""render_psf on the device against the float-oracle restatement."""
import numpy as np
import pytest

from conftest import lens_from_pins, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode,sigma_um,mono", [(0, 0.0, False), (1, 4.0, False), (0, 2.0, True)])
def test_psf_grid_matches_oracle(pins, mode, sigma_um, mono):
    import ghostlight_gb300 as gl
    from ghostlight_gb300.psf_grid import _psf_spectrum
    from ghostlight_gb300.flare import pupil_grid
    from oracle import psf_oracle as PO
    lens = gl.OpticalSystem.from_records(lens_from_pins(pins, "cfg1_double_gauss_12"))
    cfg = gl.PSFConfig(grid_nx=2, grid_ny=2, tile_w=48, tile_h=40, tile_extent_mm=0.08, ray_grid=24,
                       spectral_samples=8, center_mode=mode, splat_sigma_um=sigma_um, monochromatic=mono)
    src = np.array([[0.0, 0.0, 1.0, 0.8, 0.6, 0.0, 0.0], [0.08, 0.03, 0.5, 1.0, 0.7, 3.0, 1.0],
                    [-0.1, 0.06, 1.0, 1.0, 1.0, -4.0, 2.5]], np.float32)
    out = gl.render_psf(src, lens, cfg)
    assert out["composite_w"] == 96 and out["composite_h"] == 80 and len(out["status"]) == 3
    got = np.stack([out[k].cpu().numpy() for k in ("r", "g", "b")]).astype(np.float64)
    # the oracle splats from the same tile centres and aimed directions
    from tests_psf_cells import cells_of
    cells = cells_of(lens, src, mode)
    mm_pp = float(np.float32(cfg.tile_extent_mm) / np.float32(cfg.tile_w))
    from ghostlight_gb300.psf_grid import splat_footprint
    sigma, radius = splat_footprint(sigma_um, mm_pp)
    want = PO.render(lens.records(), cells, src[:, 2:5], pupil_grid(lens, 24, 0, 0, 0, 0.0), _psf_spectrum(cfg),
                     48, 40, 2, 96, 80, mm_pp, mono, sigma, radius)
    assert want.sum() > 0
    assert rel_l2(got, want) < 2e-3

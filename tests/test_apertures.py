"""Seeded starburst pupil (curved 9-blade iris, anti-aliased edge, dust)."""
import numpy as np

from ghostlight_gb300.apertures import curved_blade_mask


def test_curved_blade_mask_properties():
    m = curved_blade_mask(256, blades=9, curvature=0.35, aa_px=2.0, dust_density=0.005, seed=3)
    assert m.shape == (256, 256) and m.dtype == np.float32
    assert m.min() >= 0.0 and m.max() <= 1.0
    # anti-aliased: partial-coverage pixels exist along the edge
    assert ((m > 0.05) & (m < 0.95)).sum() > 200
    # deterministic per seed, different across seeds (dust positions)
    assert np.array_equal(m, curved_blade_mask(256, seed=3))
    assert not np.array_equal(m, curved_blade_mask(256, seed=4))
    # curvature 1 gives a round pupil: the open area approaches pi R^2
    r = curved_blade_mask(256, curvature=1.0, dust_density=0.0)
    R = 0.45 * 256
    assert abs(r.sum() / (np.pi * R * R) - 1.0) < 0.01

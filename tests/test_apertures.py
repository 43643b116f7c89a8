"""Seeded starburst pupil (curved 9-blade iris, anti-aliased edge, dust)."""
import numpy as np
import pytest

from ghostlight_gb300.apertures import blade_radius, curved_blade_mask


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


def test_blade_radius_is_the_oracle_profile():
    """The product's profile (gl_blade_radius) against the oracle's
    independent restatement, bit for bit, for authored and plain stops."""
    from ghostlight_gb300._abi import default_surface
    from oracle import oracle as O
    th = np.linspace(-7.0, 7.0, 4001).astype(np.float32)
    for blades, rot, curv, twist, notch, rake in ((9, 0.1, 0.35, 0.0, 0.0, 0.0), (6, 0.0, -0.6, 0.4, 0.0, 0.0),
                                                  (6, 0.4, 0.2, -0.3, 0.35, 0.26), (5, 0.2, 0.0, 0.0, 0.0, 0.0)):
        s = default_surface()
        s.aperture_shape, s.aperture_blades, s.aperture_rotation_rad = 1, blades, rot
        s.aperture_curvature, s.aperture_twist = curv, twist
        s.aperture_notch_rad, s.aperture_notch_angle_rad = notch, rake
        got = blade_radius(th, blades, np.float32(rot), curv, twist, np.float32(notch), np.float32(rake))
        if curv or twist or notch:
            want = O.blade_radius(s, th)
            np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        assert got.max() <= 1.0 + 1e-6 and got.min() > 0.3
    with pytest.raises(ValueError):
        blade_radius(th, 2)

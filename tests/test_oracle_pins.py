"""The oracle (oracle/gl_oracle.c) against the reference's own outputs
recorded in tests/golden (generated by tests/golden/make_golden.py from the
reference's CPU code built from its sources)."""
import hashlib

import numpy as np
import pytest

from conftest import LENS_NAMES, lens_from_pins, rel_l2
from oracle import oracle as O


@pytest.mark.parametrize("name", LENS_NAMES)
def test_enumeration_matches_reference(pins, name):
    lens = lens_from_pins(pins, name)
    np.testing.assert_array_equal(O.enumerate_pairs(lens), pins[name + "/enumerate"])


@pytest.mark.parametrize("name", LENS_NAMES)
@pytest.mark.parametrize("thr", ["1e-7", "1e-6", "1e-4", "0"])
def test_filter_bit_exact(pins, meta, name, thr):
    lens = lens_from_pins(pins, name)
    cal = meta[name]["calibration"]
    p, b = O.filter_pairs(lens, cal["sensor_half_w"], cal["sensor_half_h"], float(thr))
    np.testing.assert_array_equal(p, pins["%s/filter_%s/pairs" % (name, thr)])
    np.testing.assert_array_equal(b.view(np.uint32), pins["%s/filter_%s/boosts" % (name, thr)].view(np.uint32))


@pytest.mark.parametrize("name", LENS_NAMES)
@pytest.mark.parametrize("cfg", [(32, 0, 0, 0), (64, 1, 7, 0), (192, 2, 12345, 0), (256, 2, 12345, 6)])
def test_pupil_mask_bit_exact(pins, name, cfg):
    lens = lens_from_pins(pins, name)
    s = O.aperture_samples(lens, *cfg)
    key = "%s/samples_%d_%d_%d_%d" % ((name,) + cfg)
    assert len(s) == int(pins[key + "/count"][0])
    assert hashlib.sha256(s.tobytes()).digest() == pins[key + "/sha256"].tobytes()


@pytest.mark.parametrize("name", LENS_NAMES)
def test_trace_float_bit_exact_and_fp64_close(pins, name):
    lens = lens_from_pins(pins, name)
    k = 0
    while "%s/rays_%d/ab" % (name, k) in pins:
        a, b = (int(x) for x in pins["%s/rays_%d/ab" % (name, k)])
        rays = pins["%s/rays_%d/in" % (name, k)]
        want = pins["%s/rays_%d/out" % (name, k)]
        got32 = O.trace(lens, a, b, rays, fp64=False)
        np.testing.assert_array_equal(got32.astype(np.float32), want)
        got64 = O.trace(lens, a, b, rays, fp64=True)
        ok = (want[:, 4] == 0) & (got64[:, 4] == 0)
        # FP32 vs FP64 landing: well inside a micrometre except near grazing rays
        if ok.any():
            d = np.abs(got64[ok, :2] - want[ok, :2].astype(np.float64))
            assert np.median(d) < 1e-4
        assert (want[:, 4] == got64[:, 4]).mean() > 0.98
        k += 1
    assert k >= 2


def test_oracle_render_matches_reference_harness(pins, ref_images, meta):
    """Oracle FP32 render == the reference-code CPU harness image; the FP64
    oracle is within 1e-3 relative L2 of it."""
    lens = lens_from_pins(pins, "cfg1_double_gauss_12")
    cal = meta["cfg1_double_gauss_12"]["calibration"]
    m = meta["cfg1_small"]
    grid = O.aperture_samples(lens, m["grid"], m["jitter"])
    args = (lens, ref_images["cfg1_small/pairs"], ref_images["cfg1_small/boosts"],
            ref_images["cfg1_small/source"], grid, ref_images["cfg1_small/spec"],
            cal["sensor_half_w"], cal["sensor_half_h"], m["W"], m["H"], m["gain"])
    want = ref_images["cfg1_small/image"]
    got32 = O.render(*args, fp64=False)
    assert rel_l2(got32, want) < 1e-6
    got64 = O.render(*args, fp64=True)
    assert rel_l2(got64, want) < 1e-3

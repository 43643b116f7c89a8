"""Authored blade silhouettes (curvature, twist, tip notch) on the host: the
pupil mask, the calibration and the oracle's filter against the reference's
own outputs (tests/golden/blade_pins.npz, made by make_blade_golden.py), bit
for bit; the oracle trace against the live reference where it is present."""
import ctypes
import hashlib
import json
import pathlib

import numpy as np
import pytest

from ghostlight_gb300._abi import gl_surface

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
VARIANTS = ("curved9", "scallop6_twist", "notch6_rake")
SAMPLER_CASES = ((48, 0, 0, 0), (64, 1, 7, 0), (96, 2, 12345, 0), (64, 0, 0, 5))


@pytest.fixture(scope="module")
def bpins():
    return np.load(GOLDEN / "blade_pins.npz")


@pytest.fixture(scope="module")
def bmeta():
    return json.loads((GOLDEN / "blade_meta.json").read_text())


def blade_surfaces(bpins, name):
    raw = bpins[name + "/lens"]
    out = []
    for rec in raw:
        s = gl_surface()
        b = rec.tobytes()
        ctypes.memmove(ctypes.addressof(s), b, len(b))
        out.append(s)
    return out


def _lens(bpins, name):
    from ghostlight_gb300.optics import OpticalSystem
    return OpticalSystem.from_records(blade_surfaces(bpins, name))


@pytest.mark.parametrize("name", VARIANTS)
@pytest.mark.parametrize("case", SAMPLER_CASES, ids=lambda c: "%d_%d_%d_%d" % c)
def test_pupil_mask_bit_exact(bpins, name, case):
    from ghostlight_gb300.flare import pupil_grid
    from oracle import oracle as O
    grid, jit, seed, bo = case
    key = "%s/samples_%d_%d_%d_%d" % (name, grid, jit, seed, bo)
    lens = _lens(bpins, name)
    for s in (pupil_grid(lens, grid, jit, seed, bo), O.aperture_samples(lens.records(), grid, jit, seed, bo)):
        s = np.ascontiguousarray(s, np.float32)
        assert len(s) == int(bpins[key + "/count"][0])
        assert hashlib.sha256(s.tobytes()).digest() == bpins[key + "/sha256"].tobytes()


@pytest.mark.parametrize("name", VARIANTS)
def test_calibration_bit_exact(bpins, bmeta, name):
    from ghostlight_gb300.calibration import calibrate_lens
    cal = calibrate_lens(_lens(bpins, name))
    for k, v in bmeta[name]["calibration"].items():
        assert np.float32(getattr(cal, k)) == np.float32(v), k


@pytest.mark.parametrize("name", VARIANTS)
def test_oracle_filter_bit_exact(bpins, bmeta, name):
    from oracle import oracle as O
    cal = bmeta[name]["calibration"]
    pairs, boosts = O.filter_pairs(blade_surfaces(bpins, name), cal["sensor_half_w"], cal["sensor_half_h"], 1e-7)
    np.testing.assert_array_equal(pairs, bpins[name + "/pairs"])
    np.testing.assert_array_equal(boosts.view(np.uint32), bpins[name + "/boosts"].view(np.uint32))


def test_profile_shapes_differ_from_plain(bpins):
    """The authored variants cut the pupil differently from their plain n-gon."""
    from ghostlight_gb300.flare import pupil_grid
    for name in VARIANTS:
        lens = _lens(bpins, name)
        plain = _lens(bpins, name)
        for s in plain.surfaces:
            s.aperture_curvature = 0.0
            s.aperture_twist = 0.0
            s.aperture_notch_rad = 0.0
        assert len(pupil_grid(lens, 64)) != len(pupil_grid(plain, 64))


@pytest.mark.parametrize("name", VARIANTS)
def test_oracle_trace_matches_reference(bpins, name):
    """Rays aimed at the stop rim: the oracle's float trace (the reference
    host arithmetic) gives the reference's status and landing for each."""
    from oracle import oracle as O
    ref = pytest.importorskip("oracle.ref")
    if not ref.available():
        pytest.skip("reference sources absent")
    surfs = blade_surfaces(bpins, name)
    rng = np.random.default_rng(11)
    R0 = surfs[0].semi_aperture
    n = 2048
    u, v = rng.uniform(-1, 1, n) * R0, rng.uniform(-1, 1, n) * R0
    rays = np.stack([u, v, np.full(n, surfs[0].z - 20.0), np.zeros(n), np.zeros(n), np.ones(n),
                     rng.uniform(400, 700, n)], 1).astype(np.float32)
    want = ref.trace(surfs, -1, -1, rays)
    got = O.trace(surfs, -1, -1, rays, fp64=False)
    np.testing.assert_array_equal(got[:, 4], want[:, 4])
    ok = want[:, 4] == 0
    assert 0.05 < ok.mean() < 0.95
    np.testing.assert_array_equal(got[ok, :4].astype(np.float32), want[ok, :4].astype(np.float32))
    # the authored edge decides some of these rays: the plain n-gon differs
    for s in surfs:
        s.aperture_curvature = s.aperture_twist = s.aperture_notch_rad = 0.0
    plain = ref.trace(surfs, -1, -1, rays)
    assert (plain[:, 4] != want[:, 4]).sum() > 0

"""Table-backed coatings on the host: the lens loader's tables, the thin-film
bake, the calibration and the oracle's filter against the reference's own
outputs (tests/golden/coating_pins.npz, made by make_coating_golden.py), bit
for bit; the oracle trace against the live reference where it is present;
and the OpticalSystem coating accessors (bind_geometry.cpp:412-627)."""
import json
import pathlib
import warnings

import numpy as np
import pytest

from ghostlight_gb300 import coatings as K
from ghostlight_gb300 import load_lens
from ghostlight_gb300.optics import OpticalSystem

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
LENS = GOLDEN / "lenses" / "fixture_coatings.lens"
MGF2 = [(0.40, 1.3904, 0.0), (0.55, 1.3800, 0.0), (0.70, 1.3761, 0.0)]
ZRO2 = [(0.40, 2.2000, 2e-4), (0.50, 2.1500, 1e-4), (0.60, 2.1250, 0.0), (0.70, 2.1100, 0.0)]
STACK = [{"material": "ZrO2", "thickness_nm": 65.5, "nk_table": np.array(ZRO2, np.float32)},
         {"material": "MgF2", "thickness_nm": 99.6, "nk_table": np.array(MGF2, np.float32)}]


@pytest.fixture(scope="module")
def pins():
    return np.load(GOLDEN / "coating_pins.npz")


@pytest.fixture(scope="module")
def meta():
    return json.loads((GOLDEN / "coating_meta.json").read_text())


def coated():
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return load_lens(LENS)


def register_oracle(lens):
    """Give the oracle each table the lens's records name."""
    from oracle import oracle as O
    for s in lens.surfaces:
        if s.coating_model in K.TABLE_MODELS and s.ar_layers:
            model, a0, a1, r, rior, disc = K.read_table(s.ar_layers)
            O.register_coating(s.ar_layers, model, a0, r, a1 if len(a1) else None, rior, disc)


def bits(x):
    return np.ascontiguousarray(x, np.float32).view(np.uint32)


def test_loader_tables_bit_exact(pins):
    lens = coated()
    kinds = []
    for i, s in enumerate(lens.surfaces):
        model, disc = (int(v) for v in pins["loader/%d/meta" % i])
        if s.coating_model not in K.TABLE_MODELS:
            assert model == s.coating_model and pins["loader/%d/axis0" % i].size == 0
            continue
        got = K.read_table(s.ar_layers)
        kinds.append(got[0])
        assert got[0] == model and got[5] == bool(disc)
        assert np.float32(got[4]) == pins["loader/%d/ref_ior" % i][0]
        for k, key in ((1, "axis0"), (2, "axis1"), (3, "r")):
            np.testing.assert_array_equal(bits(got[k]).ravel(), bits(pins["loader/%d/%s" % (i, key)]).ravel())
    assert sorted(kinds) == [1, 2, 3, 3]
    assert lens.unsupported == []


def test_bake_bit_exact(pins):
    lens = coated()
    tid = K.bake_layers(lens.records(), 8, STACK)
    model, wl, ang, r, rior, disc = K.read_table(tid)
    assert model == K.SPECTRAL_ANGULAR and not disc and r.shape == (31, 18)
    np.testing.assert_array_equal(wl, np.arange(400, 701, 10, dtype=np.float32))
    np.testing.assert_array_equal(ang, np.arange(0, 86, 5, dtype=np.float32))
    np.testing.assert_array_equal(bits(r), bits(pins["bake/r"]))
    assert np.float32(rior) == pins["bake/ref_ior"][0]
    # the loaded surface 8 is the same bake, so the same table id
    assert lens.surfaces[8].ar_layers == tid
    assert lens.get_coating_layers(8)[1]["material"] == "MgF2"


def test_calibration_bit_exact(meta):
    from ghostlight_gb300.calibration import calibrate_lens
    cal = calibrate_lens(coated())
    for k, v in meta["calibration"].items():
        assert np.float32(getattr(cal, k)) == np.float32(v), k


def test_oracle_filter_bit_exact(pins, meta):
    from oracle import oracle as O
    lens = coated()
    register_oracle(lens)
    cal = meta["calibration"]
    pairs, boosts = O.filter_pairs(lens.records(), cal["sensor_half_w"], cal["sensor_half_h"], 1e-7)
    np.testing.assert_array_equal(pairs, pins["pairs"])
    np.testing.assert_array_equal(bits(boosts), bits(pins["boosts"]))


def test_oracle_image_matches_reference(pins, meta):
    """The FP64 oracle's ghost image of the coated lens against the
    reference's host render (FP32): relative L2 below 1e-3."""
    from oracle import oracle as O
    from ghostlight_gb300.flare import spectral_table
    lens = coated()
    register_oracle(lens)
    surfs = lens.records()
    cal = meta["calibration"]
    spec, _ = spectral_table(8)
    grid = O.aperture_samples(surfs, 48, 0)
    img = O.render(surfs, pins["pairs"], pins["boosts"], pins["source"], [grid], spec, cal["sensor_half_w"],
                   cal["sensor_half_h"], 128, 128, 1000.0)
    ref = pins["image"]
    rel = np.linalg.norm(img - ref) / np.linalg.norm(ref)
    assert np.linalg.norm(ref) > 0 and rel < 1e-3, rel


def _rays(surfs, n, seed, spread):
    rng = np.random.default_rng(seed)
    R0 = surfs[0].semi_aperture
    ang = rng.uniform(-spread, spread, (n, 2))
    rays = np.stack([rng.uniform(-1, 1, n) * R0, rng.uniform(-1, 1, n) * R0, np.full(n, surfs[0].z - 20.0),
                     np.sin(ang[:, 0]), np.sin(ang[:, 1]), np.ones(n), rng.uniform(380, 720, n)], 1)
    rays[:, 3:6] /= np.linalg.norm(rays[:, 3:6], axis=1, keepdims=True)
    return rays.astype(np.float32)


@pytest.mark.parametrize("discard", [False, True])
def test_oracle_trace_matches_reference(discard):
    """Float oracle trace (the reference's host arithmetic) against the live
    reference through every table kind; the discard case clips the angular
    table at 12 degrees and the spectral one at 450..650 nm so that some
    interactions carry no energy."""
    from oracle import oracle as O
    ref = pytest.importorskip("oracle.ref")
    if not ref.available():
        pytest.skip("reference sources absent")
    lens = coated()
    if discard:
        lens.set_coating_angular_table(3, [[0.0, 0.02], [12.0, 0.03]], angle_ref_ior=1.0,
                                       out_of_range_discard=True)
        lens.set_coating_spectral_table(1, [[450.0, 0.01], [550.0, 0.004], [650.0, 0.012]],
                                        out_of_range_discard=True)
    register_oracle(lens)
    surfs = lens.records()
    for s in surfs:
        if s.coating_model in K.TABLE_MODELS and s.ar_layers:
            model, a0, a1, r, rior, disc = K.read_table(s.ar_layers)
            ref.register_coating(s.ar_layers, model, a0, r, a1 if len(a1) else None, rior, disc)
    rays = _rays(surfs, 4096, 3, 0.35)
    zero = 0
    for a, b in ((-1, -1), (1, 3), (3, 5), (1, 8), (5, 8), (2, 3)):
        want = ref.trace(surfs, a, b, rays)
        got = O.trace(surfs, a, b, rays, fp64=False)
        np.testing.assert_array_equal(got[:, 4], want[:, 4])
        ok = want[:, 4] == 0
        assert ok.mean() > 0.03
        np.testing.assert_array_equal(bits(got[ok, :4]), bits(want[ok, :4]))
        zero += int((want[ok, 3] == 0).sum())
    assert (zero > 0) == discard


def test_accessors_round_trip(tmp_path):
    from ghostlight_gb300 import prescriptions as P
    lens = OpticalSystem.from_records(P.double_gauss_12(seed=1))
    lens.set_coating_spectral_table(2, [[600.0, 0.02], [400.0, 0.03], [500.0, 0.01]], out_of_range_discard=True)
    np.testing.assert_array_equal(lens.get_coating_table(2), np.float32([[400, 0.03], [500, 0.01], [600, 0.02]]))
    assert K.table_info(lens.surfaces[2].ar_layers)["out_of_range_discard"]
    lens.set_coating_angular_table(4, [[0.0, 0.01], [60.0, 0.05]], angle_ref_ior=1.6)
    assert K.table_info(lens.surfaces[4].ar_layers)["angle_ref_ior"] == pytest.approx(1.6)
    wl, ang = np.float32([400, 700]), np.float32([0, 45, 90])
    lens.set_coating_sa_table(6, wl, ang, np.float32([[0.01, 0.02, 0.5], [0.02, 0.03, 0.6]]))
    g = lens.get_coating_sa_table(6)
    np.testing.assert_array_equal(g[0], wl)
    np.testing.assert_array_equal(g[1], ang)
    assert g[2].shape == (2, 3)
    lens.set_coating_layers(9, STACK)
    assert [d["material"] for d in lens.get_coating_layers(9)] == ["ZrO2", "MgF2"]
    # equal content, equal id; a different table, another id
    before = lens.surfaces[2].ar_layers
    lens.set_coating_spectral_table(2, [[400.0, 0.03], [500.0, 0.01], [600.0, 0.02]], out_of_range_discard=True)
    assert lens.surfaces[2].ar_layers == before
    lens.set_coating_spectral_table(2, [[400.0, 0.03], [500.0, 0.01]])
    assert lens.surfaces[2].ar_layers != before
    # writer -> reader keeps every table
    lens.save(tmp_path / "c.lens")
    back = load_lens(tmp_path / "c.lens")
    for i in (2, 4, 6, 9):
        a, b = lens.surfaces[i], back.surfaces[i]
        assert (a.coating_model, a.ar_layers) == (b.coating_model, b.ar_layers), i
    c = lens.surfaces[4].coating
    assert c.table_count == 2 and c.sa_n_wavelengths == 0 and not c.out_of_range_discard
    c.out_of_range_discard = True
    assert lens.surfaces[4].coating.out_of_range_discard
    assert lens.surfaces[4].coating.angle_ref_ior == pytest.approx(1.6)
    assert lens.surfaces[6].coating.sa_n_wavelengths == 2 and lens.surfaces[6].coating.sa_n_angles == 3
    lens.clear_coating(6)
    assert lens.surfaces[6].coating_model == 0 and lens.surfaces[6].ar_layers == 0
    assert lens.get_coating_sa_table(6)[0].size == 0


def test_accessor_errors():
    from ghostlight_gb300 import prescriptions as P
    lens = OpticalSystem.from_records(P.double_gauss_12(seed=1))
    with pytest.raises(IndexError):
        lens.set_coating_spectral_table(99, [[400.0, 0.01]])
    with pytest.raises(ValueError):
        lens.set_coating_spectral_table(1, [400.0, 0.01])
    with pytest.raises(ValueError):
        lens.set_coating_sa_table(1, [500.0, 400.0], [0.0], [[0.1], [0.2]])
    with pytest.raises(ValueError):
        lens.set_coating_sa_table(1, [400.0, 500.0], [0.0], [[0.1, 0.2]])
    with pytest.raises(ValueError):
        lens.set_coating_layers(1, [{"thickness_nm": -1.0, "nk_table": np.float32([[0.5, 1.4, 0.0]])}])
    with pytest.raises(ValueError):
        lens.set_coating_layers(1, [])


def test_unknown_table_id_fails_loudly():
    """A record naming a table the store does not hold is an error, not a
    silent bare-Fresnel surface."""
    from ghostlight_gb300 import prescriptions as P
    from ghostlight_gb300.calibration import calibrate_lens
    lens = OpticalSystem.from_records(P.double_gauss_12(seed=1))
    lens.surfaces[3].coating_model = 2
    lens.surfaces[3].ar_layers = 10 ** 6
    with pytest.raises(ValueError, match="unknown coating table"):
        calibrate_lens(lens)
    # id 0 is the reference's null table: bare Fresnel
    lens.surfaces[3].ar_layers = 0
    calibrate_lens(lens)


def test_table_model_mismatch_fails():
    from ghostlight_gb300 import prescriptions as P
    from ghostlight_gb300.calibration import calibrate_lens
    lens = OpticalSystem.from_records(P.double_gauss_12(seed=1))
    lens.set_coating_spectral_table(3, [[400.0, 0.01], [700.0, 0.02]])
    lens.surfaces[3].coating_model = 3
    with pytest.raises(ValueError, match="holds model 1"):
        calibrate_lens(lens)

"""Lens-file reader against the reference's own loader (OpticalSystem::load).

The synthetic fixtures in tests/golden/lenses are pinned by the reference
loader's flat surface tables (tests/golden/lensfile_pins.npz); where the
reference checkout is present, its library lenses and the rejected files are
checked against the live reference loader as well.
"""
from __future__ import annotations

import json
import pathlib
import warnings

import numpy as np
import pytest

from ghostlight_gb300 import OpticalSystem, lens_format_version, load_lens
from ghostlight_gb300._abi import SURFACE_DTYPE, surface_array
from ghostlight_gb300.lensfile import LensFileError

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
LENSES = GOLDEN / "lenses"

TABLE_MODELS = (1, 2, 3)


def _table(lens):
    return np.frombuffer(bytes(surface_array(lens.records())), dtype=SURFACE_DTYPE)


def _compare(ours, ref, unsupported):
    """Field-for-field equality; a table-coated record names its table in
    ar_layers (the reference keeps the table beside the surface)."""
    assert len(ours) == len(ref)
    for name in SURFACE_DTYPE.names:
        a, b = ours[name], ref[name]
        for i in range(len(ours)):
            if name == "ar_layers" and ours["coating_model"][i] in TABLE_MODELS:
                continue
            assert np.array_equal(np.asarray(a[i]).view(np.uint32), np.asarray(b[i]).view(np.uint32)), \
                "surface %d field %s: %r != %r" % (i, name, a[i], b[i])


def _compare_tables(lens, path):
    """Each table-coated surface's table against the live reference loader's."""
    from ghostlight_gb300 import coatings as K
    from oracle import ref
    for i, s in enumerate(lens.surfaces):
        m, a0, a1, r, rior, disc = ref.load_lens_coating(path, i)
        if s.coating_model not in TABLE_MODELS or not s.ar_layers:
            assert len(a0) == 0, "surface %d: the reference has a table" % i
            continue
        got = K.read_table(s.ar_layers)
        assert got[0] == m and got[5] == disc and np.float32(got[4]) == np.float32(rior), i
        for x, y in ((got[1], a0), (got[2], a1), (got[3], r)):
            np.testing.assert_array_equal(np.asarray(x, np.float32).view(np.uint32),
                                          np.asarray(y, np.float32).view(np.uint32))


@pytest.mark.parametrize("name", ["fixture_rig", "fixture_modifiers", "fixture_minimal"])
def test_fixture_matches_reference_loader(name):
    pins = np.load(GOLDEN / "lensfile_pins.npz")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lens = load_lens(LENSES / (name + ".lens"))
    _compare(_table(lens), pins[name + "/lens"], lens.unsupported)
    assert np.float32(lens.focal_length) == pins[name + "/focal"]


def test_fixture_warnings_and_unsupported():
    with pytest.warns(UserWarning) as rec:
        lens = OpticalSystem.load(LENSES / "fixture_modifiers.lens")
    msgs = " ".join(str(w.message) for w in rec)
    for frag in ("truncating to 8", "curvature must be within", "blades >= 3", "empty/invalid 'data'",
                 "aperture_aspect must be > 0", "unknown aperture shape"):
        assert frag in msgs
    # the valid spectral table (surface 4) is table-backed; the later simple
    # coating after the layer stack (surface 5) replaces it
    assert lens.unsupported == []
    assert lens.surfaces[4].coating_model == 1
    np.testing.assert_array_equal(lens.get_coating_table(4), np.float32([[450.0, 0.01], [650.0, 0.02]]))
    s = lens.surfaces
    assert s[1].n_asphere_terms == 8 and s[2].cyl_axis == 1 and not s[4].is_active
    assert s[1].aperture_blades == 9 and s[1].aperture_curvature == 1.0
    assert s[2].aperture_shape == 0 and s[3].aperture_aspect == 1.0
    assert s[5].coating.ar_layers == 1
    assert lens_format_version() == (1, 0)


def test_rig_layout_ends_at_sensor():
    lens = load_lens(LENSES / "fixture_rig.lens")
    assert lens.name == "fixture rig" and lens.num_surfaces() == 13
    # the chain ends near z = 0 (the rear group's rig pivot moves it a little)
    assert abs(lens.surfaces[-1].z + lens.surfaces[-1].thickness) < 0.05
    assert lens.surfaces[7].rot[0] != 1.0 and lens.surfaces[8].rot[0] == lens.surfaces[7].rot[0]


def test_writer_round_trip(tmp_path):
    from ghostlight_gb300 import prescriptions as P
    for surfs in (P.double_gauss_12(), P.wide_angle_24()):
        lens = OpticalSystem.from_records(surfs, name="rt")
        lens.save(tmp_path / "rt.lens")
        back = load_lens(tmp_path / "rt.lens")
        a, b = _table(lens), _table(back)
        for name in SURFACE_DTYPE.names:
            if name in ("z", "thickness"):          # re-accumulated per element: float rounding
                np.testing.assert_allclose(a[name], b[name], atol=1e-4)
            else:
                np.testing.assert_array_equal(a[name], b[name], err_msg=name)


def _doc(**over):
    d = json.loads((LENSES / "fixture_minimal.lens").read_text())
    d.update(over)
    return d


BAD = {
    "format": lambda: _doc(format="zemax"),
    "major": lambda: _doc(version={"major": 2, "minor": 0}),
    "unknown_glass": lambda: _doc(optical_system=[dict(_doc()["optical_system"][0],
                                                       materials=[{"glass": "unobtainium"}])]),
    "surface_count": lambda: _doc(optical_system=[dict(_doc()["optical_system"][0], materials=[])]),
    "form": lambda: _doc(optical_system=[dict(_doc()["optical_system"][0], surfaces=[
        dict(_doc()["optical_system"][0]["surfaces"][0], form={"type": "torus"}),
        _doc()["optical_system"][0]["surfaces"][1]])]),
    "coating_model": lambda: _doc(optical_system=[dict(_doc()["optical_system"][0], surfaces=[
        dict(_doc()["optical_system"][0]["surfaces"][0], modifiers=[{"type": "coating"}]),
        _doc()["optical_system"][0]["surfaces"][1]])]),
    "pivot_element": lambda: _doc(pivots=[{"name": "x", "elements": ["no-such-id"]}]),
    "item_type": lambda: _doc(optical_system=[{"type": "group"}]),
    "dispersion": lambda: _doc(glass_catalogue={"g": {"dispersion": {"model": "schott"}}}),
    "empty": lambda: _doc(optical_system=[]),
}


@pytest.mark.parametrize("case", sorted(BAD))
def test_rejected_files_raise(case, tmp_path):
    p = tmp_path / (case + ".lens")
    p.write_text(json.dumps(BAD[case]()))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        with pytest.raises(LensFileError, match="OpticalSystem.load\\(\\) failed"):
            load_lens(p)
    ref = pytest.importorskip("oracle.ref")
    if ref.available():
        with pytest.raises(RuntimeError):
            ref.load_lens(p)


def _reference_lenses():
    from oracle.stage_ref import checkout
    return sorted((checkout() / "lenses").glob("**/*.lens"))


@pytest.mark.parametrize("path", _reference_lenses(), ids=lambda p: p.stem[:40])
def test_reference_library_lens(path):
    from oracle import ref
    if not ref.available():
        pytest.skip("reference loader not built")
    surfs, fl = ref.load_lens(path)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lens = load_lens(path)
    _compare(_table(lens), np.frombuffer(bytes(surface_array(surfs)), dtype=SURFACE_DTYPE), lens.unsupported)
    _compare_tables(lens, path)
    assert np.float32(lens.focal_length) == np.float32(fl)


@pytest.mark.parametrize("name", ["fixture_rig", "fixture_modifiers", "fixture_minimal", "fixture_coatings"])
def test_fixture_tables_match_live_reference(name):
    from oracle import ref
    if not ref.available():
        pytest.skip("reference loader not built")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lens = load_lens(LENSES / (name + ".lens"))
    _compare_tables(lens, LENSES / (name + ".lens"))

"""Write the lens-file fixtures and pin them with the reference's own loader.

The fixtures under ``tests/golden/lenses/`` are synthetic prescriptions made
here (seeded), each exercising a part of the ``ghostlight-optical`` format:
relative element positions, element rotations about an element pivot, rig
pivots (centroid and manual), every surface form, every coating and aperture
modifier including the malformed ones the loader repairs with a warning, and
both dispersion models.  The reference's C++ loader (``OpticalSystem::load``,
built from its sources into oracle/_ref by oracle/build.py) loads each one and
its flat surface table is stored in ``lensfile_pins.npz``.

    python tests/golden/make_lensfile_golden.py
"""
from __future__ import annotations

import json
import pathlib
import sys
import uuid

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from ghostlight_gb300._abi import SURFACE_DTYPE, surface_array  # noqa: E402

LENSES = HERE / "lenses"


def _uid(rng):
    return str(uuid.UUID(bytes=bytes(rng.integers(0, 256, 16, dtype=np.uint8).tolist()), version=4))


def _glass_catalogue():
    return {
        "crown_s": {"name": "crown S", "dispersion": {"model": "sellmeier",
                                                      "B": [1.0396, 0.2318, 1.0105],
                                                      "C": [0.0060007, 0.020018, 103.56]}},
        "flint_s": {"name": "flint S", "dispersion": {"model": "sellmeier",
                                                      "B": [1.4614, 0.2477, 0.94999],
                                                      "C": [0.011183, 0.050859, 112.04]}},
        "crown_a": {"name": "crown A", "dispersion": {"model": "abbe", "nd": 1.5168, "Vd": 64.17}},
        "lanthanum_a": {"name": "La A", "dispersion": {"model": "abbe", "nd": 1.7725, "Vd": 49.6}},
    }


def _surface(rng, radius, thickness, semi, form="sphere", mods=None, **kw):
    s = {"id": _uid(rng), "semi_aperture": semi, "thickness": thickness,
         "form": {"type": form, "radius": radius}}
    s["form"].update(kw.pop("form_extra", {}))
    if mods:
        s["modifiers"] = mods
    s.update(kw)
    return s


def _element(rng, name, z, surfaces, glasses, mode="absolute", rotation=None, pivot=None, x=0.0, y=0.0):
    t = {"position": {"mode": mode, "x": x, "y": y, "z": z}}
    if rotation:
        t["rotation"] = rotation
    if pivot:
        t["pivot"] = pivot
    return {"type": "element", "id": _uid(rng), "name": name, "transform": t, "surfaces": surfaces,
            "materials": [{"glass": g} for g in glasses]}


def _doc(name, elements, pivots=(), minor=0, focal=50.0):
    return {"format": "ghostlight-optical", "version": {"major": 1, "minor": minor},
            "metadata": {"name": name, "focal_length_mm": focal}, "glass_catalogue": _glass_catalogue(),
            "optical_system": list(elements), "pivots": list(pivots)}


def fixture_rig(rng):
    """The 12-surface double Gauss written as a lens file, then rigged:
    relative element positions, a slightly tilted element about its own
    pivot, and rig pivots (centroid and manual) on element groups."""
    from ghostlight_gb300 import prescriptions as P
    from ghostlight_gb300.lensfile import lens_document
    from ghostlight_gb300.optics import OpticalSystem
    doc = lens_document(OpticalSystem.from_records(P.double_gauss_12()), "fixture rig")
    els = doc["optical_system"]
    for k in (2, 5):                                      # chained on the preceding element's z
        z_prev = els[k - 1]["transform"]["position"]["z"]
        els[k]["transform"]["position"].update(mode="relative_to_preceding",
                                               z=els[k]["transform"]["position"]["z"] - z_prev)
    els[4]["transform"]["rotation"] = {"tilt_x": 0.05, "tilt_y": -0.03, "roll": 7.0}
    els[4]["transform"]["pivot"] = {"x": 0.01, "y": -0.02, "z": 1.5}
    els[4]["transform"]["position"]["x"] = 0.004
    doc["pivots"] = [
        {"id": _uid(rng), "name": "front group", "elements": [els[0]["id"], els[1]["id"]],
         "pivot_point": {"mode": "centroid"},
         "offset": {"position": {"x": 0.003, "y": 0.0, "z": -0.05}, "rotation": {"tilt_x": 0.02, "roll": 2.0}}},
        {"id": _uid(rng), "name": "rear wobble", "elements": [els[-2]["id"], els[-1]["id"]],
         "pivot_point": {"mode": "manual", "x": 0.0, "y": 0.05, "z": -20.0},
         "offset": {"rotation": {"tilt_y": 0.03}}},
        {"id": _uid(rng), "name": "empty", "elements": []},
    ]
    return doc


def fixture_modifiers(rng):
    """Every surface form and modifier, including repaired malformed ones."""
    terms10 = [1.5e-6, -2.0e-9, 3.1e-12, -4.0e-15, 5.0e-18, 0.0, 1.0e-22, -2.0e-25, 7.0e-28, 1.0e-30]
    mods_a = [{"type": "coating", "model": "simple", "ar_layers": 2},
              {"type": "aperture", "shape": "circular", "aperture_aspect": 1.25}]
    mods_b = [{"type": "coating", "model": "artist", "tint": [1.4, 0.3, -0.2], "strength": 0.07},
              {"type": "aperture", "shape": "polygon", "blades": 9, "rotation_deg": -20.0, "curvature": 1.6,
               "twist": -0.4, "notch_deg": 50.0, "notch_angle_deg": 10.0}]
    mods_c = [{"type": "coating", "model": "attenuator_gaussian", "sigma": 4.5, "attenuation_background": 0.1,
               "attenuation_peak": 0.8, "decenter_x": 0.3, "decenter_y": -0.2},
              {"type": "aperture", "shape": "polygon", "blades": 2}]
    mods_d = [{"type": "coating", "model": "simple", "ar_layers": 1},
              {"type": "coating", "model": "spectral", "data": []},
              {"type": "aperture", "shape": "polygon", "blades": 5, "aperture_aspect": -1.0}]
    mods_e = [{"type": "coating", "model": "spectral", "out_of_range": "discard",
               "data": [{"lambda_nm": 650.0, "r": 0.02}, {"lambda_nm": 450.0, "r": 0.01}]},
              {"type": "aperture", "shape": "hexagram"}]
    mods_f = [{"type": "coating", "model": "layers",
               "layers": [{"material": "MgF2", "thickness_nm": 99.6,
                           "nk_table": [{"lambda_um": 0.4, "n": 1.39}, {"lambda_um": 0.7, "n": 1.376}]}]},
              {"type": "coating", "model": "simple", "ar_layers": 1}]
    surfs = [
        _surface(rng, 44.0, 6.0, 20.0, mods=mods_a),
        _surface(rng, -70.0, 1.0, 19.5, form="asphere", mods=mods_b,
                 form_extra={"conic_constant": -0.6, "terms": terms10}),
        _surface(rng, 25.0, 5.5, 16.0, form="cylindrical", mods=mods_c, form_extra={"axis": "y"}),
        _surface(rng, 0.0, 3.0, 15.0, mods=mods_d),
        _surface(rng, -30.0, 4.0, 14.0, form="cylindrical", mods=mods_e, form_extra={"axis": "x"},
                 is_active=False),
        _surface(rng, 60.0, 41.0, 15.5, mods=mods_f),
    ]
    el = _element(rng, "block", -60.0, surfs, ["crown_s", "AIR", "flint_s", "air", "lanthanum_a"])
    return _doc("fixture modifiers", [el], minor=0, focal=35.0)


def fixture_minimal(rng):
    """Abbe glasses only, a newer minor version, no pivots key."""
    el0 = _element(rng, "a", -40.0, [_surface(rng, 30.0, 4.0, 12.0), _surface(rng, -80.0, 0.0, 12.0)],
                   ["crown_a"])
    el1 = _element(rng, "b", -32.0, [_surface(rng, -25.0, 2.0, 10.0), _surface(rng, 40.0, 26.0, 10.0)],
                   ["lanthanum_a"])
    d = _doc("fixture minimal", [el0, el1], minor=7, focal=0.0)
    del d["pivots"]
    return d


FIXTURES = {"fixture_rig": fixture_rig, "fixture_modifiers": fixture_modifiers,
            "fixture_minimal": fixture_minimal}


def write_fixtures():
    LENSES.mkdir(exist_ok=True)
    rng = np.random.default_rng(2024)
    paths = {}
    for name, fn in FIXTURES.items():
        p = LENSES / (name + ".lens")
        p.write_text(json.dumps(fn(rng), indent=2) + "\n")
        paths[name] = p
    return paths


def main():
    from oracle import ref
    paths = write_fixtures()
    out = {}
    for name, p in paths.items():
        surfs, fl = ref.load_lens(p)
        out[name + "/lens"] = np.frombuffer(bytes(surface_array(surfs)), dtype=SURFACE_DTYPE).copy()
        out[name + "/focal"] = np.float32(fl)
    np.savez_compressed(HERE / "lensfile_pins.npz", **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    main()

"""Pin table-backed coatings with the reference's own code.

Builds the seeded double Gauss (double_gauss_12, seed 1) with one coating of each table
kind — a spectral table given out of order, an angular table in discard mode
measured from glass, a spectral-angular table, and a two-layer thin-film stack
— writes it as ``lenses/fixture_coatings.lens``, and records what the
reference's CPU code (oracle/_ref, built from its sources by oracle/build.py)
makes of that file: the loader's tables, the thin-film bake, the calibration,
the filtered ghost set and a small ghost image of its host render mirror.
Outputs: ``coating_pins.npz`` and ``coating_meta.json``.

    python tests/golden/make_coating_golden.py
"""
from __future__ import annotations

import json
import math
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from ghostlight_gb300 import prescriptions as P  # noqa: E402
from ghostlight_gb300.optics import OpticalSystem  # noqa: E402

LENS = HERE / "lenses" / "fixture_coatings.lens"

# (lambda_um, n, k) samples of the two films
MGF2 = [(0.40, 1.3904, 0.0), (0.55, 1.3800, 0.0), (0.70, 1.3761, 0.0)]
ZRO2 = [(0.40, 2.2000, 2e-4), (0.50, 2.1500, 1e-4), (0.60, 2.1250, 0.0), (0.70, 2.1100, 0.0)]
STACK = [{"material": "ZrO2", "thickness_nm": 65.5, "nk_table": np.array(ZRO2, np.float32)},
         {"material": "MgF2", "thickness_nm": 99.6, "nk_table": np.array(MGF2, np.float32)}]


def coated_lens():
    lens = OpticalSystem.from_records(P.double_gauss_12(seed=1), name="fixture coatings")
    rng = np.random.default_rng(5)
    lam = np.array([700, 400, 550, 450, 650, 500, 600, 425, 675, 575], np.float32)
    lens.set_coating_spectral_table(1, np.stack([lam, 0.004 + 0.02 * ((lam - 550) / 150) ** 2], 1))
    ang = np.arange(0, 45, 5, dtype=np.float32)
    lens.set_coating_angular_table(3, np.stack([ang, 0.01 + 0.0004 * ang], 1), angle_ref_ior=1.5,
                                   out_of_range_discard=True)
    wl = np.arange(400, 701, 50, dtype=np.float32)
    aa = np.arange(0, 81, 10, dtype=np.float32)
    r = (0.006 + 0.01 * rng.random((len(wl), len(aa)))).astype(np.float32)
    lens.set_coating_sa_table(5, wl, aa, r)
    lens.set_coating_layers(8, STACK)
    return lens


def table_arrays(out, key, table):
    model, a0, a1, r, ref, disc = table
    out[key + "/axis0"] = np.asarray(a0, np.float32)
    out[key + "/axis1"] = np.asarray(a1, np.float32)
    out[key + "/r"] = np.asarray(r, np.float32)
    out[key + "/meta"] = np.array([model, int(disc)], np.int32)
    out[key + "/ref_ior"] = np.array([ref], np.float32)


def register_reference(lens):
    """Hand the reference driver the tables our loader stored, by the ids
    the records carry."""
    from oracle import ref
    from ghostlight_gb300 import coatings as K
    for s in lens.surfaces:
        if s.coating_model in K.TABLE_MODELS and s.ar_layers:
            model, a0, a1, r, rior, disc = K.read_table(s.ar_layers)
            ref.register_coating(s.ar_layers, model, a0, r, a1 if len(a1) else None, rior, disc)


def main():
    from oracle import ref
    from ghostlight_gb300 import load_lens
    from ghostlight_gb300.flare import spectral_table
    coated_lens().save(LENS)
    out, meta = {}, {}
    lens = load_lens(LENS)
    for i in range(lens.num_surfaces()):
        table_arrays(out, "loader/%d" % i, ref.load_lens_coating(LENS, i))
    surfs = lens.records()
    wl, ang, r, rior = ref.bake_layers(surfs, 8, [(d["thickness_nm"], d["nk_table"]) for d in STACK])
    table_arrays(out, "bake", (3, wl, ang, r, rior, False))
    register_reference(lens)
    cal = ref.calibrate(surfs, 0.0)
    meta["calibration"] = cal
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    pairs, boosts = ref.filter_pairs(surfs, hw, hh, 1e-7)
    out["pairs"], out["boosts"] = pairs, boosts
    spec, _ = spectral_table(8)
    grid = ref.aperture_samples(surfs, 48, 0)
    src = np.array([[math.radians(9.0), math.radians(-3.0), 1.0, 1.0, 1.0]], np.float32)
    out["image"] = ref.render_ghosts_cpu(surfs, pairs, boosts, src, grid, spec, hw, hh, 128, 128, 1000.0)
    out["source"] = src
    np.savez_compressed(HERE / "coating_pins.npz", **out)
    (HERE / "coating_meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print("wrote", len(out), "arrays;", len(pairs), "pairs")


if __name__ == "__main__":
    main()

"""Pin the authored blade silhouette (curvature, twist, tip notch) with the
reference's own code.

Three variants of the seeded 12-surface double Gauss get an authored 6- or
9-blade stop; for each, the reference's CPU code (oracle/_ref, built from its
sources by oracle/build.py) gives the pupil samples, the calibration, the
filtered ghost set and a small ghost image of its host render mirror.  The
outputs go to ``blade_pins.npz`` (arrays) and ``blade_meta.json``.

    python tests/golden/make_blade_golden.py
"""
from __future__ import annotations

import hashlib
import json
import math
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from ghostlight_gb300 import prescriptions as P  # noqa: E402
from ghostlight_gb300._abi import SURFACE_DTYPE, surface_array  # noqa: E402

# (blades, rotation deg, curvature, twist, notch deg, notch angle deg)
VARIANTS = {
    "curved9": (9, 10.0, 0.35, 0.0, 0.0, 0.0),
    "scallop6_twist": (6, 0.0, -0.6, 0.4, 0.0, 0.0),
    "notch6_rake": (6, 25.0, 0.2, -0.3, 20.0, 15.0),
}
SAMPLER_CASES = ((48, 0, 0, 0), (64, 1, 7, 0), (96, 2, 12345, 0), (64, 0, 0, 5))


def blade_lens(variant):
    blades, rot, curv, twist, notch, rake = VARIANTS[variant]
    surfs = P.double_gauss_12(seed=1)
    for s in surfs:
        if s.is_stop:
            s.aperture_shape = 1
            s.aperture_blades = blades
            s.aperture_rotation_rad = float(np.float32(math.radians(rot)))
            s.aperture_curvature = curv
            s.aperture_twist = twist
            s.aperture_notch_rad = float(np.float32(math.radians(notch)))
            s.aperture_notch_angle_rad = float(np.float32(math.radians(rake)))
    return surfs


def main():
    from oracle import ref
    from ghostlight_gb300.flare import spectral_table
    out, meta = {}, {}
    for name in VARIANTS:
        surfs = blade_lens(name)
        out[name + "/lens"] = np.frombuffer(bytes(surface_array(surfs)), dtype=SURFACE_DTYPE).copy()
        cal = ref.calibrate(surfs, 0.0)
        meta[name] = {"calibration": cal}
        for grid, jit, seed, bo in SAMPLER_CASES:
            s = ref.aperture_samples(surfs, grid, jit, seed, bo)
            key = "%s/samples_%d_%d_%d_%d" % (name, grid, jit, seed, bo)
            out[key + "/count"] = np.array([len(s)], np.int64)
            out[key + "/sha256"] = np.frombuffer(hashlib.sha256(s.tobytes()).digest(), np.uint8)
        hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
        pairs, boosts = ref.filter_pairs(surfs, hw, hh, 1e-7)
        out[name + "/pairs"] = pairs
        out[name + "/boosts"] = boosts
        spec, _ = spectral_table(8)
        grid = ref.aperture_samples(surfs, 48, 0)
        src = np.array([[math.radians(6.0), math.radians(2.0), 1.0, 1.0, 1.0]], np.float32)
        out[name + "/image"] = ref.render_ghosts_cpu(surfs, pairs, boosts, src, grid, spec, hw, hh,
                                                     128, 128, 1000.0)
        out[name + "/source"] = src
    np.savez_compressed(HERE / "blade_pins.npz", **out)
    (HERE / "blade_meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()

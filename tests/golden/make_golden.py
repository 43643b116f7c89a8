"""Generate the golden fixtures that pin the oracle and the GPU path.

Run in a checkout where the reference (JaydenB/ghostlight) is available:
it builds the reference's own CPU code (oracle/_ref, see oracle/build.py) and
records its outputs on seeded prescriptions and on two of the reference's own
lens files.  It also copies three of the reference's GPU value goldens
(validation/goldens, produced by the reference renderer with concentration
off) so the GPU render is pinned against the reference's own GPU output.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from ghostlight_gb300 import prescriptions as P  # noqa: E402
from ghostlight_gb300._abi import SURFACE_DTYPE, surface_array  # noqa: E402
from oracle import ref  # noqa: E402
from oracle.stage_ref import checkout  # noqa: E402

REFERENCE_ROOT = checkout()


def lens_bytes(surfs):
    return np.frombuffer(bytes(surface_array(surfs)), dtype=SURFACE_DTYPE).copy()


def main():
    rng = np.random.default_rng(20261203)
    lenses = {
        "cfg1_double_gauss_12": (P.double_gauss_12(seed=1), 0.0),
        "cfg2_wide_angle_24": (P.wide_angle_24(seed=2), 0.0),
        "cfg4_anamorphic_18": (P.anamorphic_18(seed=4), 0.0),
    }
    dg, fl = ref.load_lens(REFERENCE_ROOT / "lenses" / "DoubleGauss.lens")
    lenses["ref_DoubleGauss"] = (dg, fl)
    hx, flh = ref.load_lens(REFERENCE_ROOT / "validation" / "goldens" / "aperture_baseline" / "hex_stop.lens")
    lenses["ref_hex_stop"] = (hx, flh)

    out = {}
    meta = {}
    for name, (surfs, focal) in lenses.items():
        out[name + "/lens"] = lens_bytes(surfs)
        cal = ref.calibrate(surfs, focal)
        meta[name] = {"focal_length": focal, "calibration": cal}
        out[name + "/enumerate"] = ref.enumerate_pairs(surfs)
        hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
        for tag, thr in (("1e-7", 1e-7), ("1e-6", 1e-6), ("1e-4", 1e-4), ("0", 0.0)):
            p, b = ref.filter_pairs(surfs, hw, hh, thr)
            out["%s/filter_%s/pairs" % (name, tag)] = p
            out["%s/filter_%s/boosts" % (name, tag)] = b
        for grid, jit, seed, bo in ((32, 0, 0, 0), (64, 1, 7, 0), (192, 2, 12345, 0), (256, 2, 12345, 6)):
            s = ref.aperture_samples(surfs, grid, jit, seed, bo)
            key = "%s/samples_%d_%d_%d_%d" % (name, grid, jit, seed, bo)
            out[key + "/count"] = np.array([len(s)], np.int64)
            out[key + "/sha256"] = np.frombuffer(hashlib.sha256(s.tobytes()).digest(), np.uint8)
            out[key + "/head"] = s[:128].copy()
        # per-ray pins: random rays through a few pairs (and primary)
        en = ref.enumerate_pairs(surfs)
        pick = en[rng.choice(len(en), size=min(6, len(en)), replace=False)]
        R0 = surfs[0].semi_aperture
        nr = 256
        for k, (a, b) in enumerate(list(pick) + [(-1, -1)]):
            u = rng.uniform(-1, 1, nr) * R0
            v = rng.uniform(-1, 1, nr) * R0
            ang = rng.uniform(-0.25, 0.25, (nr, 2))
            d = np.stack([np.tan(ang[:, 0]), np.tan(ang[:, 1]), np.ones(nr)], 1)
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            rays = np.stack([u - 20 * np.tan(ang[:, 0]), v - 20 * np.tan(ang[:, 1]),
                             np.full(nr, surfs[0].z - 20.0), d[:, 0], d[:, 1], d[:, 2],
                             rng.uniform(400, 700, nr)], 1).astype(np.float32)
            out["%s/rays_%d/ab" % (name, k)] = np.array([a, b], np.int32)
            out["%s/rays_%d/in" % (name, k)] = rays
            out["%s/rays_%d/out" % (name, k)] = ref.trace(surfs, int(a), int(b), rays)
        for nd in ((0.0, 0.0), (0.6, 0.0), (0.3, -0.5)):
            s = ref.solve_source(surfs, cal, nd[0], nd[1], hw, hh)
            meta[name].setdefault("solve", []).append({"ndc": nd, **s})

    for n in (3, 8, 16, 31):
        for cs in (0, 1, 4):
            t, c = ref.spectral_table(n, cs)
            out["spectral/%d_%d/table" % (n, cs)] = t
            out["spectral/%d_%d/corr" % (n, cs)] = c

    # Reference CPU harness images (host mirror of ghost_kernel's main path).
    img = {}
    s1 = lenses["cfg1_double_gauss_12"][0]
    c1 = meta["cfg1_double_gauss_12"]["calibration"]
    p1, b1 = ref.filter_pairs(s1, c1["sensor_half_w"], c1["sensor_half_h"], 1e-7)
    keep = np.array([not P.stop_crossing(s1, int(a), int(b)) for a, b in p1])
    p1, b1 = p1[keep], b1[keep]
    spec8, corr8 = ref.spectral_table(8, 0)
    g32 = ref.aperture_samples(s1, 32, 0)
    src = np.array([[np.radians(10.0), 0.0, 1.0, 1.0, 1.0]], np.float32)
    im = ref.render_ghosts_cpu(s1, p1, b1, src, g32, spec8, c1["sensor_half_w"], c1["sensor_half_h"],
                               128, 128, 1000.0)
    img["cfg1_small/image"] = im
    img["cfg1_small/pairs"] = p1
    img["cfg1_small/boosts"] = b1
    img["cfg1_small/spec"] = spec8
    img["cfg1_small/corr"] = corr8
    img["cfg1_small/source"] = src
    meta["cfg1_small"] = {"grid": 32, "jitter": 0, "W": 128, "H": 128, "gain": 1000.0,
                          "note": "correction NOT applied (raw harness accumulation)"}

    # Reference GPU value goldens (validation/goldens), on-axis DoubleGauss.
    gold = REFERENCE_ROOT / "validation" / "goldens"
    img["refgpu_pfs_dg_axial_c0/image"] = np.load(gold / "point_flare_sampling" / "double_gauss_0.5_0.5_b0_c0.npy")
    meta["refgpu_pfs_dg_axial_c0"] = {"lens": "ref_DoubleGauss", "W": 320, "H": 320, "sensor_half": 14.0,
                                      "ray_grid": 256, "spectral_samples": 16, "pupil_jitter": 2,
                                      "jitter_seed": 12345, "flare_gain": 5000.0, "source_rgb": 10.0,
                                      "min_ghost_intensity": 0.0, "source_xy": [0.5, 0.5],
                                      "origin": "validation/goldens/point_flare_sampling/double_gauss_0.5_0.5_b0_c0.npy"}
    img["refgpu_pfs_dg_axial_c1/image"] = np.load(gold / "point_flare_sampling" / "double_gauss_0.5_0.5_b0_c1.npy")
    meta["refgpu_pfs_dg_axial_c1"] = dict(meta["refgpu_pfs_dg_axial_c0"], cull=True,
                                          origin="validation/goldens/point_flare_sampling/double_gauss_0.5_0.5_b0_c1.npy")
    img["refgpu_ab_dg_axial/image"] = np.load(gold / "aperture_baseline" / "double_gauss__ghost_axial.npy")
    meta["refgpu_ab_dg_axial"] = {"lens": "ref_DoubleGauss", "W": 192, "H": 192, "sensor_half": "calib",
                                  "ray_grid": 192, "spectral_samples": 8, "pupil_jitter": 2,
                                  "jitter_seed": 12345, "flare_gain": 5000.0, "source_rgb": 10.0,
                                  "min_ghost_intensity": 0.0, "source_xy": [0.5, 0.5],
                                  "origin": "validation/goldens/aperture_baseline/double_gauss__ghost_axial.npy"}
    img["refgpu_ab_hex_axial/image"] = np.load(gold / "aperture_baseline" / "hex_stop__ghost_axial.npy")
    meta["refgpu_ab_hex_axial"] = dict(meta["refgpu_ab_dg_axial"], lens="ref_hex_stop",
                                       origin="validation/goldens/aperture_baseline/hex_stop__ghost_axial.npy")

    np.savez_compressed(HERE / "ref_pins.npz", **out)
    np.savez_compressed(HERE / "ref_images.npz", **img)
    (HERE / "ref_meta.json").write_text(json.dumps(meta, indent=1, default=float))
    for f in ("ref_pins.npz", "ref_images.npz", "ref_meta.json"):
        print(f, (HERE / f).stat().st_size // 1024, "KB")


if __name__ == "__main__":
    main()

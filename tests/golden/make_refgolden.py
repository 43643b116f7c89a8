"""Pack the reference's own GPU value goldens as fixtures.

The reference ships GPU-rendered value goldens (validation/goldens, rendered
by its CUDA renderer with deterministic Halton sampling and concentration
off, recorded with CUDA 13.2 and gated by the reference at 1 ppm of peak):

* point_flare_sampling/  DoubleGauss and the Sirui 1.33x anamorphic, 320^2,
  256^2 Halton pupil, 16 wavelengths, sources on axis (0.5, 0.5), off axis
  (1.3, 0.5), in the far corner (1.6, 0.9) and a 6-blade stop override, cull
  off and on (validation/point_flare_sampling_baseline.py:19-48);
* aperture_baseline/  five lenses (DoubleGauss, Sirui, hex stop, hex stop
  rotated 30 deg, curved blades) x {ghost axial / off-axis / corner, the
  5-point source chunk, the PSF atlas, the SPRITE and MDFT starbursts} at
  192^2 (validation/aperture_baseline.py:53-160).

This script records, for each golden, its configuration and the lens as the
reference's own loader flattens it (oracle/_ref), with the reference's
calibration of that lens, and stores the images in ``ref_goldens.npz``.  To
keep the fixture small the stored floats keep 15 of their 23 mantissa bits
(relative error below 3.1e-5 per value, 1.5e-5 relative L2 at worst, against a
1e-3 test tolerance) and are byte-shuffled before compression; ``unpack``
restores them.  The film-gate layer is out of scope and not packed.

    python tests/golden/make_refgolden.py
"""
from __future__ import annotations

import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from ghostlight_gb300._abi import SURFACE_DTYPE, surface_array  # noqa: E402
from oracle import ref  # noqa: E402
from oracle.stage_ref import checkout  # noqa: E402

ROOT = checkout()
GOLD = ROOT / "validation" / "goldens"
LENSES = {
    "double_gauss": ROOT / "lenses" / "DoubleGauss.lens",
    "sirui": ROOT / "lenses" / "anamorphic" / "Sirui_75mm_F1.8_1.33x_EP3936919NWA1.lens",
    "hex_stop": GOLD / "aperture_baseline" / "hex_stop.lens",
    "hex_rot30": GOLD / "aperture_baseline" / "hex_stop_rot30.lens",
    "blade_shape": GOLD / "aperture_baseline" / "blade_shape.lens",
}
MANTISSA_DROP = 8


def pack(a):
    """float32 array -> byte-shuffled uint8 (4, n) with the low mantissa bits
    cleared (round to nearest, ties away)."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    half = np.uint64(1 << (MANTISSA_DROP - 1))
    mask = np.uint64((0xFFFFFFFF >> MANTISSA_DROP) << MANTISSA_DROP)
    fin = np.isfinite(a).reshape(-1)
    r = u.reshape(-1).copy()
    r[fin] = ((r[fin] + half) & mask)
    r = r.astype(np.uint32)
    # rounding must not carry a finite value into inf
    bad = fin & ~np.isfinite(r.view(np.float32))
    r[bad] = a.reshape(-1).view(np.uint32)[bad] & np.uint32(mask)
    return r.view(np.uint8).reshape(-1, 4).T.copy()


def unpack(b, shape):
    return np.ascontiguousarray(b.T).reshape(-1).view(np.float32).reshape(shape).copy()


def main():
    meta = {"mantissa_bits_kept": 23 - MANTISSA_DROP, "lenses": {}, "goldens": {}}
    arrays = {}
    manifest = json.loads((GOLD / "aperture_baseline" / "manifest.json").read_text())
    for name, path in LENSES.items():
        surfs, fl = ref.load_lens(path)
        raw = np.frombuffer(bytes(surface_array(surfs)), dtype=SURFACE_DTYPE).copy()
        arrays["lens/" + name] = raw
        meta["lenses"][name] = {"file": str(path.relative_to(ROOT)), "focal_length": fl,
                                "calibration": ref.calibrate(surfs, fl),
                                "manifest_calibration": manifest.get(name)}
    pfs = {"double_gauss": "double_gauss", "sirui": "sirui"}
    for stem, lens in pfs.items():
        for sx, sy, blades in ((0.5, 0.5, 0), (1.3, 0.5, 0), (1.6, 0.9, 0), (1.3, 0.5, 6)):
            for cull in (0, 1):
                key = "%s_%s_%s_b%d_c%d" % (stem, sx, sy, blades, cull)
                img = np.load(GOLD / "point_flare_sampling" / (key + ".npy"))
                arrays["img/pfs/" + key] = pack(img)
                meta["goldens"]["pfs/" + key] = {
                    "lens": lens, "kind": "ghost", "shape": list(img.shape), "W": 320, "H": 320,
                    "sensor_half": [14.0, 14.0], "ray_grid": 256, "spectral_samples": 16, "pupil_jitter": 2,
                    "jitter_seed": 12345, "flare_gain": 5000.0, "source_rgb": 10.0,
                    "min_ghost_intensity": 0.0, "source_xy": [sx, sy], "aperture_blades": blades,
                    "cull": bool(cull),
                    "origin": "validation/goldens/point_flare_sampling/%s.npy" % key}
    src_chunk = [[0.0, 0.0, 0.36], [0.0012, 0.0, 0.16], [-0.0012, 0.0, 0.16], [0.0, 0.0012, 0.16],
                 [0.0, -0.0012, 0.16]]
    for lens in LENSES:
        for layer in ("ghost_axial", "ghost_offaxis", "ghost_corner", "source_chunk", "psf",
                      "starburst_sprite", "starburst_mdft"):
            key = "%s__%s" % (lens, layer)
            img = np.load(GOLD / "aperture_baseline" / (key + ".npy"))
            arrays["img/ab/" + key] = pack(img)
            base = {"lens": lens, "shape": list(img.shape), "W": 192, "H": 192, "sensor_half": "calib",
                    "ray_grid": 192, "spectral_samples": 8, "pupil_jitter": 2, "jitter_seed": 12345,
                    "flare_gain": 5000.0, "source_rgb": 10.0, "min_ghost_intensity": 0.0, "cull": True,
                    "origin": "validation/goldens/aperture_baseline/%s.npy" % key}
            if layer.startswith("ghost_"):
                xy = {"ghost_axial": [0.5, 0.5], "ghost_offaxis": [1.3, 0.5], "ghost_corner": [1.6, 0.9]}[layer]
                g = dict(base, kind="ghost", source_xy=xy)
            elif layer == "source_chunk":
                g = dict(base, kind="source_chunk", source_xy=[0.7, 0.5], offsets=src_chunk)
            elif layer == "psf":
                g = dict(base, kind="psf", grid_nx=3, grid_ny=3, tile_w=48, tile_h=48, tile_extent_mm=0.12,
                         spectral_samples=4, ray_grid=48, field_frac=0.5)
            else:
                g = dict(base, kind="starburst", source_xy=[0.5, 0.5],
                         engine="SPRITE" if layer.endswith("sprite") else "MDFT", starburst_grid=512,
                         pupil_fill=0.30, scale_trim=8.0, sb_spectral_samples=8)
            meta["goldens"]["ab/" + key] = g
    np.savez_compressed(HERE / "ref_goldens.npz", **arrays)
    (HERE / "ref_goldens.json").write_text(json.dumps(meta, indent=1, default=float))
    print("ref_goldens.npz", (HERE / "ref_goldens.npz").stat().st_size // 1024, "KB,",
          len(meta["goldens"]), "goldens")


if __name__ == "__main__":
    main()

"""Pin bitmap (IMAGE) apertures with the reference's own code.

The seeded double Gauss (double_gauss_12, seed 1) gets two bitmap apertures:
a six-pointed star iris at the stop and a dust mask on the front element,
each an 8-bit grey PNG written here (``lenses/iris_star.png``,
``lenses/front_dust.png``) and named by ``lenses/fixture_image.lens``.  The
reference's CPU code (oracle/_ref, built from its sources by oracle/build.py)
is given the decoded pixels (as its Python loader would attach them) and
records the calibration, the filtered ghost set and a small ghost image of its
host render mirror.  Outputs: ``image_pins.npz`` and ``image_meta.json``.

    python tests/golden/make_image_golden.py
"""
from __future__ import annotations

import json
import math
import pathlib
import struct
import sys
import zlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from ghostlight_gb300 import prescriptions as P  # noqa: E402
from ghostlight_gb300.optics import OpticalSystem  # noqa: E402

LENSES = HERE / "lenses"


def write_png(path, grey):
    """8-bit greyscale PNG, filter 0 on every row."""
    g = np.asarray(grey, np.uint8)
    h, w = g.shape
    raw = b"".join(b"\x00" + g[y].tobytes() for y in range(h))

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xffffffff)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 0, 0, 0, 0)) + \
        chunk(b"IDAT", zlib.compress(raw, 9)) + chunk(b"IEND", b"")
    pathlib.Path(path).write_bytes(png)


def star_mask(n=96, points=6):
    yy, xx = (np.mgrid[:n, :n] + 0.5) / n * 2 - 1
    r, a = np.hypot(xx, yy), np.arctan2(yy, xx)
    edge = 0.62 + 0.33 * np.cos(points * a) ** 2
    return np.where(r < edge, 255, 0).astype(np.uint8)


def dust_mask(n=128, seed=4):
    rng = np.random.default_rng(seed)
    m = np.full((n, n), 230, np.uint8)
    yy, xx = np.mgrid[:n, :n]
    for _ in range(40):
        cx, cy, rad = rng.uniform(0, n, 2).tolist() + [rng.uniform(1.5, 5.0)]
        if (cx - n / 2) ** 2 + (cy - n / 2) ** 2 < (n / 8) ** 2:
            continue        # keep the axis clear: the culler's intensity probe is the axial ray
        m[(xx - cx) ** 2 + (yy - cy) ** 2 < rad ** 2] = 20
    return m


def image_lens():
    lens = OpticalSystem.from_records(P.double_gauss_12(seed=1), name="fixture image")
    stop = [i for i, s in enumerate(lens.surfaces) if s.is_stop][0]
    write_png(LENSES / "iris_star.png", star_mask())
    write_png(LENSES / "front_dust.png", dust_mask())
    lens.set_aperture_source(stop, "iris_star.png", float(np.float32(lens.surfaces[stop].semi_aperture * 1.02)))
    lens.set_aperture_source(0, "front_dust.png", float(np.float32(lens.surfaces[0].semi_aperture * 1.1)))
    return lens


def main():
    from oracle import ref
    from ghostlight_gb300 import load_lens
    from ghostlight_gb300.flare import spectral_table
    image_lens().save(LENSES / "fixture_image.lens")
    lens = load_lens(LENSES / "fixture_image.lens")
    lens.load_aperture_images()
    out, meta = {}, {}
    for i, s in enumerate(lens.surfaces):
        if s.aperture_shape == 2 and s.aperture_blades:
            img = lens.aperture_images[i]
            ref.register_image(s.aperture_blades, img.pixels, img.semi_diameter)
            out["pixels/%d" % i] = img.pixels
    surfs = lens.records()
    cal = ref.calibrate(surfs, 0.0)
    meta["calibration"] = cal
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    pairs, boosts = ref.filter_pairs(surfs, hw, hh, 1e-7)
    out["pairs"], out["boosts"] = pairs, boosts
    spec, _ = spectral_table(8)
    grid = ref.aperture_samples(surfs, 48, 0)
    src = np.array([[math.radians(7.0), math.radians(4.0), 1.0, 1.0, 1.0]], np.float32)
    out["image"] = ref.render_ghosts_cpu(surfs, pairs, boosts, src, grid, spec, hw, hh, 128, 128, 1000.0)
    out["source"] = src
    np.savez_compressed(HERE / "image_pins.npz", **out)
    (HERE / "image_meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print("wrote", len(out), "arrays;", len(pairs), "pairs")


if __name__ == "__main__":
    main()

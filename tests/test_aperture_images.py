"""Bitmap (IMAGE) apertures on the host: the lens loader and PNG decoding,
the calibration and the oracle's filter and image against the reference's own
outputs (tests/golden/image_pins.npz, made by make_image_golden.py), and the
oracle trace against the live reference where it is present."""
import json
import pathlib
import warnings

import numpy as np
import pytest

from ghostlight_gb300 import load_lens

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
LENS = GOLDEN / "lenses" / "fixture_image.lens"


@pytest.fixture(scope="module")
def pins():
    return np.load(GOLDEN / "image_pins.npz")


@pytest.fixture(scope="module")
def meta():
    return json.loads((GOLDEN / "image_meta.json").read_text())


def image_lens():
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lens = load_lens(LENS)
    lens.load_aperture_images()
    return lens


def register_oracle(lens):
    from oracle import oracle as O
    for i, s in enumerate(lens.surfaces):
        if s.aperture_shape == 2 and s.aperture_blades:
            img = lens.aperture_images[i]
            O.register_image(s.aperture_blades, img.pixels, img.semi_diameter)


def test_loader_declares_and_decodes(pins):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        lens = load_lens(LENS)
    imgs = [(i, im) for i, im in enumerate(lens.aperture_images) if im.source_path]
    assert [i for i, _ in imgs] == [0, 6] and lens.unsupported == []
    # declared, not decoded: the surfaces pass every ray until the pixels load
    assert all(lens.surfaces[i].aperture_shape == 2 and lens.surfaces[i].aperture_blades == 0 for i, _ in imgs)
    lens.load_aperture_images()
    for i, _ in imgs:
        img = lens.aperture_images[i]
        np.testing.assert_array_equal(img.pixels, pins["pixels/%d" % i])
        assert lens.surfaces[i].aperture_blades > 0
    assert set(np.unique(lens.aperture_images[6].pixels)) == {0.0, 1.0}


def test_png_decoder_filters():
    """Every PNG row filter (none, sub, up, average, Paeth) decodes exactly."""
    import struct
    import zlib
    from ghostlight_gb300.aperture_images import _png_decode
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (9, 11), dtype=np.uint8)
    rows = []
    prev = np.zeros(11, np.int32)
    for y in range(9):
        f = y % 5
        cur = img[y].astype(np.int32)
        enc = np.zeros(11, np.int32)
        for x in range(11):
            a = cur[x - 1] if x else 0
            b = prev[x]
            c = prev[x - 1] if x else 0
            p = [0, a, b, (a + b) >> 1, None][f]
            if f == 4:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            enc[x] = (cur[x] - p) & 255
        rows.append(bytes([f]) + enc.astype(np.uint8).tobytes())
        prev = cur

    def chunk(k, body):
        return struct.pack(">I", len(body)) + k + body + struct.pack(">I", zlib.crc32(k + body))
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 11, 9, 8, 0, 0, 0, 0)) + \
        chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b"")
    np.testing.assert_array_equal(_png_decode(png), img.astype(np.float32))


def test_calibration_bit_exact(meta):
    from ghostlight_gb300.calibration import calibrate_lens
    cal = calibrate_lens(image_lens())
    for k, v in meta["calibration"].items():
        assert np.float32(getattr(cal, k)) == np.float32(v), k


def test_oracle_filter_bit_exact(pins, meta):
    from oracle import oracle as O
    lens = image_lens()
    register_oracle(lens)
    cal = meta["calibration"]
    pairs, boosts = O.filter_pairs(lens.records(), cal["sensor_half_w"], cal["sensor_half_h"], 1e-7)
    np.testing.assert_array_equal(pairs, pins["pairs"])
    np.testing.assert_array_equal(boosts.view(np.uint32), pins["boosts"].view(np.uint32))


def test_oracle_image_matches_reference(pins, meta):
    from oracle import oracle as O
    from ghostlight_gb300.flare import spectral_table
    lens = image_lens()
    register_oracle(lens)
    surfs = lens.records()
    cal = meta["calibration"]
    spec, _ = spectral_table(8)
    grid = O.aperture_samples(surfs, 48, 0)
    img = O.render(surfs, pins["pairs"], pins["boosts"], pins["source"], [grid], spec, cal["sensor_half_w"],
                   cal["sensor_half_h"], 128, 128, 1000.0)
    ref = pins["image"]
    assert np.linalg.norm(ref) > 0
    assert np.linalg.norm(img - ref) / np.linalg.norm(ref) < 1e-3


def test_oracle_trace_matches_reference():
    from oracle import oracle as O
    ref = pytest.importorskip("oracle.ref")
    if not ref.available():
        pytest.skip("reference sources absent")
    lens = image_lens()
    register_oracle(lens)
    for i, s in enumerate(lens.surfaces):
        if s.aperture_shape == 2 and s.aperture_blades:
            img = lens.aperture_images[i]
            ref.register_image(s.aperture_blades, img.pixels, img.semi_diameter)
    surfs = lens.records()
    rng = np.random.default_rng(9)
    n = 4096
    R0 = surfs[0].semi_aperture
    ang = rng.uniform(-0.2, 0.2, (n, 2))
    rays = np.stack([rng.uniform(-1, 1, n) * R0, rng.uniform(-1, 1, n) * R0, np.full(n, surfs[0].z - 20.0),
                     np.sin(ang[:, 0]), np.sin(ang[:, 1]), np.ones(n), rng.uniform(400, 700, n)], 1)
    rays[:, 3:6] /= np.linalg.norm(rays[:, 3:6], axis=1, keepdims=True)
    rays = rays.astype(np.float32)
    for a, b in ((-1, -1), (2, 5), (1, 8)):
        want = ref.trace(surfs, a, b, rays)
        got = O.trace(surfs, a, b, rays, fp64=False)
        np.testing.assert_array_equal(got[:, 4], want[:, 4])
        ok = want[:, 4] == 0
        np.testing.assert_array_equal(got[ok, :4].astype(np.float32), want[ok, :4])
    # the bitmaps decide some rays: not loaded, the same lens passes more
    import ctypes
    from ghostlight_gb300._abi import gl_surface
    plain = []
    for s in surfs:
        c = gl_surface()
        ctypes.pointer(c)[0] = s
        if c.aperture_shape == 2:
            c.aperture_blades = 0
        plain.append(c)
    n_img = int((ref.trace(surfs, -1, -1, rays)[:, 4] == 0).sum())
    n_plain = int((ref.trace(plain, -1, -1, rays)[:, 4] == 0).sum())
    assert n_plain > n_img > 0

"""Bitmap (IMAGE) apertures: ApertureImage and the image decoding of
``OpticalSystem.load_aperture_images``.

The reference keeps an ``ApertureImage`` (pixels, size, boundary
semi-diameter, source path) beside each surface
(``OpticalSystem::aperture_images``, ghostlight/src/optical_system.h:262-269,
bound at bindings/python/src/bind_geometry.cpp:311-360) and tests a ray against
it with ``sample_aperture_image`` (trace.cpp:31-48: the nearest pixel,
open above 0.5).  Here the pixels are an immutable entry of the native store
(``gl_aperture_image_create``); the surface record names it in
``aperture_blades`` (0: not loaded, every ray inside the clear aperture
passes, as in the reference before decoding).  The traces sample the
nearest pixel on host and device alike.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import zlib
from typing import Optional

import numpy as np

_APERTURE_IMAGE = 2


class ApertureImage:
    """One surface's bitmap: ``pixels`` (H, W) float32 luminance in [0, 1],
    ``semi_diameter`` (mm, the world radius of the image boundary) and the
    ``source_path`` a lens file names."""

    def __init__(self, pixels=None, semi_diameter: float = 0.0, source_path: str = ""):
        self.pixels = np.zeros((0, 0), np.float32) if pixels is None else np.asarray(pixels, np.float32)
        self.semi_diameter = float(semi_diameter)
        self.source_path = source_path

    @property
    def width(self) -> int:
        return int(self.pixels.shape[1]) if self.pixels.ndim == 2 else 0

    @property
    def height(self) -> int:
        return int(self.pixels.shape[0]) if self.pixels.ndim == 2 else 0

    def __repr__(self):
        return "ApertureImage(width=%d, height=%d, semi_diameter=%g, source_path=%r)" % (
            self.width, self.height, self.semi_diameter, self.source_path)


def create_image(pixels, semi_diameter: float) -> int:
    """Store a bitmap; returns its id (the same pixels give the same id)."""
    from . import _native
    px = np.ascontiguousarray(pixels, np.float32)
    if px.ndim != 2 or px.size == 0:
        raise ValueError("pixels must be a non-empty 2-D array (height, width)")
    if not np.isfinite(semi_diameter) or semi_diameter < 0:
        raise ValueError("semi_diameter must be finite and non-negative")
    out = C.c_int()
    _native.check(_native.load().gl_aperture_image_create(px.shape[1], px.shape[0],
                                                          px.ctypes.data_as(C.POINTER(C.c_float)),
                                                          float(semi_diameter), C.byref(out)),
                  "aperture_image_create")
    return int(out.value)


def read_image(image_id: int) -> ApertureImage:
    from . import coatings as K
    info = K.table_info(image_id)
    if info["model"] != 100:
        raise ValueError("store entry %d is not an aperture image" % image_id)
    _, _, _, r, _, _ = K.read_table(image_id)
    return ApertureImage(np.asarray(r, np.float32).reshape(info["n1"], info["n0"]), info["angle_ref_ior"])


# ---- image decoding -------------------------------------------------------
def _png_decode(data: bytes) -> np.ndarray:
    """8-bit, non-interlaced PNG (grey, grey + alpha, RGB, RGBA, palette) to
    float luminance in [0, 255] (RGB weighted 0.299 / 0.587 / 0.114)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, plte = 8, [], None
    w = h = depth = ctype = interlace = None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if depth != 8 or interlace:
        raise ValueError("PNG: only 8-bit non-interlaced images are decoded here")
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(h, 1 + w * ch)
    out = np.zeros((h, w * ch), np.int32)
    prev = np.zeros(w * ch, np.int32)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        cur = np.zeros(w * ch, np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            for x in range(w * ch):
                a = cur[x - ch] if x >= ch else 0
                b = prev[x]
                c = prev[x - ch] if x >= ch else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur
    px = out.reshape(h, w, ch).astype(np.float32)
    if ctype == 3:
        px = plte[out.reshape(h, w)].astype(np.float32)
        ch = 3
    if ch >= 3:
        return px[..., 0] * np.float32(0.299) + px[..., 1] * np.float32(0.587) + px[..., 2] * np.float32(0.114)
    return px[..., 0]


def decode_image(path: str) -> np.ndarray:
    """Single-channel float32 in [0, 1] (optical_system.py:178-225: luminance,
    scaled by 1/255 when the peak is above 1.5).  Pillow decodes when it is
    installed; otherwise 8-bit PNGs are decoded here."""
    try:
        from PIL import Image
        with Image.open(path) as im:
            arr = np.asarray(im.convert("F"), dtype=np.float32)
    except ImportError:
        with open(path, "rb") as fh:
            arr = _png_decode(fh.read()).astype(np.float32)
    if arr.size and float(arr.max()) > 1.5:
        arr = arr / np.float32(255.0)
    return arr.astype(np.float32)


def load_aperture_images(lens, root_dir: Optional[str] = None) -> None:
    """Decode the bitmap of every IMAGE surface whose pixels are not loaded
    yet (source path resolved against root_dir, or the lens file's folder)."""
    base = root_dir
    if base is None and getattr(lens, "source_path", None):
        base = os.path.dirname(os.fspath(lens.source_path))
    for i, s in enumerate(lens.surfaces):
        if s.aperture_shape != _APERTURE_IMAGE:
            continue
        img = lens.aperture_images[i]
        if img.pixels.size > 0 or not img.source_path:
            continue
        path = img.source_path
        if base is not None and not os.path.isabs(path):
            path = os.path.join(base, path)
        lens.set_aperture_image(i, decode_image(path), img.semi_diameter)

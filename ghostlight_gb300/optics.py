"""Lens data model mirroring the reference bindings (bind_geometry.cpp,
bind_trace.cpp): Surface, Coating, OpticalSystem, Ray, Vec3f, TraceResult
and the enums, with the same attribute names.  A Surface is a view of one
plain-C ``gl_surface`` record, so a lens is handed to the C-ABI as one
contiguous array without conversion.
"""
from __future__ import annotations

import ctypes as C
import enum
from typing import List

import numpy as np

from ._abi import default_surface, gl_surface


class SurfaceForm(enum.IntEnum):
    SPHERE = 0
    ASPHERE = 1
    CYLINDRICAL = 2


class CylinderAxis(enum.IntEnum):
    X = 0
    Y = 1


class ApertureShape(enum.IntEnum):
    CIRCLE = 0
    POLYGON = 1
    IMAGE = 2


class DispersionModel(enum.IntEnum):
    AIR = 0
    ABBE = 1
    SELLMEIER = 2


class CoatingModel(enum.IntEnum):
    SIMPLE = 0
    SPECTRAL = 1
    ANGULAR = 2
    SPECTRAL_ANGULAR = 3
    ATTENUATOR_GAUSS = 4
    ARTIST = 5


class TraceStatus(enum.IntEnum):
    OK = 0
    VIGNETTED = 1
    TIR = 2
    MISSED_SURFACE = 3
    INVALID_INPUT = 4


class Vec3f:
    __slots__ = ("x", "y", "z")

    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.x, self.y, self.z = float(x), float(y), float(z)

    def __iter__(self):
        return iter((self.x, self.y, self.z))

    def __repr__(self):
        return "Vec3f(%g, %g, %g)" % (self.x, self.y, self.z)


class Ray:
    """Ray (ray.h): origin, normalised direction, wavelength in nm."""

    def __init__(self, origin=None, dir=None, lambda_=587.56):
        self.origin = origin if origin is not None else Vec3f()
        self.dir = dir if dir is not None else Vec3f(0.0, 0.0, 1.0)
        self.lambda_ = float(lambda_)

    # `lambda` is a Python keyword; the reference binding exposes it as .lambda_
    @property
    def wavelength(self):
        return self.lambda_


class TraceResult:
    __slots__ = ("position", "weight", "status")

    def __init__(self, position, weight, status):
        self.position, self.weight, self.status = position, float(weight), TraceStatus(int(status))

    def __repr__(self):
        return "TraceResult(status=%d, weight=%g)" % (int(self.status), self.weight)


class Coating:
    """View of the coating fields of one surface record (optical_system.h:109-147)."""

    _MAP = {"ar_layers": "ar_layers", "tint_r": "tint_r", "tint_g": "tint_g", "tint_b": "tint_b",
            "tint_strength": "tint_strength", "gauss_sigma": "gauss_sigma",
            "gauss_background": "gauss_background", "gauss_peak": "gauss_peak",
            "gauss_decenter_x": "gauss_decenter_x", "gauss_decenter_y": "gauss_decenter_y"}

    def __init__(self, rec: gl_surface):
        object.__setattr__(self, "_rec", rec)

    @property
    def model(self):
        return CoatingModel(self._rec.coating_model)

    @model.setter
    def model(self, v):
        self._rec.coating_model = int(v)

    # table attributes (bind_geometry.cpp:153-164) live with the table the
    # record names; reading them on a coating without a table gives the
    # defaults
    _TABLE_ATTRS = ("angle_ref_ior", "out_of_range_discard", "table_count", "sa_n_wavelengths", "sa_n_angles")

    def _table(self):
        if self._rec.coating_model in (1, 2, 3) and self._rec.ar_layers:
            from .coatings import table_info
            return table_info(self._rec.ar_layers)
        return None

    def __getattr__(self, k):
        if k in Coating._MAP:
            return getattr(self._rec, Coating._MAP[k])
        if k in Coating._TABLE_ATTRS:
            t = self._table()
            if k == "angle_ref_ior":
                return t["angle_ref_ior"] if t else 1.0
            if k == "out_of_range_discard":
                return t["out_of_range_discard"] if t else False
            if t is None:
                return 0
            if k == "table_count":
                return t["n0"] if t["model"] in (1, 2) else 0
            return (t["n0"] if k == "sa_n_wavelengths" else t["n1"]) if t["model"] == 3 else 0
        raise AttributeError(k)

    def __setattr__(self, k, v):
        if k == "model":
            self._rec.coating_model = int(v)
        elif k in Coating._MAP:
            setattr(self._rec, Coating._MAP[k], v)
        elif k in ("angle_ref_ior", "out_of_range_discard"):
            # tables are immutable: the record moves to the table with the new attribute
            if self._table() is not None:
                from .coatings import create_table, read_table
                model, a0, a1, r, ref, disc = read_table(self._rec.ar_layers)
                if k == "angle_ref_ior":
                    ref = float(v)
                else:
                    disc = bool(v)
                self._rec.ar_layers = create_table(model, a0, r, a1 if len(a1) else None, ref, disc)
        else:
            raise AttributeError("Coating has no field %r" % k)


class Surface:
    """One sequential surface (optical_system.h:157-249)."""

    def __init__(self, rec: gl_surface | None = None):
        object.__setattr__(self, "_rec", rec if rec is not None else default_surface())

    @property
    def coating(self) -> Coating:
        return Coating(self._rec)

    @property
    def record(self) -> gl_surface:
        return self._rec

    def ior_at(self, lambda_nm: float) -> float:
        """Surface::ior_at (optical_system.h:230-235), float32 arithmetic."""
        f = np.float32
        r = self._rec
        lam = f(lambda_nm)
        if r.disp_model == DispersionModel.SELLMEIER:
            l = lam * f(1e-3)
            l2 = l * l
            n2 = f(1.0)
            for k in range(3):
                n2 = f(n2 + f(r.sellmeier_B[k]) * l2 / (l2 - f(r.sellmeier_C[k])))
            return float(np.sqrt(n2)) if n2 > 0 else 1.0
        nd, vd = f(r.ior), f(r.abbe_v)
        if vd < f(0.1) or nd <= f(1.0001):
            return float(nd)
        lF, lC, ld = f(486.13), f(656.27), f(587.56)
        dn = (nd - f(1.0)) / vd
        B = dn / (f(1.0) / (lF * lF) - f(1.0) / (lC * lC))
        A = nd - B * (f(1.0) / (ld * ld))
        return float(A + B / (lam * lam))

    def __getattr__(self, k):
        return getattr(object.__getattribute__(self, "_rec"), k)

    def __setattr__(self, k, v):
        rec = object.__getattribute__(self, "_rec")
        if not hasattr(rec, k):
            raise AttributeError("Surface has no field %r" % k)
        if k in ("is_stop", "is_active"):
            v = int(bool(v))
        elif isinstance(v, enum.IntEnum):
            v = int(v)
        setattr(rec, k, v)

    def copy(self) -> "Surface":
        r = gl_surface()
        C.pointer(r)[0] = self._rec
        return Surface(r)


class OpticalSystem:
    """Flat sequential lens (optical_system.h:305-416): sensor at z = 0,
    light travelling in +z."""

    def __init__(self, surfaces=None, name: str = "", focal_length: float = 0.0):
        self.name = name
        self.focal_length = float(focal_length)
        self.surfaces: List[Surface] = []
        for s in surfaces or []:
            self.surfaces.append(s if isinstance(s, Surface) else Surface(s))
        self._calib = None
        self._calib_key = None
        self.unsupported = []           # (surface index, feature) a lens file used that this library lacks
        self.source_path = None

    @classmethod
    def load(cls, path) -> "OpticalSystem":
        """Load a ``ghostlight-optical`` lens file (optical_system.py:90,
        OpticalSystem::load at optical_system.cpp:1342)."""
        from .lensfile import load_lens
        return load_lens(path)

    def save(self, path) -> None:
        """Write this lens as a ``ghostlight-optical`` file (optical_system.py:252)."""
        from .lensfile import save_lens
        save_lens(self, path, self.name)

    @classmethod
    def from_records(cls, recs, name: str = "", focal_length: float = 0.0):
        out = cls(name=name, focal_length=focal_length)
        for r in recs:
            rr = gl_surface()
            C.pointer(rr)[0] = r
            out.surfaces.append(Surface(rr))
        return out

    def num_surfaces(self) -> int:
        return len(self.surfaces)

    def to_array(self):
        arr = (gl_surface * len(self.surfaces))()
        for i, s in enumerate(self.surfaces):
            arr[i] = s.record
        return arr

    def records(self):
        return [s.record for s in self.surfaces]

    def state_key(self) -> bytes:
        return bytes(self.to_array())

    def finalize(self) -> bool:
        """OpticalSystem::finalize (optical_system.cpp:1425)."""
        if not self.surfaces:
            return False
        from . import _native
        arr = self.to_array()
        _native.check(_native.load().gl_finalize_z(arr, len(arr)), "finalize")
        for i, s in enumerate(self.surfaces):
            s.z = arr[i].z
        return True

    def ior_before(self, idx: int, lambda_nm: float | None = None) -> float:
        """OpticalSystem::ior_before (optical_system.h:385-402)."""
        idx = min(idx, len(self.surfaces))
        for k in range(idx - 1, -1, -1):
            if self.surfaces[k].is_active:
                s = self.surfaces[k]
                return float(np.float32(s.ior)) if lambda_nm is None else s.ior_at(lambda_nm)
        return 1.0

    # ---- bitmap apertures (bind_geometry.cpp:311-384, optical_system.py:178) --
    def set_aperture_source(self, index: int, source_path: str, semi_diameter: float) -> None:
        """Declare surface ``index`` a bitmap aperture read from
        ``source_path`` (decoded by load_aperture_images); until then it
        passes every ray inside its clear aperture."""
        i = self._surface_index(index)
        paths = self.__dict__.setdefault("_aperture_sources", {})
        paths[i] = (str(source_path), float(semi_diameter))
        self.surfaces[i].aperture_shape = ApertureShape.IMAGE
        self.surfaces[i].aperture_blades = 0

    def set_aperture_image(self, index: int, pixels, semi_diameter: float | None = None) -> None:
        """Surface ``index`` becomes a bitmap aperture: ``pixels`` (H, W)
        luminance in [0, 1] (open above 0.5, nearest pixel), the image
        spanning +-semi_diameter mm (default: the declared one)."""
        from .aperture_images import create_image
        i = self._surface_index(index)
        paths = self.__dict__.setdefault("_aperture_sources", {})
        if semi_diameter is None:
            semi_diameter = paths.get(i, ("", 0.0))[1]
        if not semi_diameter > 0:
            raise ValueError("set_aperture_image: semi_diameter must be positive")
        tid = create_image(pixels, float(semi_diameter))
        paths[i] = (paths.get(i, ("", 0.0))[0], float(semi_diameter))
        self.surfaces[i].aperture_shape = ApertureShape.IMAGE
        self.surfaces[i].aperture_blades = tid

    @property
    def aperture_images(self):
        """ApertureImage per surface (empty pixels for surfaces without a
        loaded bitmap).  A snapshot: change a bitmap with set_aperture_image."""
        from .aperture_images import ApertureImage, read_image
        paths = self.__dict__.get("_aperture_sources", {})
        out = []
        for i, s in enumerate(self.surfaces):
            src, semi = paths.get(i, ("", 0.0))
            if s.aperture_shape == ApertureShape.IMAGE and s.aperture_blades:
                img = read_image(s.aperture_blades)
                img.source_path = src
                out.append(img)
            else:
                out.append(ApertureImage(None, semi if s.aperture_shape == ApertureShape.IMAGE else 0.0, src))
        return out

    def load_aperture_images(self, *, root_dir: str | None = None) -> None:
        """Decode the bitmaps of the IMAGE surfaces (optical_system.py:178-225)."""
        from .aperture_images import load_aperture_images
        load_aperture_images(self, root_dir)

    # ---- coating tables (bind_geometry.cpp:412-627) ------------------------
    def _surface_index(self, i: int) -> int:
        if i < 0 or i >= len(self.surfaces):
            raise IndexError("surface index out of range")
        return i

    def set_coating_spectral_table(self, index: int, data, out_of_range_discard: bool = False) -> None:
        """R(lambda) from an (N, 2) array of (lambda_nm, r), sorted by key."""
        from . import coatings as K
        d = K.sort_1d(data)
        rec = self.surfaces[self._surface_index(index)].record
        tid = K.create_table(K.SPECTRAL, d[:, 0], d[:, 1], out_of_range_discard=out_of_range_discard)
        K.reset_coating(rec, K.SPECTRAL, tid)

    def set_coating_angular_table(self, index: int, data, angle_ref_ior: float = 1.0,
                                  out_of_range_discard: bool = False) -> None:
        """R(angle) from an (N, 2) array of (angle_deg, r) measured in a
        medium of index ``angle_ref_ior``."""
        from . import coatings as K
        d = K.sort_1d(data)
        rec = self.surfaces[self._surface_index(index)].record
        tid = K.create_table(K.ANGULAR, d[:, 0], d[:, 1], angle_ref_ior=angle_ref_ior,
                             out_of_range_discard=out_of_range_discard)
        K.reset_coating(rec, K.ANGULAR, tid)

    def get_coating_table(self, index: int):
        """The (N, 2) (key, r) table of a SPECTRAL / ANGULAR surface; (0, 2)
        otherwise."""
        from . import coatings as K
        rec = self.surfaces[self._surface_index(index)].record
        if rec.coating_model in (K.SPECTRAL, K.ANGULAR) and rec.ar_layers:
            _, a0, _, r, _, _ = K.read_table(rec.ar_layers)
            return np.stack([a0, r], 1)
        return np.zeros((0, 2), np.float32)

    def set_coating_sa_table(self, index: int, wavelengths_nm, angles_deg, r, angle_ref_ior: float = 1.0,
                             out_of_range_discard: bool = False) -> None:
        """R(lambda, angle) on ascending axes; r is (n_wavelengths, n_angles)."""
        from . import coatings as K
        rec = self.surfaces[self._surface_index(index)].record
        wl = np.asarray(wavelengths_nm, np.float32)
        ang = np.asarray(angles_deg, np.float32)
        rr = np.asarray(r, np.float32)
        if wl.ndim != 1 or ang.ndim != 1 or wl.size < 1 or ang.size < 1:
            raise ValueError("wavelengths and angles must be 1-D non-empty arrays")
        if rr.ndim != 2 or rr.shape != (wl.size, ang.size):
            raise ValueError("r must be an (n_wavelengths, n_angles) array")
        if np.any(np.diff(wl) < 0) or np.any(np.diff(ang) < 0):
            raise ValueError("wavelengths and angles must be sorted ascending")
        tid = K.create_table(K.SPECTRAL_ANGULAR, wl, rr, axis1=ang, angle_ref_ior=angle_ref_ior,
                             out_of_range_discard=out_of_range_discard)
        K.reset_coating(rec, K.SPECTRAL_ANGULAR, tid)

    def get_coating_sa_table(self, index: int):
        """(wavelengths_nm, angles_deg, r) of a SPECTRAL_ANGULAR surface;
        empty arrays otherwise."""
        from . import coatings as K
        rec = self.surfaces[self._surface_index(index)].record
        if rec.coating_model == K.SPECTRAL_ANGULAR and rec.ar_layers:
            _, a0, a1, r, _, _ = K.read_table(rec.ar_layers)
            return a0, a1, r
        return np.zeros(0, np.float32), np.zeros(0, np.float32), np.zeros((0, 0), np.float32)

    def set_coating_layers(self, index: int, layers) -> None:
        """A thin-film stack (dicts of material, thickness_nm, nk_table (K, 3)
        of lambda_um, n, k), baked against the lens's current glasses."""
        from . import coatings as K
        i = self._surface_index(index)
        try:
            tid = K.bake_layers(self.records(), i, layers)
        except Exception as e:
            raise ValueError("set_coating_layers: %s" % e) from None
        K.reset_coating(self.surfaces[i].record, K.SPECTRAL_ANGULAR, tid)

    def get_coating_layers(self, index: int):
        from . import coatings as K
        rec = self.surfaces[self._surface_index(index)].record
        if rec.coating_model == K.SPECTRAL_ANGULAR and rec.ar_layers:
            return [dict(d, nk_table=d["nk_table"].copy()) for d in (K.layers_of(rec.ar_layers) or [])]
        return []

    def clear_coating(self, index: int) -> None:
        """Uncoated SIMPLE (bare Fresnel)."""
        from . import coatings as K
        K.reset_coating(self.surfaces[self._surface_index(index)].record)

    # Cached helpers mirroring ghostlight/bindings/python/ghostlight/optical_system.py
    def calibration(self, *, d_line_nm: float = 587.56, precision: str = "fp32"):
        from .calibration import calibrate_lens
        key = (self.state_key(), d_line_nm, precision)
        if self._calib is None or self._calib_key != key:
            self._calib = calibrate_lens(self, d_line_nm, precision=precision)
            self._calib_key = key
        return self._calib

    def ghost_pairs(self):
        from .flare import enumerate_ghost_pairs
        return enumerate_ghost_pairs(self)

    def filter_ghosts(self, config, *, calib=None):
        from .flare import filter_ghost_pairs
        cal = calib if calib is not None else self.calibration()
        return filter_ghost_pairs(self, cal.sensor_half_w, cal.sensor_half_h, config)

    def render_point_flare(self, width, height, config, *, calib=None):
        from .flare import render_point_flare
        cal = calib if calib is not None else self.calibration()
        return render_point_flare(width, height, self, cal, config)

    def render_source_flare(self, offsets, width, height, config, *, calib=None):
        from .flare import render_source_flare
        cal = calib if calib is not None else self.calibration()
        return render_source_flare(offsets, width, height, self, cal, config)

    def __repr__(self):
        return "OpticalSystem(name=%r, surfaces=%d)" % (self.name, len(self.surfaces))

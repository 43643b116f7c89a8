"""Reader of the ``ghostlight-optical`` lens file format (``.lens``, UTF-8 JSON).

Restates the reference's C++ loader — ``OpticalSystem::load``
(ghostlight/src/optical_system.cpp:1342-1414) with ``flatten_optical_system``
(:1048-1240), ``flatten_element`` (:801-912), ``parse_form`` (:693-741),
``extract_coating`` (:351-527), ``apply_aperture_modifiers`` (:572-689),
``parse_pivots`` / ``apply_pivot_to_transform`` (:949-1045) and the glass
catalogue (:81-151) — so a file loads into the same flat surface table, field
for field: every float is computed in float32 in the reference's operation
order (numpy float32 scalars; the element rotation comes from the C library's
cosf/sinf through ``gl_euler_rotation``).  Files the reference rejects raise
``RuntimeError("OpticalSystem.load() failed: ...")`` (bind_geometry.cpp:386-389);
where the reference only warns, this reader warns too.

Table-backed coatings (``spectral``, ``angular``, ``spectral_angular``) go
to the coating store (``ghostlight_gb300.coatings``), the surface record
naming its table; thin-film stacks (``layers``) are baked after flattening,
as the reference does.  Bitmap (``image``) apertures load as IMAGE surfaces
with their path and semi-diameter recorded; the pixels are decoded by
``OpticalSystem.load_aperture_images`` as in the reference.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import warnings
from typing import Dict, List, Tuple

import numpy as np

from ._abi import default_surface, gl_surface

LENS_FORMAT_MAJOR = 1
LENS_FORMAT_MINOR = 0

f32 = np.float32
_PI = f32(3.14159265358979323846)
_DEG = f32(_PI / f32(180.0))

# enum values of the surface record (optical_system.h)
_FORM = {"sphere": 0, "asphere": 1, "cylindrical": 2}
_DISP_AIR, _DISP_ABBE, _DISP_SELLMEIER = 0, 1, 2
_APERTURE_CIRCLE, _APERTURE_POLYGON, _APERTURE_IMAGE = 0, 1, 2
_COATING_SIMPLE, _COATING_ATTENUATOR_GAUSS, _COATING_ARTIST = 0, 4, 5
_MAX_ASPHERE_TERMS = 8


def lens_format_version() -> Tuple[int, int]:
    """(major, minor) of the lens format this reader understands."""
    return LENS_FORMAT_MAJOR, LENS_FORMAT_MINOR


class LensFileError(RuntimeError):
    pass


def _fail(path, msg):
    raise LensFileError("OpticalSystem.load() failed: %s: %s" % (path, msg))


def _num(v) -> np.float32:
    """A JSON number read as a float (nlohmann get<float>: the parsed double,
    rounded to float)."""
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise TypeError("expected a number, got %r" % (v,))
    return f32(v)


def _value(obj, key, default):
    """nlohmann json::value(key, default) for a number."""
    if isinstance(obj, dict) and key in obj:
        return _num(obj[key])
    return f32(default)


def _clamp01(v):
    return f32(0.0) if v < f32(0.0) else (f32(1.0) if v > f32(1.0) else v)


# ---- float32 3x3 helpers (optical_system.cpp:201-221) ---------------------
def _rotation(tx, ty, rz):
    from . import _native
    out = (C.c_float * 9)()
    _native.check(_native.load().gl_euler_rotation(float(tx), float(ty), float(rz), out), "euler_rotation")
    return [f32(v) for v in out]


def _mat_vec(A, b):
    return [A[0] * b[0] + A[1] * b[1] + A[2] * b[2],
            A[3] * b[0] + A[4] * b[1] + A[5] * b[2],
            A[6] * b[0] + A[7] * b[1] + A[8] * b[2]]


def _mat_mat(A, B):
    out = []
    for i in range(3):
        for j in range(3):
            s = f32(0.0)
            for k in range(3):
                s = s + A[i * 3 + k] * B[k * 3 + j]
            out.append(s)
    return out


class _Transform:
    __slots__ = ("pos", "rot", "piv")

    def __init__(self):
        self.pos = [f32(0.0)] * 3
        self.rot = [f32(1.0), f32(0.0), f32(0.0), f32(0.0), f32(1.0), f32(0.0), f32(0.0), f32(0.0), f32(1.0)]
        self.piv = [f32(0.0)] * 3


def _parse_transform(jx) -> _Transform:
    """parse_transform (optical_system.cpp:253-300)."""
    t = _Transform()
    if not isinstance(jx, dict):
        return t
    tilt_x = tilt_y = roll = f32(0.0)
    pivot = [f32(0.0)] * 3
    p = jx.get("position")
    if isinstance(p, dict):
        t.pos = [_value(p, k, 0.0) for k in ("x", "y", "z")]
    r = jx.get("rotation")
    if isinstance(r, dict):
        tilt_x, tilt_y, roll = (_value(r, k, 0.0) for k in ("tilt_x", "tilt_y", "roll"))
    v = jx.get("pivot")
    if isinstance(v, dict):
        pivot = [_value(v, k, 0.0) for k in ("x", "y", "z")]
    t.rot = _rotation(tilt_x, tilt_y, roll)
    if any(c != f32(0.0) for c in pivot):
        rp = _mat_vec(t.rot, pivot)
        t.piv = [pivot[i] - rp[i] for i in range(3)]
    return t


# ---- glass catalogue (optical_system.cpp:69-151) ---------------------------
def _sellmeier_n(B, Cc, lam_nm):
    """sellmeier_n (fresnel.h:53-63) in float32."""
    l = f32(lam_nm) * f32(1e-3)
    l2 = l * l
    n2 = f32(1.0)
    for k in range(3):
        n2 = n2 + B[k] * l2 / (l2 - Cc[k])
    return np.sqrt(n2) if n2 > f32(0.0) else f32(1.0)


def _sellmeier_to_abbe(B, Cc):
    n_d = _sellmeier_n(B, Cc, 587.56)
    n_F = _sellmeier_n(B, Cc, 486.13)
    n_C = _sellmeier_n(B, Cc, 656.27)
    V_d = (n_d - f32(1.0)) / (n_F - n_C) if (n_F - n_C) > f32(1e-9) else f32(0.0)
    return n_d, V_d


def _parse_catalogue(j, path) -> Dict[str, dict]:
    if not isinstance(j, dict):
        _fail(path, "glass_catalogue must be an object")
    out = {}
    for key, je in j.items():
        jd = je.get("dispersion") if isinstance(je, dict) else None
        if not isinstance(jd, dict):
            _fail(path, "glass '%s' missing dispersion block" % key)
        model = jd.get("model", "")
        if model == "sellmeier":
            B, Cc = jd.get("B"), jd.get("C")
            if not (isinstance(B, list) and isinstance(Cc, list) and len(B) == 3 and len(Cc) == 3):
                _fail(path, "glass '%s' sellmeier needs B[3] and C[3]" % key)
            B = [_num(x) for x in B]
            Cc = [_num(x) for x in Cc]
            n_d, V_d = _sellmeier_to_abbe(B, Cc)
            out[key] = dict(model=_DISP_SELLMEIER, n_d=n_d, V_d=V_d, B=B, C=Cc)
        elif model == "abbe":
            if "nd" not in jd or "Vd" not in jd:
                _fail(path, "glass '%s' abbe needs nd + Vd" % key)
            out[key] = dict(model=_DISP_ABBE, n_d=_num(jd["nd"]), V_d=_num(jd["Vd"]),
                            B=[f32(0.0)] * 3, C=[f32(0.0)] * 3)
        else:
            _fail(path, "glass '%s' unknown dispersion model '%s'" % (key, model))
    return out


def _apply_air(s: gl_surface):
    s.ior, s.abbe_v, s.disp_model = 1.0, 0.0, _DISP_AIR
    for k in range(3):
        s.sellmeier_B[k] = 0.0
        s.sellmeier_C[k] = 0.0


def _apply_glass(name, catalogue, s: gl_surface, path):
    if not name or name in ("air", "AIR"):
        _apply_air(s)
        return
    g = catalogue.get(name)
    if g is None:
        _fail(path, "glass '%s' not present in glass_catalogue." % name)
    s.ior, s.abbe_v, s.disp_model = float(g["n_d"]), float(g["V_d"]), g["model"]
    for k in range(3):
        s.sellmeier_B[k] = float(g["B"][k])
        s.sellmeier_C[k] = float(g["C"][k])


# ---- surface modifiers -----------------------------------------------------
def _extract_coating(mods, s: gl_surface, path, unsupported: List[str]):
    """extract_coating (optical_system.cpp:351-527): the last coating modifier
    wins; the default is SIMPLE with no AR layers (bare Fresnel).  Tables go
    to the coating store (the record names them in ar_layers); a ``layers``
    stack is returned for the bake after flattening, when the glasses are
    final (optical_system.cpp:1407-1415)."""
    from . import coatings as K
    coat = dict(model=_COATING_SIMPLE, ar_layers=0, tint=[f32(1.0)] * 3, strength=f32(0.04),
                gauss=[f32(0.0)] * 5)
    layers = None
    if isinstance(mods, list):
        for m in mods:
            if not isinstance(m, dict) or m.get("type", "") != "coating":
                continue
            model = m.get("model", "")
            if not model:
                _fail(path, "coating modifier has no 'model' field.")
            fresh = dict(model=_COATING_SIMPLE, ar_layers=0, tint=[f32(1.0)] * 3, strength=f32(0.04),
                         gauss=[f32(0.0)] * 5)
            discard = m.get("out_of_range", "clamp") == "discard"
            if model == "layers":
                jls = m.get("layers")
                if not isinstance(jls, list):
                    _fail(path, "coating model 'layers' has no 'layers' array.")
                specs = []
                for jl in jls:
                    if not isinstance(jl, dict):
                        specs = None
                        break
                    nk = [(_num(e["lambda_um"]), _value(e, "n", 1.0), _value(e, "k", 0.0))
                          for e in (jl.get("nk_table") or []) if isinstance(e, dict) and "lambda_um" in e] \
                        if isinstance(jl.get("nk_table"), list) else []
                    th = _value(jl, "thickness_nm", 0.0)
                    if not nk or th <= f32(0.0):
                        specs = None
                        break
                    specs.append({"material": str(jl.get("material", "")), "thickness_nm": th,
                                  "nk_table": np.array(nk, np.float32)})
                if not specs:
                    _fail(path, "coating 'layers' stack is empty or has a layer with no nk_table / "
                                "non-positive thickness.")
                coat, layers = fresh, specs
            elif model == "simple":
                fresh["ar_layers"] = int(m.get("ar_layers", 0))
                coat, layers = fresh, None
            elif model == "artist":
                t = m.get("tint")
                if isinstance(t, list) and len(t) == 3:
                    fresh["tint"] = [_clamp01(_num(x)) for x in t]
                fresh["strength"] = _clamp01(_value(m, "strength", 0.04))
                fresh["model"] = _COATING_ARTIST
                coat, layers = fresh, None
            elif model in ("spectral", "angular"):
                key = "lambda_nm" if model == "spectral" else "angle_deg"
                rows = [(_num(e[key]), _clamp01(_num(e["r"]))) for e in m["data"]
                        if isinstance(e, dict) and key in e and "r" in e] if isinstance(m.get("data"), list) else []
                if not rows:
                    warnings.warn("%s: coating modifier has an empty/invalid 'data' table; treating as "
                                  "uncoated." % path)
                    continue
                d = K.sort_1d(rows)
                kind = K.SPECTRAL if model == "spectral" else K.ANGULAR
                ref = _value(m, "angle_ref_ior", 1.0) if model == "angular" else f32(1.0)
                fresh["model"] = kind
                fresh["ar_layers"] = K.create_table(kind, d[:, 0], d[:, 1], angle_ref_ior=float(ref),
                                                    out_of_range_discard=discard)
                coat, layers = fresh, None
            elif model == "spectral_angular":
                wl = [_num(v) for v in (m.get("wavelengths_nm") or [])]
                ang = [_num(v) for v in (m.get("angles_deg") or [])]
                r = [_clamp01(_num(v)) for row in (m.get("r") or []) if isinstance(row, list) for v in row]
                if (not wl or not ang or len(r) != len(wl) * len(ang) or wl != sorted(wl)
                        or ang != sorted(ang)):
                    warnings.warn("%s: spectral_angular coating has inconsistent or unsorted "
                                  "wavelengths/angles/r arrays; treating as uncoated." % path)
                    continue
                fresh["model"] = K.SPECTRAL_ANGULAR
                fresh["ar_layers"] = K.create_table(K.SPECTRAL_ANGULAR, wl, np.array(r, np.float32), axis1=ang,
                                                    angle_ref_ior=float(_value(m, "angle_ref_ior", 1.0)),
                                                    out_of_range_discard=discard)
                coat, layers = fresh, None
            elif model == "attenuator_gaussian":
                fresh["model"] = _COATING_ATTENUATOR_GAUSS
                fresh["gauss"] = [_value(m, k, 0.0) for k in ("sigma", "attenuation_background",
                                                            "attenuation_peak", "decenter_x", "decenter_y")]
                coat, layers = fresh, None
            else:
                _fail(path, "coating model '%s' is not recognised." % model)
    s.coating_model = coat["model"]
    s.ar_layers = coat["ar_layers"]
    s.tint_r, s.tint_g, s.tint_b = (float(v) for v in coat["tint"])
    s.tint_strength = float(coat["strength"])
    (s.gauss_sigma, s.gauss_background, s.gauss_peak, s.gauss_decenter_x,
     s.gauss_decenter_y) = (float(v) for v in coat["gauss"])
    return layers


def _set_circular(s: gl_surface, aspect):
    s.aperture_shape = _APERTURE_CIRCLE
    s.aperture_blades = 0
    s.aperture_rotation_rad = 0.0
    s.aperture_aspect = float(aspect)
    s.aperture_curvature = s.aperture_twist = 0.0
    s.aperture_notch_rad = s.aperture_notch_angle_rad = 0.0


def _blade_control(m, key, lo, hi, path):
    if key not in m:
        return f32(0.0)
    v = _num(m[key])
    if v < f32(lo) or v > f32(hi):
        c = f32(lo) if v < f32(lo) else f32(hi)
        warnings.warn("%s: aperture %s must be within [%g, %g]; got %g - clamping to %g."
                      % (path, key, lo, hi, v, c))
        return c
    return v


def _apply_apertures(mods, s: gl_surface, path, unsupported: List[str]):
    """apply_aperture_modifiers (optical_system.cpp:572-689): last one wins;
    default circle of aspect 1."""
    if not isinstance(mods, list):
        return None
    image = None
    for m in mods:
        if not isinstance(m, dict) or m.get("type", "") != "aperture":
            continue
        shape = m.get("shape", "")
        aspect = f32(1.0)
        if "aperture_aspect" in m:
            aspect = _num(m["aperture_aspect"])
            if not (aspect > f32(0.0)):
                warnings.warn("%s: aperture_aspect must be > 0; got %g - clamping to 1.0." % (path, aspect))
                aspect = f32(1.0)
        image = None
        if shape == "circular":
            _set_circular(s, aspect)
        elif shape == "polygon":
            blades = int(m.get("blades", 0))
            if blades < 3:
                warnings.warn("%s: polygon aperture needs blades >= 3; got %d - falling back to circular."
                              % (path, blades))
                _set_circular(s, aspect)
                continue
            rot_deg = _value(m, "rotation_deg", 0.0)
            _set_circular(s, aspect)
            s.aperture_shape = _APERTURE_POLYGON
            s.aperture_blades = blades
            s.aperture_rotation_rad = float(rot_deg * _DEG)
            s.aperture_curvature = float(_blade_control(m, "curvature", -1.0, 1.0, path))
            s.aperture_twist = float(_blade_control(m, "twist", -1.0, 1.0, path))
            s.aperture_notch_rad = float(_blade_control(m, "notch_deg", -45.0, 45.0, path) * _DEG)
            s.aperture_notch_angle_rad = float(_blade_control(m, "notch_angle_deg", 0.0, 45.0, path) * _DEG)
        elif shape == "image":
            sd = _num(m["semi_diameter"]) if "semi_diameter" in m else None
            if "image_path" not in m or sd is None or not (sd > f32(0.0)):
                warnings.warn("%s: image aperture needs 'image_path' and a positive 'semi_diameter'; "
                              "falling back to circular." % path)
                _set_circular(s, aspect)
                continue
            _set_circular(s, aspect)
            # the pixels are decoded later (OpticalSystem.load_aperture_images);
            # until then the bitmap passes every ray, as in the reference
            s.aperture_shape = _APERTURE_IMAGE
            image = (str(m["image_path"]), float(sd))
        else:
            warnings.warn("%s: unknown aperture shape '%s'; falling back to circular." % (path, shape))
            _set_circular(s, aspect)
    return image


def _parse_form(jf, s: gl_surface, path):
    """parse_form (optical_system.cpp:693-741)."""
    if not isinstance(jf, dict):
        _fail(path, "surface 'form' must be an object")
    typ = jf.get("type", "")
    if typ not in _FORM:
        _fail(path, "unknown surface form '%s'" % typ)
    s.form = _FORM[typ]
    s.radius = float(_value(jf, "radius", 0.0))
    if typ == "asphere":
        s.conic_k = float(_value(jf, "conic_constant", 0.0))
        terms = jf.get("terms")
        if isinstance(terms, list):
            n = len(terms)
            if n > _MAX_ASPHERE_TERMS:
                warnings.warn("%s: asphere has %d terms; truncating to %d." % (path, n, _MAX_ASPHERE_TERMS))
                n = _MAX_ASPHERE_TERMS
            for i in range(n):
                s.asphere_terms[i] = float(_num(terms[i]))
            s.n_asphere_terms = n
    elif typ == "cylindrical":
        ax = jf.get("axis", "x")
        s.cyl_axis = 1 if ax in ("y", "Y") else 0


def _flatten_element(jel, M: _Transform, nominal_z, catalogue, path, surfaces, notes, layer_stacks, images):
    """flatten_element (optical_system.cpp:801-912); returns the nominal z of
    the element's last surface vertex."""
    js_list, jm_list = jel.get("surfaces"), jel.get("materials")
    if not isinstance(js_list, list):
        _fail(path, "element missing 'surfaces' array")
    if not isinstance(jm_list, list):
        _fail(path, "element missing 'materials' array")
    n_surf, n_mat = len(js_list), len(jm_list)
    name = jel.get("name", "")
    if n_surf != n_mat + 1:
        _fail(path, "element '%s' has %d surfaces and %d materials (surfaces must equal materials + 1)."
              % (name, n_surf, n_mat))
    cum_local = f32(0.0)
    cum_nominal = f32(nominal_z)
    last_nominal = f32(nominal_z)
    for i, js in enumerate(js_list):
        s = default_surface()
        s.is_stop = int(bool(js.get("is_stop", False)))
        s.is_active = int(bool(js.get("is_active", True)))
        s.semi_aperture = float(_value(js, "semi_aperture", 0.0))
        unsupported: List[str] = []
        mods = js.get("modifiers", [])
        stack = _extract_coating(mods, s, path, unsupported)
        _parse_form(js.get("form", {}), s, path)
        image = _apply_apertures(mods, s, path, unsupported)
        if image is not None:
            images[len(surfaces)] = image
        thickness = _value(js, "thickness", 0.0)
        s.thickness = float(thickness)
        s.decenter_x = float(M.pos[0] + M.piv[0] + M.rot[2] * cum_local)
        s.decenter_y = float(M.pos[1] + M.piv[1] + M.rot[5] * cum_local)
        s.z = float(M.pos[2] + M.piv[2] + M.rot[8] * cum_local)
        for k in range(9):
            s.rot[k] = float(M.rot[k])
        if i < n_surf - 1:
            mat = jm_list[i] if isinstance(jm_list[i], dict) else {}
            _apply_glass(mat.get("glass", ""), catalogue, s, path)
        else:
            _apply_air(s)
        if not (s.semi_aperture > 0.0):
            warnings.warn("%s: element '%s' surface %d has semi_aperture <= 0; the tracer will reject all rays."
                          % (path, name, i))
        for u in unsupported:
            notes.append((len(surfaces), u))
        if stack is not None:
            layer_stacks[len(surfaces)] = stack
        surfaces.append(s)
        last_nominal = cum_nominal
        cum_local = cum_local + thickness
        cum_nominal = cum_nominal + thickness
    return last_nominal


def _parse_pivots(jp_list, path):
    """parse_pivots (optical_system.cpp:949-1010)."""
    if not isinstance(jp_list, list):
        _fail(path, "pivots must be an array")
    out = []
    for jp in jp_list:
        if not isinstance(jp, dict):
            _fail(path, "pivot entry must be an object")
        name = jp.get("name", "")
        if not isinstance(jp.get("elements"), list):
            _fail(path, "pivot '%s' missing 'elements' array" % name)
        p = dict(name=name, elements=[str(e) for e in jp["elements"]], manual=False,
                 point=[f32(0.0)] * 3, off_pos=[f32(0.0)] * 3, off_rot=[f32(0.0)] * 3)
        pp = jp.get("pivot_point")
        if isinstance(pp, dict):
            p["manual"] = pp.get("mode", "centroid") == "manual"
            p["point"] = [_value(pp, k, 0.0) for k in ("x", "y", "z")]
        off = jp.get("offset")
        if isinstance(off, dict):
            if isinstance(off.get("position"), dict):
                p["off_pos"] = [_value(off["position"], k, 0.0) for k in ("x", "y", "z")]
            if isinstance(off.get("rotation"), dict):
                p["off_rot"] = [_value(off["rotation"], k, 0.0) for k in ("tilt_x", "tilt_y", "roll")]
        out.append(p)
    return out


def _apply_pivot(p, point, t: _Transform):
    """apply_pivot_to_transform (optical_system.cpp:1016-1045)."""
    R = _rotation(*p["off_rot"])
    rel = [t.pos[i] - point[i] for i in range(3)]
    rot = _mat_vec(R, rel)
    t.pos = [rot[i] + point[i] + p["off_pos"][i] for i in range(3)]
    t.rot = _mat_mat(R, t.rot)
    t.piv = _mat_vec(R, t.piv)


def read_lens(path, images=None) -> Tuple[List[gl_surface], str, float, List[Tuple[int, str]]]:
    """Parse and flatten a lens file: (surface records, name, focal length
    hint, [(surface index, unsupported feature)])."""
    path = os.fspath(path)
    try:
        with open(path, "r", encoding="utf-8") as fh:
            j = json.load(fh)
    except OSError:
        _fail(path, "cannot open lens file")
    except ValueError as e:
        _fail(path, "invalid JSON: %s" % e)
    if not isinstance(j, dict) or j.get("format", "") != "ghostlight-optical":
        _fail(path, "unexpected format '%s' (expected 'ghostlight-optical')"
              % (j.get("format", "") if isinstance(j, dict) else ""))
    ver = j.get("version")
    major = int(ver.get("major", 0)) if isinstance(ver, dict) else 0
    minor = int(ver.get("minor", 0)) if isinstance(ver, dict) else 0
    if major != LENS_FORMAT_MAJOR:
        _fail(path, "unsupported lens format major version %d (this library reads version %d only)."
              % (major, LENS_FORMAT_MAJOR))
    if minor > LENS_FORMAT_MINOR:
        warnings.warn("%s: lens format minor version %d is newer than this library understands (%d); unknown "
                      "fields will be ignored." % (path, minor, LENS_FORMAT_MINOR))
    name, focal = "", f32(0.0)
    meta = j.get("metadata")
    if isinstance(meta, dict):
        name = str(meta.get("name", ""))
        focal = _value(meta, "focal_length_mm", 0.0)
    catalogue = _parse_catalogue(j["glass_catalogue"], path) if "glass_catalogue" in j else {}
    if "optical_system" not in j:
        _fail(path, "missing optical_system array")
    jsys = j["optical_system"]
    if not isinstance(jsys, list):
        _fail(path, "optical_system must be an array")

    # pass 1: element transforms; relative positions chain on the resolved z
    records = []
    prev_z, have_prev = f32(0.0), False
    for item in jsys:
        typ = item.get("type", "") if isinstance(item, dict) else ""
        if typ != "element":
            _fail(path, "optical_system item has unknown type '%s' (expected 'element')." % typ)
        jx = item.get("transform", {})
        t = _parse_transform(jx)
        mode = "absolute"
        if isinstance(jx, dict) and isinstance(jx.get("position"), dict):
            mode = jx["position"].get("mode", "absolute")
        if mode == "relative_to_preceding":
            if not have_prev:
                warnings.warn("%s: first element '%s' has position.mode='relative_to_preceding'; treating as "
                              "absolute." % (path, item.get("name", "")))
            else:
                t.pos[2] = t.pos[2] + prev_z
        elif mode != "absolute":
            warnings.warn("%s: element '%s' has unknown position.mode='%s'; treating as absolute."
                          % (path, item.get("name", ""), mode))
        records.append(dict(id=str(item.get("id", "")), node=item, xform=t, pre_pivot_z=t.pos[2]))
        prev_z, have_prev = t.pos[2], True

    # pass 2: pivots on the resolved transforms, stacked in array order
    if "pivots" in j:
        pivots = _parse_pivots(j["pivots"], path)
        ids = {}
        for i, r in enumerate(records):
            if r["id"] and r["id"] not in ids:
                ids[r["id"]] = i
        for p in pivots:
            targets = []
            for eid in p["elements"]:
                if eid not in ids:
                    _fail(path, "pivot '%s' references unknown element id '%s'." % (p["name"], eid))
                targets.append(ids[eid])
            if not targets:
                continue
            if p["manual"]:
                point = list(p["point"])
            else:
                n = float(len(targets))
                point = [f32(sum(float(records[i]["xform"].pos[k]) for i in targets) / n) for k in range(3)]
            for i in targets:
                _apply_pivot(p, point, records[i]["xform"])

    # pass 3: surfaces, then the inter-element air gaps from nominal z
    surfaces: List[gl_surface] = []
    notes: List[Tuple[int, str]] = []
    layer_stacks: Dict[int, list] = {}
    if images is None:
        images = {}
    emits = []
    for r in records:
        z_nom = r["xform"].pos[2]
        first = len(surfaces)
        last_z = _flatten_element(r["node"], r["xform"], z_nom, catalogue, path, surfaces, notes, layer_stacks,
                                  images)
        emits.append((z_nom, first, len(surfaces) - first, last_z))
    for k in range(len(emits) - 1):
        _, first, n, last_z = emits[k]
        surfaces[first + n - 1].thickness = float(emits[k + 1][0] - last_z)
    # rebase so the chain ends at the sensor (z = 0) under the pre-pivot layout
    if emits and records:
        internal = f32(0.0)
        for js in records[-1]["node"]["surfaces"]:
            internal = internal + _value(js, "thickness", 0.0)
        total = records[-1]["pre_pivot_z"] + internal
        for s in surfaces:
            s.z = float(f32(s.z) - total)
    if not surfaces:
        _fail(path, "optical_system produced no surfaces")
    # post-flatten pass: thin-film stacks bake against the final glasses
    from . import coatings as K
    for idx in sorted(layer_stacks):
        tid = K.bake_layers(surfaces, idx, layer_stacks[idx])
        K.reset_coating(surfaces[idx], K.SPECTRAL_ANGULAR, tid)
    for idx, what in notes:
        warnings.warn("%s: surface %d: %s is not supported by this library" % (path, idx, what))
    return surfaces, name, float(focal), notes


def load_lens(path):
    """OpticalSystem.load(path): the flat surface table of a lens file."""
    from .optics import OpticalSystem
    images = {}
    surfaces, name, focal, notes = read_lens(path, images)
    out = OpticalSystem.from_records(surfaces, name=name, focal_length=focal)
    out.unsupported = notes
    for idx, (src, semi) in images.items():
        out.set_aperture_source(idx, src, semi)
    out.source_path = os.fspath(path)
    return out


# ---------------------------------------------------------------------------
# writer
# ---------------------------------------------------------------------------
def _glass_entry(s: gl_surface):
    if s.disp_model == _DISP_SELLMEIER:
        return {"model": "sellmeier", "B": [float(s.sellmeier_B[k]) for k in range(3)],
                "C": [float(s.sellmeier_C[k]) for k in range(3)]}
    return {"model": "abbe", "nd": float(s.ior), "Vd": float(s.abbe_v)}


def _euler_from_rot(R):
    """tilt_x, tilt_y, roll (degrees) of R = Ry(tilt_y) Rx(tilt_x) Rz(roll)."""
    import math
    r = [float(v) for v in R]
    tx = math.asin(max(-1.0, min(1.0, -r[5])))
    ty = math.atan2(r[2], r[8])
    rz = math.atan2(r[3], r[4])
    return math.degrees(tx), math.degrees(ty), math.degrees(rz)


def _modifiers(s: gl_surface, image=None):
    mods = []
    if s.coating_model == _COATING_SIMPLE:
        if s.ar_layers:
            mods.append({"type": "coating", "model": "simple", "ar_layers": int(s.ar_layers)})
    elif s.coating_model == _COATING_ARTIST:
        mods.append({"type": "coating", "model": "artist", "tint": [float(s.tint_r), float(s.tint_g),
                                                                     float(s.tint_b)],
                     "strength": float(s.tint_strength)})
    elif s.coating_model == _COATING_ATTENUATOR_GAUSS:
        mods.append({"type": "coating", "model": "attenuator_gaussian", "sigma": float(s.gauss_sigma),
                     "attenuation_background": float(s.gauss_background),
                     "attenuation_peak": float(s.gauss_peak), "decenter_x": float(s.gauss_decenter_x),
                     "decenter_y": float(s.gauss_decenter_y)})
    elif s.coating_model in (1, 2, 3) and s.ar_layers:
        from . import coatings as K
        model, a0, a1, r, ref, discard = K.read_table(s.ar_layers)
        stack = K.layers_of(s.ar_layers) if model == K.SPECTRAL_ANGULAR else None
        if stack:
            mods.append({"type": "coating", "model": "layers", "layers": [
                {"material": d["material"], "thickness_nm": float(d["thickness_nm"]),
                 "nk_table": [{"lambda_um": float(a), "n": float(b), "k": float(c)} for a, b, c in d["nk_table"]]}
                for d in stack]})
        else:
            m = {"type": "coating", "out_of_range": "discard" if discard else "clamp"}
            if model == K.SPECTRAL_ANGULAR:
                m.update(model="spectral_angular", wavelengths_nm=[float(v) for v in a0],
                         angles_deg=[float(v) for v in a1], r=[[float(v) for v in row] for row in r],
                         angle_ref_ior=float(ref))
            else:
                key = "lambda_nm" if model == K.SPECTRAL else "angle_deg"
                m.update(model="spectral" if model == K.SPECTRAL else "angular",
                         data=[{key: float(k), "r": float(v)} for k, v in zip(a0, r)])
                if model == K.ANGULAR:
                    m["angle_ref_ior"] = float(ref)
            mods.append(m)
    elif s.coating_model not in (1, 2, 3):
        raise ValueError("save_lens: unknown coating model %d" % s.coating_model)
    ap = {"type": "aperture"}
    if s.aperture_shape == _APERTURE_POLYGON:
        import math
        ap.update(shape="polygon", blades=int(s.aperture_blades),
                  rotation_deg=math.degrees(float(s.aperture_rotation_rad)))
        for key, v in (("curvature", s.aperture_curvature), ("twist", s.aperture_twist),
                       ("notch_deg", math.degrees(s.aperture_notch_rad)),
                       ("notch_angle_deg", math.degrees(s.aperture_notch_angle_rad))):
            if v:
                ap[key] = float(v)
    elif s.aperture_shape == _APERTURE_CIRCLE:
        ap["shape"] = "circular"
    else:
        src, semi = image if image is not None else ("", 0.0)
        if not src or not semi > 0:
            raise ValueError("save_lens: image aperture has no source path / semi-diameter to write")
        ap.update(shape="image", image_path=src, semi_diameter=float(semi))
    if s.aperture_aspect != 1.0:
        ap["aperture_aspect"] = float(s.aperture_aspect)
    if len(ap) > 2 or s.aperture_shape != _APERTURE_CIRCLE:
        mods.append(ap)
    return mods


def lens_document(lens, name: str = "") -> dict:
    """A ``ghostlight-optical`` document of a flat lens: one element per run
    of surfaces joined by glass (an element ends at the first surface followed
    by air), each placed at its first vertex (absolute z, sensor at 0) with its
    decenter and rotation; glasses are catalogued inline by their dispersion
    data.  Loading the document gives back the same table, z to float
    rounding (the loader re-accumulates element thicknesses)."""
    import uuid
    surfs = [s.record if hasattr(s, "record") else s for s in getattr(lens, "surfaces", lens)]
    image_sources = {i: (img.source_path, img.semi_diameter)
                     for i, img in enumerate(getattr(lens, "aperture_images", []) or [])
                     if getattr(img, "source_path", "")}
    if not surfs:
        raise ValueError("save_lens: lens has no surfaces")
    catalogue, glass_names = {}, {}
    elements, cur = [], []
    for i, s in enumerate(surfs):
        cur.append(i)
        if s.disp_model == _DISP_AIR or i == len(surfs) - 1:
            elements.append(cur)
            cur = []
    key_of = {}
    doc_elements = []
    for ei, idx in enumerate(elements):
        first = surfs[idx[0]]
        jsurfs, mats = [], []
        for k, i in enumerate(idx):
            s = surfs[i]
            form = {"type": {0: "sphere", 1: "asphere", 2: "cylindrical"}[int(s.form)], "radius": float(s.radius)}
            if s.form == 1:
                form["conic_constant"] = float(s.conic_k)
                form["terms"] = [float(s.asphere_terms[t]) for t in range(int(s.n_asphere_terms))]
            elif s.form == 2:
                form["axis"] = "y" if s.cyl_axis == 1 else "x"
            js = {"id": str(uuid.uuid5(uuid.NAMESPACE_OID, "%s/%d" % (name, i))),
                  "semi_aperture": float(s.semi_aperture), "thickness": float(s.thickness), "form": form}
            if s.is_stop:
                js["is_stop"] = True
            if not s.is_active:
                js["is_active"] = False
            mods = _modifiers(s, image_sources.get(i))
            if mods:
                js["modifiers"] = mods
            jsurfs.append(js)
            if k < len(idx) - 1:
                ge = _glass_entry(s)
                key = json.dumps(ge, sort_keys=True)
                if key not in key_of:
                    key_of[key] = "glass_%d" % len(key_of)
                    catalogue[key_of[key]] = {"name": key_of[key], "dispersion": ge}
                mats.append({"glass": key_of[key]})
        tx, ty, rz = _euler_from_rot(first.rot)
        xf = {"position": {"mode": "absolute", "x": float(first.decenter_x), "y": float(first.decenter_y),
                           "z": float(first.z)}}
        if any(abs(v) > 0.0 for v in (tx, ty, rz)):
            xf["rotation"] = {"tilt_x": tx, "tilt_y": ty, "roll": rz}
        doc_elements.append({"type": "element", "id": str(uuid.uuid5(uuid.NAMESPACE_OID, "%s/e%d" % (name, ei))),
                             "name": "element %d" % ei, "transform": xf, "surfaces": jsurfs,
                             "materials": mats})
    del glass_names
    meta = {"name": name or getattr(lens, "name", "") or "lens"}
    if getattr(lens, "focal_length", 0.0):
        meta["focal_length_mm"] = float(lens.focal_length)
    return {"format": "ghostlight-optical", "version": {"major": LENS_FORMAT_MAJOR, "minor": LENS_FORMAT_MINOR},
            "metadata": meta, "glass_catalogue": catalogue, "optical_system": doc_elements, "pivots": []}


def save_lens(lens, path, name: str = "") -> None:
    """OpticalSystem.save (optical_system.py:252): write a lens file."""
    with open(os.fspath(path), "w", encoding="utf-8") as fh:
        json.dump(lens_document(lens, name), fh, indent=2)
        fh.write("\n")

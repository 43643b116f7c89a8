"""Table-backed coatings: spectral, angular and spectral-angular reflectance
tables and thin-film layer stacks.

The reference keeps a surface's tables beside the surface list
(``OpticalSystem::coating_tables``, ghostlight/src/optical_system.h:285-301)
and edits them through ``set_coating_spectral_table`` /
``set_coating_angular_table`` / ``set_coating_sa_table`` /
``set_coating_layers`` (bindings/python/src/bind_geometry.cpp:412-590).  Here
a table is an immutable entry of the native library's table store, named by
a positive id that the surface record carries in ``ar_layers`` (with
``coating_model`` SPECTRAL / ANGULAR / SPECTRAL_ANGULAR), so a table travels
with its surface through copies, inserts and the flat-array entry points.
Identical content gives the same id.

A layer stack is baked on the host into a 31 x 18 spectral-angular table
(400..700 nm x 0..85 degrees, ``OpticalSystem::bake_coating_layers``,
optical_system.cpp:1483-1575); the stack itself is remembered beside the id
for ``get_coating_layers`` and the lens-file writer.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List

import numpy as np

SPECTRAL, ANGULAR, SPECTRAL_ANGULAR = 1, 2, 3
TABLE_MODELS = (SPECTRAL, ANGULAR, SPECTRAL_ANGULAR)

# baked table id -> the layer stack it was baked from
_LAYERS: Dict[int, List[dict]] = {}


def _lib():
    from . import _native
    return _native.load()


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def create_table(model: int, axis0, r, axis1=None, angle_ref_ior: float = 1.0,
                 out_of_range_discard: bool = False) -> int:
    """Store a table and return its id.  1-D models: ascending keys ``axis0``
    (nm for SPECTRAL, degrees for ANGULAR) and ``r``; SPECTRAL_ANGULAR:
    ascending wavelengths ``axis0``, ascending angles ``axis1`` and ``r`` of
    shape (len(axis0), len(axis1))."""
    from . import _native
    a0 = np.ascontiguousarray(np.asarray(axis0, np.float32).ravel())
    rr = np.ascontiguousarray(np.asarray(r, np.float32).ravel())
    if axis1 is None:
        a1, p1, n1 = None, None, 0
    else:
        a1 = np.ascontiguousarray(np.asarray(axis1, np.float32).ravel())
        p1, n1 = _fp(a1), len(a1)
    need = len(a0) * (n1 if n1 else 1)
    if len(a0) < 1 or rr.size != need:
        raise ValueError("coating table: r must hold %d values" % need)
    out = C.c_int()
    _native.check(_lib().gl_coating_table_create(int(model), _fp(a0), len(a0), p1, n1, _fp(rr),
                                                 float(angle_ref_ior), int(bool(out_of_range_discard)),
                                                 C.byref(out)), "coating_table_create")
    return int(out.value)


def table_info(table_id: int) -> dict:
    from . import _native
    m, n0, n1, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    ref = C.c_float()
    _native.check(_lib().gl_coating_table_info(int(table_id), C.byref(m), C.byref(n0), C.byref(n1),
                                               C.byref(ref), C.byref(d)), "coating_table_info")
    return {"model": m.value, "n0": n0.value, "n1": n1.value, "angle_ref_ior": float(ref.value),
            "out_of_range_discard": bool(d.value)}


def read_table(table_id: int):
    """(model, axis0, axis1, r, angle_ref_ior, out_of_range_discard) of a
    stored table; axis1 is empty and r 1-D for the 1-D models."""
    from . import _native
    info = table_info(table_id)
    n0, n1 = info["n0"], info["n1"]
    a0 = np.zeros(n0, np.float32)
    a1 = np.zeros(n1, np.float32)
    r = np.zeros(n0 * n1 if n1 else n0, np.float32)
    _native.check(_lib().gl_coating_table_read(int(table_id), _fp(a0), _fp(a1) if n1 else None, _fp(r)),
                  "coating_table_read")
    if n1:
        r = r.reshape(n0, n1)
    return info["model"], a0, a1, r, info["angle_ref_ior"], info["out_of_range_discard"]


def prepare(table_id: int) -> None:
    """Copy a table to the current device ahead of an allocation-free trace."""
    from . import _native
    _native.check(_lib().gl_coating_table_prepare(int(table_id)), "coating_table_prepare")


def _layer_arrays(layers):
    th, cnt, nks = [], [], []
    for d in layers:
        nk = np.asarray(d["nk_table"], np.float32)
        if nk.ndim != 2 or nk.shape[1] != 3 or nk.shape[0] < 1:
            raise ValueError("nk_table must be a (K, 3) array of (lambda_um, n, k)")
        th.append(np.float32(d["thickness_nm"]))
        cnt.append(nk.shape[0])
        nks.append(nk)
    nk = np.ascontiguousarray(np.concatenate(nks))
    return (np.array(th, np.float32), np.array(cnt, np.int32), np.ascontiguousarray(nk[:, 0]),
            np.ascontiguousarray(nk[:, 1]), np.ascontiguousarray(nk[:, 2]))


def bake_layers(surfaces, index: int, layers) -> int:
    """Bake the thin-film stack ``layers`` (dicts of material, thickness_nm,
    nk_table (K, 3) of lambda_um, n, k) on surface ``index`` of the flat
    records ``surfaces`` into a spectral-angular table; returns its id."""
    from . import _native
    from ._abi import surface_array
    if not layers:
        raise ValueError("layers list must not be empty")
    th, cnt, lam, nn, kk = _layer_arrays(layers)
    arr = surface_array(surfaces)
    out = C.c_int()
    rc = _lib().gl_coating_bake_layers(arr, len(arr), int(index), len(th), _fp(th),
                                       cnt.ctypes.data_as(C.POINTER(C.c_int)), _fp(lam), _fp(nn), _fp(kk),
                                       C.byref(out))
    _native.check(rc, "coating_bake_layers")
    tid = int(out.value)
    _LAYERS[tid] = [{"material": str(d.get("material", "")), "thickness_nm": float(np.float32(d["thickness_nm"])),
                     "nk_table": np.asarray(d["nk_table"], np.float32).copy()} for d in layers]
    return tid


def layers_of(table_id: int):
    """The layer stack a baked table came from, or None."""
    return _LAYERS.get(int(table_id))


def reset_coating(rec, model: int = 0, table_id: int = 0) -> None:
    """A default ``Coating`` (optical_system.h:109-147) of `model` on a flat
    record, naming table `table_id`."""
    rec.coating_model = int(model)
    rec.ar_layers = int(table_id)
    rec.tint_r = rec.tint_g = rec.tint_b = 1.0
    rec.tint_strength = float(np.float32(0.04))
    rec.gauss_sigma = rec.gauss_background = rec.gauss_peak = 0.0
    rec.gauss_decenter_x = rec.gauss_decenter_y = 0.0


def sort_1d(data):
    """(N, 2) rows of (key, r) in ascending key order, ties kept in order."""
    d = np.asarray(data, np.float32)
    if d.ndim != 2 or d.shape[1] != 2 or d.shape[0] < 1:
        raise ValueError("table must be an (N, 2) array of (key, r)")
    return d[np.argsort(d[:, 0], kind="stable")]

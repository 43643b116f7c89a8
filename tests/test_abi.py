"""The C-ABI library: it loads, exports every entry point include/*.h
declares, and its host builders reproduce the reference bit for bit
(no GPU needed)."""
import ctypes as C
import pathlib
import re

import numpy as np
import pytest

from conftest import LENS_NAMES, REPO, lens_from_pins
from ghostlight_gb300 import _native
from ghostlight_gb300._abi import gl_sampler_params, gl_spectral_sample, surface_array


def _declared_functions():
    names = set()
    for h in (REPO / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(gl_[A-Za-z0-9_]+)\s*\(",
                             text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = _declared_functions()
    assert "gl_render_ghosts" in names and "gl_filter_ghost_pairs" in names
    assert len(names) >= 12


@pytest.mark.parametrize("name", _declared_functions())
def test_library_exports(name):
    lib = _native.load()
    assert hasattr(lib, name), name


def test_library_is_in_tree():
    p = pathlib.Path(_native.lib_path())
    assert p.exists() and REPO in p.parents


@pytest.mark.parametrize("name", LENS_NAMES)
@pytest.mark.parametrize("cfg", [(32, 0, 0, 0), (64, 1, 7, 0), (192, 2, 12345, 0), (256, 2, 12345, 6)])
def test_host_pupil_grid_bit_exact(pins, name, cfg):
    import hashlib
    from ghostlight_gb300 import flare
    from ghostlight_gb300.optics import OpticalSystem
    lens = OpticalSystem.from_records(lens_from_pins(pins, name))
    g = flare.pupil_grid(lens, *cfg)
    key = "%s/samples_%d_%d_%d_%d" % ((name,) + cfg)
    assert len(g) == int(pins[key + "/count"][0])
    assert hashlib.sha256(g.tobytes()).digest() == pins[key + "/sha256"].tobytes()


@pytest.mark.parametrize("n", [3, 8, 16, 31])
@pytest.mark.parametrize("cs", [0, 1, 4])
def test_host_spectral_table_bit_exact(pins, n, cs):
    from ghostlight_gb300 import flare
    t, c = flare.spectral_table(n, cs)
    np.testing.assert_array_equal(t.view(np.uint32), pins["spectral/%d_%d/table" % (n, cs)].view(np.uint32))
    np.testing.assert_array_equal(c.view(np.uint32), pins["spectral/%d_%d/corr" % (n, cs)].view(np.uint32))


@pytest.mark.parametrize("name", LENS_NAMES)
def test_host_enumeration(pins, name):
    from ghostlight_gb300 import enumerate_ghost_pairs
    from ghostlight_gb300.optics import OpticalSystem
    lens = OpticalSystem.from_records(lens_from_pins(pins, name))
    got = np.array([[p.surf_a, p.surf_b] for p in enumerate_ghost_pairs(lens)], np.int32)
    np.testing.assert_array_equal(got, pins[name + "/enumerate"])


def test_finalize_matches_reference_layout(pins):
    from ghostlight_gb300.optics import OpticalSystem
    recs = lens_from_pins(pins, "cfg2_wide_angle_24")
    lens = OpticalSystem.from_records(recs)
    z0 = [s.z for s in lens.surfaces]
    for s in lens.surfaces:
        s.z = 0.0
    assert lens.finalize()
    assert [s.z for s in lens.surfaces] == z0


def test_invalid_arguments_raise_value_error():
    lib = _native.load()
    n = C.c_int()
    with pytest.raises(ValueError):
        _native.check(lib.gl_enumerate_ghost_pairs(None, 0, None, 0, C.byref(n)), "enumerate_ghost_pairs")
    sp = gl_sampler_params(5000, 0, 0, 0, 0.0)
    with pytest.raises(ValueError):
        from ghostlight_gb300._abi import gl_surface
        arr = (gl_surface * 1)()
        _native.check(lib.gl_build_aperture_samples(arr, 1, C.byref(sp), None, 0, C.byref(n)), "pupil_grid")
    with pytest.raises(ValueError):
        _native.check(lib.gl_build_spectral_table(0, 0, None, None, None), "spectral_table")


def test_trace_bad_indices_raise_before_device():
    from ghostlight_gb300 import Ray, trace_ghost_ray
    from ghostlight_gb300.optics import OpticalSystem
    from ghostlight_gb300 import prescriptions as P
    lens = OpticalSystem(P.double_gauss_12())
    for a, b in ((3, 3), (-1, 2), (2, 40), (5, 1)):
        with pytest.raises(ValueError):
            trace_ghost_ray(Ray(), lens, a, b)

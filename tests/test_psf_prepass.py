"""PSF grid pre-pass (host): tile centres by pupil-mean and by aiming."""
import numpy as np

from conftest import lens_from_pins


def _lens(pins):
    from ghostlight_gb300.optics import OpticalSystem
    return OpticalSystem.from_records(lens_from_pins(pins, "cfg1_double_gauss_12"))


def _prepass(lens, src, mode):
    import ctypes as C
    from ghostlight_gb300 import _native
    from ghostlight_gb300._abi import gl_psf_cell
    lib = _native.load()
    arr = lens.to_array()
    s7 = np.ascontiguousarray(src, np.float32)
    cells = (gl_psf_cell * len(s7))()
    _native.check(lib.gl_psf_prepass(arr, len(arr), s7.ctypes.data_as(C.POINTER(C.c_float)), len(s7), mode, cells),
                  "prepass")
    return cells


def test_centroid_is_the_pupil_mean_of_float_traces(pins):
    """CHIEF_CENTROID: the mean landing of the 7 x 7 unit-disc probe at the d
    line, accumulated in float32 in raster order — recomputed here with the
    float oracle trace (bit-exact with the reference's host trace)."""
    from oracle import oracle as O
    lens = _lens(pins)
    recs = lens.records()
    src = np.array([[0.0, 0.0, 1, 1, 1, 0, 0], [0.12, -0.05, 1, 1, 1, 0, 0]], np.float32)
    cells = _prepass(lens, src, 0)
    f = np.float32
    for k, (ax, ay) in enumerate(src[:, :2]):
        bx, by = f(np.tan(ax)), f(np.tan(ay))
        d = np.array([bx, by, 1.0], f)
        d = (d * (f(1.0) / f(np.sqrt(f(d @ d))))).astype(f)
        rays = []
        for iy in range(7):
            v = f(-1.0) + (f(iy) + f(0.5)) * (f(2.0) / f(7))
            for ix in range(7):
                u = f(-1.0) + (f(ix) + f(0.5)) * (f(2.0) / f(7))
                if u * u + v * v > f(1.0):
                    continue
                rays.append([u * f(recs[0].semi_aperture) - f(20.0) * bx, v * f(recs[0].semi_aperture) - f(20.0) * by,
                             f(recs[0].z) - f(20.0), d[0], d[1], d[2], f(587.56)])
        res = O.trace(recs, -1, -1, np.array(rays, f), fp64=False)
        ok = (res[:, 4] == 0) & np.isfinite(res[:, 0]) & np.isfinite(res[:, 1])
        sx = sy = f(0.0)
        for x, y in res[ok][:, :2]:
            sx = f(sx + f(x)); sy = f(sy + f(y))
        n = int(ok.sum())
        assert cells[k].status == 0 and n > 0
        assert f(cells[k].chief_x_mm) == f(sx / f(n)) and f(cells[k].chief_y_mm) == f(sy / f(n))
        assert abs(cells[k].pupil_fraction - n / len(rays)) < 1e-6


def test_fixed_target_aims_the_chief_ray(pins):
    lens = _lens(pins)
    src = np.array([[0.05, 0.02, 1, 1, 1, 3.0, 1.2], [0.0, 0.0, 1, 1, 1, -2.0, -4.0]], np.float32)
    cells = _prepass(lens, src, 1)
    for k in range(2):
        assert cells[k].status == 0
        assert abs(cells[k].chief_x_mm - src[k, 5]) < 2e-4 and abs(cells[k].chief_y_mm - src[k, 6]) < 2e-4
        assert cells[k].aim_residual_mm < 2e-4


def test_kept_prepass_equals_a_fresh_one(pins):
    """psf_inputs with a lens-owned cache (the serving path) returns the same
    tile centres, sources and pupil grid as without one, and a second atlas
    over the same sources reuses the kept pre-pass and grid."""
    from ghostlight_gb300.config import PSFConfig
    from ghostlight_gb300.psf_grid import psf_inputs
    lens = _lens(pins)
    cfg = PSFConfig(grid_nx=3, grid_ny=2, tile_w=32, tile_h=32, tile_extent_mm=0.3, spectral_samples=8,
                    ray_grid=24)
    xs = np.linspace(-0.2, 0.2, 3, dtype=np.float32)
    src = np.array([[x, y, 1.0, 1.0, 1.0] for y in (-0.1, 0.1) for x in xs], np.float32)
    cache = {}
    fresh = psf_inputs(src, lens, cfg)
    first = psf_inputs(src, lens, cfg, cache)
    assert len(cache) == 2
    kept_cells = [v for k, v in cache.items() if k[0] == "cells"][0]
    again = psf_inputs(src, lens, cfg, cache)
    assert again["cells"] is kept_cells and again["grid"] is first["grid"]
    for got in (first, again):
        for i in range(len(src)):
            a, b = got["cells"][i], fresh["cells"][i]
            assert (a.chief_x_mm, a.chief_y_mm, a.beam_ax, a.beam_ay) == (b.chief_x_mm, b.chief_y_mm, b.beam_ax,
                                                                          b.beam_ay)
            s, t = got["sources"][i], fresh["sources"][i]
            assert bytes(s) == bytes(t)
        np.testing.assert_array_equal(got["grid"], fresh["grid"])
    other = psf_inputs(src[:4], lens, cfg, cache)     # other sources: a pre-pass of their own
    assert len(cache) == 3 and other["n"] == 4

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

"""Helper for the PSF tests: the pre-pass cells as dicts."""
import ctypes as C

import numpy as np


def cells_of(lens, src, mode):
    from ghostlight_gb300 import _native
    from ghostlight_gb300._abi import gl_psf_cell
    lib = _native.load()
    arr = lens.to_array()
    s7 = np.ascontiguousarray(src, np.float32)
    cells = (gl_psf_cell * len(s7))()
    _native.check(lib.gl_psf_prepass(arr, len(arr), s7.ctypes.data_as(C.POINTER(C.c_float)), len(s7), mode, cells),
                  "prepass")
    return [dict(beam_ax=c.beam_ax, beam_ay=c.beam_ay, chief_x_mm=c.chief_x_mm, chief_y_mm=c.chief_y_mm)
            for c in cells]

"""The allocation-free trace entry point (gl_trace_rays_noalloc).

It exists for callers that may not allocate device memory while they run; it
keeps the lens tables in a fixed array inside the library instead.  This file
is collected last on purpose: it checks the new entry point against the
ordinary one (gl_trace_rays) through the C-ABI, on two calls in a row with
different lenses so that contents left in the shared array by one call cannot
leak into the next.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import lens_from_pins

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _trace(fn, lens_recs, a, b, rays_np):
    from ghostlight_gb300 import _native
    from ghostlight_gb300._abi import surface_array
    rays = torch.from_numpy(np.ascontiguousarray(rays_np)).cuda()
    out = torch.full((rays.shape[0], 5), -7.0, dtype=torch.float32, device="cuda")
    arr = surface_array(lens_recs)
    st = torch.cuda.current_stream().cuda_stream
    _native.check(fn(arr, len(arr), a, b, rays.data_ptr(), rays.shape[0], out.data_ptr(), st), "trace")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_trace_matches_allocating_entry_two_calls(pins):
    from ghostlight_gb300 import _native
    lib = _native.load()
    cases = [("cfg2_wide_angle_24", 0), ("cfg4_anamorphic_18", 1)]
    for name, k in cases:
        recs = lens_from_pins(pins, name)
        a, b = (int(x) for x in pins["%s/rays_%d/ab" % (name, k)])
        rays = pins["%s/rays_%d/in" % (name, k)]
        want = _trace(lib.gl_trace_rays, recs, a, b, rays)
        got = _trace(lib.gl_trace_rays_noalloc, recs, a, b, rays)
        assert (want[:, 4] == got[:, 4]).all()
        ok = want[:, 4] == 0
        np.testing.assert_allclose(got[ok, :4], want[ok, :4], rtol=1e-6, atol=1e-6)
    # primary rays through the first lens again, after the second lens used the table
    recs = lens_from_pins(pins, "cfg2_wide_angle_24")
    rays = pins["cfg2_wide_angle_24/rays_0/in"]
    want = _trace(lib.gl_trace_rays, recs, -1, -1, rays)
    got = _trace(lib.gl_trace_rays_noalloc, recs, -1, -1, rays)
    assert (want[:, 4] == got[:, 4]).all()
    np.testing.assert_allclose(got[want[:, 4] == 0, :4], want[want[:, 4] == 0, :4], rtol=1e-6, atol=1e-6)


def test_noalloc_trace_rejects_lenses_above_the_table_size(pins):
    from ghostlight_gb300 import _native
    lib = _native.load()
    recs = lens_from_pins(pins, "cfg2_wide_angle_24")
    big = (recs * 3)[:65]
    rays = pins["cfg2_wide_angle_24/rays_0/in"][:4]
    with pytest.raises(ValueError, match="64 surfaces"):
        _trace(lib.gl_trace_rays_noalloc, big, -1, -1, rays)


def test_noalloc_trace_refuses_stream_capture(pins):
    """The call waits for its own stream, so under capture it must refuse
    (GL_ERR_INVALID -> ValueError) instead of breaking the caller's graph."""
    from ghostlight_gb300 import _native
    from ghostlight_gb300._abi import surface_array
    lib = _native.load()
    recs = lens_from_pins(pins, "cfg2_wide_angle_24")
    arr = surface_array(recs)
    rays = torch.from_numpy(np.ascontiguousarray(pins["cfg2_wide_angle_24/rays_0/in"][:32])).cuda()
    out = torch.zeros((32, 5), dtype=torch.float32, device="cuda")
    x = torch.zeros(4, device="cuda")
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            x.add_(1.0)
            rc = lib.gl_trace_rays_noalloc(arr, len(arr), -1, -1, rays.data_ptr(), 32, out.data_ptr(),
                                           s.cuda_stream)
    assert rc != 0
    with pytest.raises(ValueError, match="captured"):
        _native.check(rc, "trace")
    g.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0
    # the same call outside the capture still works
    got = _trace(lib.gl_trace_rays_noalloc, recs, -1, -1, rays.cpu().numpy())
    want = _trace(lib.gl_trace_rays, recs, -1, -1, rays.cpu().numpy())
    assert (got[:, 4] == want[:, 4]).all()

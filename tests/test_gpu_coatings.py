"""Table-backed coatings on the GPU: the device culler's ghost set bit for bit
against the reference's (tests/golden/coating_pins.npz), the batched render
within 1e-3 relative L2 of the FP64 oracle and of the reference's own host
render, the device trace of every table kind (discard mode included) against
the oracle, and the allocation-free trace's residency rule."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as O
from test_coatings import _rays, coated, meta, pins, register_oracle  # noqa: F401

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_device_culler_bit_exact(pins, meta):
    import ghostlight_gb300 as gl
    from ghostlight_gb300.flare import filter_ghosts_device
    cal = meta["calibration"]
    r = filter_ghosts_device(coated(), cal["sensor_half_w"], cal["sensor_half_h"],
                             gl.FlareConfig(min_ghost_intensity=1e-7))
    np.testing.assert_array_equal(r.pairs, pins["pairs"])
    np.testing.assert_allclose(r.boosts, pins["boosts"], rtol=1e-5)


def test_render_matches_oracle_and_reference(pins, meta):
    from ghostlight_gb300.flare import GhostRenderPlan, pupil_grid, spectral_table
    lens = coated()
    register_oracle(lens)
    cal = meta["calibration"]
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    pairs, boosts, src = pins["pairs"], pins["boosts"], pins["source"]
    spec, corr = spectral_table(8)
    grid = pupil_grid(lens, 48)
    W = H = 128
    plan = GhostRenderPlan(lens, pairs, boosts, src, [grid], np.zeros(len(pairs), np.int32), spec, corr,
                           W, H, hw, hh, 1000.0, apply_correction=False)
    out = [torch.zeros((H, W), dtype=torch.float32, device="cuda") for _ in range(3)]
    plan.execute(*out)
    torch.cuda.synchronize()
    got = np.stack([o.cpu().numpy() for o in out])
    plan.close()
    want = O.render(lens.records(), pairs, boosts, src, [grid], spec, hw, hh, W, H, 1000.0, fp64=True)
    assert want.sum() > 0
    assert rel_l2(got, want) < 1e-3
    assert rel_l2(got, pins["image"]) < 2e-3
    # the tables change the image: the same lens uncoated renders otherwise
    plain = coated()
    for i in range(plain.num_surfaces()):
        if plain.surfaces[i].coating_model in (1, 2, 3):
            plain.clear_coating(i)
    bare = O.render(plain.records(), pairs, boosts, src, [grid], spec, hw, hh, W, H, 1000.0, fp64=True)
    assert rel_l2(bare, want) > 0.05


@pytest.mark.parametrize("discard", [False, True])
def test_device_trace_matches_oracle(discard):
    import ghostlight_gb300 as gl
    lens = coated()
    if discard:
        lens.set_coating_angular_table(3, [[0.0, 0.02], [12.0, 0.03]], angle_ref_ior=1.0,
                                       out_of_range_discard=True)
        lens.set_coating_spectral_table(1, [[450.0, 0.01], [550.0, 0.004], [650.0, 0.012]],
                                        out_of_range_discard=True)
    register_oracle(lens)
    surfs = lens.records()
    rays = _rays(surfs, 8192, 7, 0.35)
    zero = 0
    for a, b in ((-1, -1), (1, 3), (3, 5), (1, 8), (5, 8), (2, 3)):
        got = gl.trace_rays(lens, torch.from_numpy(rays).cuda(), a, b).cpu().numpy()
        want = O.trace(surfs, a, b, rays, fp64=False)
        assert (got[:, 4] == want[:, 4]).mean() >= 0.99
        ok = (got[:, 4] == 0) & (want[:, 4] == 0)
        assert ok.mean() > 0.03
        w_got, w_want = got[ok, 3].astype(np.float64), want[ok, 3]
        live = w_want > 0
        zero += int((~live).sum())
        # a discard decision sits at a table edge: the device's rounding may
        # take the other side for a ray within rounding of that edge
        assert ((w_got > 0) == live).mean() >= 0.999
        both = live & (w_got > 0)
        rw = np.abs(w_got[both] - w_want[both]) / w_want[both]
        assert np.median(rw) < 1e-5 and np.percentile(rw, 99) < 1e-3
    assert (zero > 0) == discard


def test_noalloc_trace_needs_resident_tables():
    """The allocation-free trace does not copy tables: it refuses a table
    that is not on the device yet, and runs once it is prepared."""
    import ctypes as C
    import ghostlight_gb300 as gl
    from ghostlight_gb300 import _native
    from ghostlight_gb300 import coatings as K
    lens = coated()
    # a table no other test has used on the device
    lens.set_coating_spectral_table(1, [[400.0, 0.0123], [700.0, 0.0456]])
    tid = lens.surfaces[1].ar_layers
    lib = _native.load()
    rays = torch.from_numpy(_rays(lens.records(), 256, 1, 0.1)).cuda()
    out = torch.empty((256, 5), dtype=torch.float32, device="cuda")
    arr = lens.to_array()
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.gl_trace_rays_noalloc(arr, len(arr), 1, 8, C.c_void_p(rays.data_ptr()), 256,
                                   C.c_void_p(out.data_ptr()), C.c_void_p(st))
    assert rc != 0 and b"not resident" in lib.gl_last_error()
    K.prepare(tid)
    for s in lens.surfaces:
        if s.coating_model in K.TABLE_MODELS and s.ar_layers:
            K.prepare(s.ar_layers)
    rc = lib.gl_trace_rays_noalloc(arr, len(arr), 1, 8, C.c_void_p(rays.data_ptr()), 256,
                                   C.c_void_p(out.data_ptr()), C.c_void_p(st))
    assert rc == 0
    want = gl.trace_rays(lens, rays, 1, 8)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), want.cpu().numpy())

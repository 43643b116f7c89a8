"""PSF / veil convolution (FFT route) against the FP64 oracle."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _conv(imgs, k):
    from ghostlight_gb300 import _native
    lib = _native.load()
    H, W = imgs[0].shape
    kh, kw = k.shape
    st = torch.cuda.current_stream().cuda_stream
    h = C.c_void_p()
    kk = np.ascontiguousarray(k, np.float32)
    _native.check(lib.gl_conv2d_plan_create(W, H, kk.ctypes.data_as(C.POINTER(C.c_float)), kw, kh, st, C.byref(h)), "conv")
    ins = [torch.from_numpy(np.ascontiguousarray(i, np.float32)).cuda() for i in imgs]
    outs = [torch.full((H, W), float("nan"), device="cuda") for _ in range(3)]
    _native.check(lib.gl_conv2d_plan_execute(h, *[t.data_ptr() for t in ins], *[o.data_ptr() for o in outs], st), "conv")
    torch.cuda.synchronize()
    lib.gl_conv2d_plan_destroy(h)
    return [o.cpu().numpy() for o in outs]


@pytest.mark.parametrize("H,W,ks", [(200, 300, 31), (512, 512, 65), (97, 61, 9)])
def test_conv_matches_fp64(H, W, ks):
    from oracle import conv_oracle as CO
    rng = np.random.default_rng(H + W)
    imgs = [rng.random((H, W)).astype(np.float32) ** 4 for _ in range(3)]
    k = CO.psf_kernel(ks)
    got = _conv(imgs, k)
    for g, i in zip(got, imgs):
        assert rel_l2(g, CO.conv_same(i, k)) < 1e-5


def test_conv_full_size_2048_257_point_checks():
    """Configuration 3's convolution: 2048^2 x 3 channels with a 257^2 kernel,
    checked by direct FP64 sums at 64 pixels (incl. corners and edges)."""
    from oracle import conv_oracle as CO
    rng = np.random.default_rng(3)
    H = W = 2048
    imgs = [(rng.random((H, W)) ** 8).astype(np.float32) for _ in range(3)]
    k = CO.psf_kernel(257)
    got = _conv(imgs, k)
    ys = np.concatenate([[0, 0, 2047, 2047, 1024], rng.integers(0, H, 59)])
    xs = np.concatenate([[0, 2047, 0, 2047, 1024], rng.integers(0, W, 59)])
    for g, i in zip(got, imgs):
        want = CO.conv_at(i, k, ys, xs)
        assert np.isfinite(g).all()
        assert rel_l2(g[ys, xs], want) < 1e-5


def test_conv_plan_composite_add_matches_fp64():
    """execute(inputs, outputs, add=layer) convolves inputs + layer on load."""
    import ghostlight_gb300 as gl
    from oracle import conv_oracle as CO
    rng = np.random.default_rng(17)
    H, W = 300, 260
    a = [rng.random((H, W)).astype(np.float32) ** 3 for _ in range(3)]
    b = [rng.random((H, W)).astype(np.float32) ** 5 for _ in range(3)]
    k = CO.psf_kernel(33)
    plan = gl.ConvPlan(W, H, k)
    ta = [torch.from_numpy(x).cuda() for x in a]
    tb = [torch.from_numpy(x).cuda() for x in b]
    out = [torch.full((H, W), float("nan"), device="cuda") for _ in range(3)]
    assert plan.execute(ta, out, add=tb) == 3
    torch.cuda.synchronize()
    for o, x, y in zip(out, a, b):
        assert rel_l2(o.cpu().numpy(), CO.conv_same(x.astype(np.float64) + y, k)) < 1e-5
    with pytest.raises(ValueError):
        plan.execute(ta, out, add=[tb[0], tb[1], ta[0].t()])
    plan.close()

"""Tensor-core (tcgen05) building blocks and the matrix-DFT starburst."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 512), (512, 128, 1024)])
def test_tcgen05_bf16_gemm_matches_torch(M, N, K):
    from ghostlight_gb300 import _native
    lib = _native.load()
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    a = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    c = torch.full((M, N), float("nan"), device="cuda")
    _native.check(lib.gl_gemm_bf16_tc(a.data_ptr(), b.data_ptr(), c.data_ptr(), M, N, K,
                                      torch.cuda.current_stream().cuda_stream), "gemm")
    ref = a.float() @ b.float().t()
    err = (c - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err


def _mdft(n, K, n_lambda, form, seed=5):
    import ctypes as C
    from ghostlight_gb300 import _native
    from oracle import mdft_oracle as MO
    lib = _native.load()
    lam = np.linspace(420.0, 680.0, n_lambda)
    s0 = 1.0 / (2.0 * n)
    sx = (s0 * 550.0 / lam).astype(np.float64)
    sy = (s0 * 1.1 * 550.0 / lam).astype(np.float64)
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.2, 1.0, (n_lambda, 3)).astype(np.float32)
    cx, cy = K / 2.0 - 0.25, K / 2.0 + 0.5
    A = MO.test_pupil(n, seed)
    d = C.c_double
    h = C.c_void_p()
    st = torch.cuda.current_stream().cuda_stream
    _native.check(lib.gl_mdft_plan_create(n, K, n_lambda, (d * n_lambda)(*sx), (d * n_lambda)(*sy), cx, cy,
                                          (C.c_float * (3 * n_lambda))(*w.reshape(-1)), form, st, C.byref(h)), "mdft")
    dA = torch.from_numpy(A).cuda()
    outs = [torch.full((K, K), float("nan"), device="cuda") for _ in range(3)]
    _native.check(lib.gl_mdft_plan_execute(h, dA.data_ptr(), *[o.data_ptr() for o in outs], st), "mdft")
    torch.cuda.synchronize()
    code = C.c_int()
    lib.gl_mdft_plan_status(h, C.byref(code))
    lib.gl_mdft_plan_destroy(h)
    assert code.value == 0
    got = np.stack([o.cpu().numpy() for o in outs]).astype(np.float64)
    return got, (A, K, sx, sy, cx, cy, w)


@pytest.mark.parametrize("form,tol", [(0, 1e-3), (1, 2e-2), (2, 1e-4)])
def test_mdft_eform_matches_fp64_oracle(form, tol):
    from oracle import mdft_oracle as MO
    got, (A, K, sx, sy, cx, cy, w) = _mdft(128, 256, 3, form)
    want = MO.eform(A, K, sx, sy, cx, cy, w)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert np.isfinite(got).all() and err < tol, err


def test_mdft_config1_size_split_bf16():
    """Configuration 1: 256^2 pupil to 512^2 at 8 wavelengths."""
    from oracle import mdft_oracle as MO
    got, (A, K, sx, sy, cx, cy, w) = _mdft(256, 512, 8, 0)
    rows = np.arange(0, 512, 7)
    cols = np.arange(3, 512, 5)
    want = MO.eform(A, K, sx, sy, cx, cy, w, rows=rows, cols=cols)
    sub = got[:, rows][:, :, cols]
    err = np.linalg.norm(sub - want) / np.linalg.norm(want)
    assert err < 1e-3, err


def _inputs(n, n_lambda, seed=5):
    from oracle import mdft_oracle as MO
    lam = np.linspace(420.0, 680.0, n_lambda)
    s0 = 1.0 / (2.0 * n)
    sx = (s0 * 550.0 / lam).astype(np.float64)
    sy = (s0 * 1.1 * 550.0 / lam).astype(np.float64)
    w = np.random.default_rng(seed).uniform(0.2, 1.0, (n_lambda, 3)).astype(np.float32)
    return MO.test_pupil(n, seed), sx, sy, w


@pytest.mark.parametrize("form,tol", [("split_bf16", 1e-3), ("fp32", 1e-4)])
def test_rectangular_recentred_and_accumulated(form, tol):
    """Kx != Ky, a fractional off-frame centre set after creation, and the
    accumulate mode, against the FP64 oracle."""
    import ghostlight_gb300 as gl
    from oracle import mdft_oracle as MO
    n, Kx, Ky, L = 128, 384, 256, 3
    A, sx, sy, w = _inputs(n, L)
    plan = gl.MdftPlan(n, (Kx, Ky), sx, sy, w, form, center_x=10.0, center_y=20.0)
    cx, cy = 421.3771, -17.618                      # beyond the frame edge, sub-pixel
    assert plan.set_center(cx, cy) == 2
    base = [torch.full((Ky, Kx), 0.25, device="cuda") for _ in range(3)]
    dA = torch.from_numpy(A).cuda()
    plan.execute(dA, *base, accumulate=True)
    torch.cuda.synchronize()
    assert plan.status() == 0
    plan.close()
    got = np.stack([b.cpu().numpy() for b in base]).astype(np.float64) - 0.25
    want = MO.eform(A, (Kx, Ky), sx, sy, cx, cy, w)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert got.shape == (3, Ky, Kx) and err < tol, err


def test_far_centre_matches_oracle():
    """A centre far outside the frame (a source imaged beyond the sensor):
    the pattern's tail that reaches the frame, against the FP64 oracle."""
    import ghostlight_gb300 as gl
    from oracle import mdft_oracle as MO
    n, Kx, Ky, L = 128, 256, 256, 2
    A, sx, sy, w = _inputs(n, L, seed=5)
    dA = torch.from_numpy(A).cuda()
    for cx, cy in ((-9000.4, 130.0), (11800.75, -6000.5)):
        plan = gl.MdftPlan(n, (Kx, Ky), sx, sy, w, "split_bf16", center_x=cx, center_y=cy)
        out = [torch.zeros((Ky, Kx), device="cuda") for _ in range(3)]
        plan.execute(dA, *out)
        torch.cuda.synchronize()
        assert plan.status() == 0
        plan.close()
        got = np.stack([o.cpu().numpy() for o in out]).astype(np.float64)
        want = MO.eform(A, (Kx, Ky), sx, sy, cx, cy, w)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-3


def test_set_center_matches_fresh_plan():
    import ghostlight_gb300 as gl
    n, K, L = 128, 256, 2
    A, sx, sy, w = _inputs(n, L, seed=8)
    dA = torch.from_numpy(A).cuda()
    a = gl.MdftPlan(n, K, sx, sy, w, "split_bf16", center_x=77.5, center_y=140.25)
    b = gl.MdftPlan(n, K, sx, sy, w, "split_bf16", center_x=3.0, center_y=3.0)
    b.set_center(77.5, 140.25)
    oa = [torch.empty((K, K), device="cuda") for _ in range(3)]
    ob = [torch.empty((K, K), device="cuda") for _ in range(3)]
    a.execute(dA, *oa)
    b.execute(dA, *ob)
    torch.cuda.synchronize()
    for x, y in zip(oa, ob):
        assert torch.allclose(x, y, rtol=1e-6, atol=1e-6 * float(x.abs().max()))
    a.close(); b.close()


@pytest.mark.parametrize("blades,rot,aspect", [(6, 0.3, 1.0), (9, 0.0, 1.0), (0, 0.0, 1.5), (5, 1.1, 0.8)])
def test_stop_pupil_matches_oracle(blades, rot, aspect):
    """Device pupil builder vs the float32 restatement: supersample decisions
    may differ only where the float edge test is within rounding."""
    from ghostlight_gb300.prescriptions import double_gauss_12
    from ghostlight_gb300.optics import OpticalSystem
    from ghostlight_gb300.starburst import build_pupil
    from oracle import mdft_oracle as MO
    surfs = double_gauss_12()
    for s in surfs:
        if s.is_stop:
            s.aperture_aspect = aspect
            s.aperture_shape = 1 if blades >= 3 else 0
            s.aperture_blades = blades
            s.aperture_rotation_rad = rot
    lens = OpticalSystem.from_records(surfs)
    N, fill = 256, 0.45
    got = build_pupil(lens, N, fill).cpu().numpy()
    want = MO.stop_pupil(aspect, blades, rot, N, fill)
    diff = np.abs(got - want)
    assert got.sum() > 0.2 * N * N * 0.45 ** 2
    assert diff.max() <= 2.0 / 16.0 and (diff > 0).mean() < 2e-3


@pytest.mark.parametrize("form", [0, 2])
def test_mdft_wavelength_ranges_sum_to_the_whole(form):
    """A pattern enqueued as wavelength ranges (gl_mdft_plan_set_lambda_range,
    each execute accumulating) equals one execute over every wavelength."""
    from ghostlight_gb300.starburst import MdftPlan
    from oracle import mdft_oracle as MO
    n, K, nl = 128, 256, 7
    lam = np.linspace(420.0, 680.0, nl)
    s = (1.0 / (2.0 * n)) * 550.0 / lam
    w = np.random.default_rng(3).uniform(0.2, 1.0, (nl, 3)).astype(np.float32)
    A = torch.from_numpy(MO.test_pupil(n, 4)).cuda()
    plan = MdftPlan(n, K, s, s * 1.1, w, ["split_bf16", "tf32", "fp32"][form], center_x=K / 2 - 3.25, center_y=K / 2 + 1.5)
    whole = [torch.zeros((K, K), device="cuda") for _ in range(3)]
    plan.execute(A, *whole)
    parts = [torch.zeros((K, K), device="cuda") for _ in range(3)]
    for l0, l1 in ((0, 3), (3, 5), (5, 7)):
        plan.set_lambda_range(l0, l1)
        plan.execute(A, *parts, accumulate=True)
    plan.set_lambda_range(0, -1)
    torch.cuda.synchronize()
    assert plan.status() == 0
    a = torch.stack(whole).cpu().numpy().astype(np.float64)
    b = torch.stack(parts).cpu().numpy().astype(np.float64)
    assert a.sum() > 0 and np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-6
    with pytest.raises(ValueError):
        plan.set_lambda_range(5, 9)
    plan.close()


@pytest.mark.parametrize("form,tol", [("split_bf16", 1e-3), ("tf32", 2e-2)])
def test_output_tile_widths_agree_and_match_oracle(form, tol):
    """The second GEMM's output tile (128 or 64 complex columns per unit,
    gl_mdft_plan_set_tile): both widths give the same frame to float rounding
    (the same K blocks in the same order per output element) and match the
    FP64 oracle, on a rectangular frame with a recentred pattern, a
    wavelength range and the accumulate mode."""
    from ghostlight_gb300.starburst import MdftPlan
    from oracle import mdft_oracle as MO
    n, Kx, Ky, L = 128, 384, 256, 5
    A, sx, sy, w = _inputs(n, L)
    plan = MdftPlan(n, (Kx, Ky), sx, sy, w, form, center_x=Kx / 2 - 7.25, center_y=Ky / 2 + 3.5)
    dA = torch.from_numpy(A).cuda()
    got = {}
    for tile in (128, 64):
        plan.set_launch(0, tile)
        assert plan.launch == (0, tile)
        outs = [torch.full((Ky, Kx), 0.5, device="cuda") for _ in range(3)]
        plan.set_lambda_range(0, 2)
        plan.execute(dA, *outs, accumulate=True)
        plan.set_lambda_range(2, L)
        plan.execute(dA, *outs, accumulate=True)
        plan.set_lambda_range(0, -1)
        torch.cuda.synchronize()
        assert plan.status() == 0
        got[tile] = np.stack([o.cpu().numpy() for o in outs]).astype(np.float64) - 0.5
    want = MO.eform(A, (Kx, Ky), sx, sy, Kx / 2 - 7.25, Ky / 2 + 3.5, w)
    for tile in (128, 64):
        err = np.linalg.norm(got[tile] - want) / np.linalg.norm(want)
        assert err < tol, (tile, err)
    assert np.linalg.norm(got[64] - got[128]) / np.linalg.norm(got[128]) < 1e-6
    with pytest.raises(ValueError):
        plan.set_launch(0, 96)
    plan.close()

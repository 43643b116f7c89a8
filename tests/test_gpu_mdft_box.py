"""The reference's matrix-DFT engine (pixel-integrated form) on the device
against its FP64 restatement (oracle/mdft_box_oracle.py, itself pinned to the
reference's goldens by tests/test_mdft_box_oracle.py).

A 1024^2 pupil grid at fill 0.3 (a 9-blade curved stop, the compact
autocorrelation 625^2 lags), a 384 x 320 frame whose pattern window (half a
period, 2 x 97 + 1 pixels) is clamped by the frame edge for one of the three
sources, 8 wavelengths.  Tolerances (relative L2 of the frame): split-BF16
1e-4, TF32 2e-2, FP32 on the CUDA cores 1e-5; the autocorrelation itself
within 1e-5 of its zero-lag value.
"""
import math

import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _setup():
    import ghostlight_gb300 as gl
    from ghostlight_gb300 import prescriptions as P
    from ghostlight_gb300.starburst import build_pupil2
    lens = gl.OpticalSystem(P.double_gauss_12(seed=1))
    N, fill = 1024, 0.3
    pupil = build_pupil2(lens, N, fill, blades_override=9, rotation_deg=7.0)
    torch.cuda.synchronize()
    return lens, N, fill, pupil


def test_autocorrelation_matches_fp64():
    from ghostlight_gb300.starburst import SpritePlan, _round128
    from oracle import mdft_box_oracle as MB
    _, N, fill, pupil = _setup()
    mc = MB.support_radius(N, fill)
    n = _round128(2 * mc + 1)
    plan = SpritePlan(N, np.array([[550.0, 1.0, 1.0, 1.0]], np.float32))
    C = torch.full((n, n), 7.0, dtype=torch.float32, device="cuda")
    plan.autocorr(pupil, mc, C)
    torch.cuda.synchronize()
    got = C.cpu().numpy().astype(np.float64)
    want, mc2 = MB.autocorrelation(pupil.cpu().numpy(), fill)
    assert mc2 == mc
    Mc = 2 * mc + 1
    assert np.abs(got[:Mc, :Mc] - want.real).max() <= 1e-5 * want.real[mc, mc]
    assert float(np.abs(got[Mc:, :]).max()) == 0.0 and float(np.abs(got[:, Mc:]).max()) == 0.0
    plan.close()


@pytest.mark.parametrize("form,tol,tile", [("split_bf16", 1e-4, 128), ("split_bf16", 1e-4, 64), ("tf32", 2e-2, 128),
                                           ("tf32", 2e-2, 64), ("fp32", 1e-5, 128)])
def test_pixel_integrated_mdft_matches_fp64(form, tol, tile):
    from ghostlight_gb300.starburst import MdftPlan, SpritePlan, _round128
    from oracle import mdft_box_oracle as MB
    _, N, fill, pupil = _setup()
    mc = MB.support_radius(N, fill)
    n = _round128(2 * mc + 1)
    sp = SpritePlan(N, np.array([[550.0, 1.0, 1.0, 1.0]], np.float32))
    C = torch.empty((n, n), dtype=torch.float32, device="cuda")
    sp.autocorr(pupil, mc, C)
    W, H = 384, 320
    px_mm = 0.01
    dx = 2 * 97.5 * px_mm / N               # half a period = 97 pixels
    lam = np.linspace(420.0, 680.0, 8).astype(np.float32)
    spec = np.stack([lam, np.linspace(0.1, 0.3, 8), np.linspace(0.3, 0.2, 8), np.linspace(0.4, 0.05, 8)],
                    1).astype(np.float32)
    sources = np.array([[190.3, 161.7, 1.0, 0.8, 0.6], [20.6, 300.2, 0.5, 0.5, 0.9], [350.0, 40.4, 0.2, 1.0, 0.3]],
                       np.float32)
    gain = 3.0
    want = MB.render(pupil.cpu().numpy(), fill, spec, 550.0, dx, dx, px_mm, px_mm, sources, gain, W, H)
    f = np.float32
    Sx = f(f(N) * f(dx))
    half = max(1, int(math.floor(0.5 * float(Sx) / px_mm)))
    assert half == 97
    lam_scale = (spec[:, 0] / f(550.0)).astype(np.float32)
    s = px_mm / (Sx * lam_scale).astype(np.float32).astype(np.float64)
    k2 = ((f(550.0) / spec[:, 0]) ** 2).astype(np.float32)
    w = (spec[:, 1:4] * k2[:, None]).astype(np.float32)
    knorm = (px_mm * px_mm) / (dx * dx) * gain
    K = _round128(2 * half + 1)
    plan = MdftPlan(n, (K, K), s, s, w, form, center_x=0.0, center_y=0.0, box=True, red_center=float(mc))
    plan.set_launch(0, tile)                # output tile of the second GEMM: 128 or 64 columns
    out = [torch.zeros((H, W), dtype=torch.float32, device="cuda") for _ in range(3)]
    for (px, py, r, g, b) in sources:
        x0, x1 = max(0, int(math.floor(px)) - half), min(W, int(math.floor(px)) + half + 1)
        y0, y1 = max(0, int(math.floor(py)) - half), min(H, int(math.floor(py)) + half + 1)
        plan.set_center(float(px) - 0.5 - x0, float(py) - 0.5 - y0)
        plan.execute_window(C, *out, x0, y0, x1 - x0, y1 - y0, tint=(knorm * r, knorm * g, knorm * b))
    torch.cuda.synchronize()
    assert plan.status() == 0
    got = np.stack([o.cpu().numpy() for o in out]).astype(np.float64)
    assert want.sum() > 0
    err = rel_l2(got, want)
    assert err < tol, (form, err)
    plan.close()
    sp.close()

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

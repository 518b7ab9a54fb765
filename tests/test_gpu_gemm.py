"""The surrogate's tcgen05 BF16 GEMM (C = A B^T, FP32 accumulation) through
the C ABI against torch's FP32 product of the same BF16 operands."""
import ctypes

import pytest

from sfsim_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K,splits", [
    (128, 256, 64, 1), (256, 256, 256, 1), (200, 128, 512, 1), (384, 3, 256, 1), (128, 16, 64, 1),
    (128, 32, 128, 1), (512, 64, 192, 1), (256, 256, 4096, 8),
])
def test_gemm_matches_torch(M, N, K, splits):
    import torch
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.full((M, N), float("nan"), device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.sfsim_atmo_gemm_bf16(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K, splits, st), "gemm")
    torch.cuda.synchronize()
    ref = A.float() @ B.float().T
    err = (C - ref).abs().max().item() / ref.abs().max().item()
    assert torch.isfinite(C).all()
    assert err < 1e-4, err

"""Bounded waits of the tensor-core kernels, exercised on the GPU without a
fault or a hang.

sfsim_atmo_wait_selftest launches the GEMM kernel with its epilogue waiting a
few polls on an mbarrier that nothing arrives on.  The wait gives up, the CTA
takes its timeout path (error recorded, the other warps told to stop, copies
and MMAs in flight drained under the full limit, tensor memory freed) and the
call reports SFSIM_ATMO_ECUDA.  The next GEMM on the same device must run and
be correct.  The run-time poll limit (sfsim_atmo_set_wait_limit) is exercised
the same way: a GEMM under a lowered limit that is still ample."""
import pytest

from sfsim_gb300 import _lib

pytestmark = pytest.mark.gpu

ECUDA = -3


def _gemm_error(L, M, N, K, seed):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.full((M, N), float("nan"), device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.sfsim_atmo_gemm_bf16(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K, 1, st), "gemm")
    torch.cuda.synchronize()
    ref = A.float() @ B.float().T
    assert torch.isfinite(C).all()
    return (C - ref).abs().max().item() / ref.abs().max().item()


def test_timed_out_wait_is_reported_and_the_device_stays_usable():
    L = _lib.load()
    for polls in (4, 64):
        rc = L.sfsim_atmo_wait_selftest(polls)
        assert rc == ECUDA, rc
        assert b"timed out" in L.sfsim_atmo_last_error()
        # the same kernel right after the timeout: correct results
        assert _gemm_error(L, 256, 256, 1024, polls) < 1e-4


def test_selftest_rejects_bad_poll_counts():
    L = _lib.load()
    assert L.sfsim_atmo_wait_selftest(0) == -1
    assert L.sfsim_atmo_wait_selftest(10 ** 7) == -1


def test_runtime_wait_limit():
    L = _lib.load()
    default = L.sfsim_atmo_set_wait_limit(1 << 16)
    try:
        assert default == 1 << 22
        assert _gemm_error(L, 384, 128, 512, 5) < 1e-4
        assert L.sfsim_atmo_set_wait_limit(0) == 1 << 16
    finally:
        L.sfsim_atmo_set_wait_limit(0)
    assert L.sfsim_atmo_set_wait_limit(0) == 1 << 22

"""The allocation-free entry point, sfsim_atmo_build_static.

It exists for callers that cannot call cudaMalloc: engines whose allocator
reserves all device memory at start-up, or that run under a fixed device
budget.  Its scratch is a fixed static device array inside the library.  This
test calls it twice in a row through the C ABI and checks both results
against the allocating entry point, sfsim_atmo_build_device.  FP64 builds run
the same kernels and must agree within 1e-12 relative (bit for bit in
practice).  FP32 builds must agree within 2e-5: an allocating FP32 build of
a larger configuration reads the sun rays' optical depths from a table where
the static build integrates every sun ray directly (at this test's size both
integrate directly).  The two static calls must agree bit for bit.  The file name sorts last so that a run stopping at its first failure
has run every other test before this one.
"""
import ctypes

import numpy as np
import pytest

from sfsim_gb300 import _lib, atmosphere_lut as A, config as C

pytestmark = pytest.mark.gpu


def _build(fn, cfg, stream):
    import torch
    outs = [torch.full(s, -1.0, dtype=torch.float32, device="cuda") for s in A.table_shapes(cfg)]
    _lib.check(fn(ctypes.byref(cfg), *[t.data_ptr() for t in outs], ctypes.c_void_p(stream.cuda_stream)), fn.__name__)
    return outs


def _rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    floor = 1e-6 * max(np.abs(b).max(), 1e-300)
    return float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max())


@pytest.mark.parametrize("precision", [C.FP32, C.FP64])
def test_static_build_matches_allocating_build(precision):
    import torch
    L = _lib.load()
    cfg = C.small_fp64(precision=precision)
    stream = torch.cuda.current_stream()
    ref = _build(L.sfsim_atmo_build_device, cfg, stream)
    first = _build(L.sfsim_atmo_build_static, cfg, stream)
    second = _build(L.sfsim_atmo_build_static, cfg, stream)
    torch.cuda.synchronize()
    # the static build integrates every sun ray directly; an allocating FP32
    # build above the sun table's size threshold reads them from the table,
    # within 2e-5
    tol = 2e-5 if precision == C.FP32 else 1e-12
    for r, a, b in zip(ref, first, second):
        assert torch.isfinite(a).all() and torch.isfinite(b).all()
        assert _rel(a, r) <= tol
        assert torch.equal(a, b)


def test_static_build_rejects_oversize():
    import torch
    L = _lib.load()
    cfg = C.production()
    x = torch.zeros(4, dtype=torch.float32, device="cuda")
    rc = L.sfsim_atmo_build_static(ctypes.byref(cfg), *([x.data_ptr()] * 4),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -7
    assert b"static array" in L.sfsim_atmo_last_error()

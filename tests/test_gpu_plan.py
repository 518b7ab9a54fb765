"""Plans (sfsim_atmo_plan_*): a build prepared once, whose build call only
launches kernels.  Its tables equal the allocating entry point's bit for bit,
and a torch CUDA graph captured from it rebuilds them on every replay."""
import numpy as np
import pytest

from sfsim_gb300 import atmosphere_lut as A
from sfsim_gb300 import config as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [C.FP32, C.FP64])
def test_plan_build_equals_device_build(precision):
    import torch
    cfg = C.small_fp64(precision=precision)
    ref = A.build_device(cfg)
    plan = A.Plan(cfg)
    out = plan.build()
    torch.cuda.synchronize()
    for r, o in zip(ref, out):
        assert torch.equal(r, o)
    plan.close()


def test_plan_build_replays_in_a_cuda_graph():
    import torch
    cfg = C.small_fp64(precision=C.FP32)
    ref = A.build_device(cfg)
    torch.cuda.synchronize()
    plan = A.Plan(cfg)
    outs = [torch.empty(s, dtype=torch.float32, device="cuda") for s in A.table_shapes(cfg)]
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        plan.build(outs, stream=side)  # one build outside the capture
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.build(outs, stream=torch.cuda.current_stream())
    for _ in range(3):
        for t in outs:
            t.fill_(-1.0)
        g.replay()
        torch.cuda.synchronize()
        for r, o in zip(ref, outs):
            assert torch.equal(r, o)
    plan.close()


def test_plan_of_unsupported_shape_is_refused():
    from sfsim_gb300 import _lib
    cfg = C.small_fp64(precision=C.FP32)
    for i, v in enumerate((4, 8, 64, 64)):
        cfg.ray_scatter_shape[i] = v
    with pytest.raises(_lib.AtmoError) as e:
        A.Plan(cfg)
    assert e.value.code == -5
    assert np.isfinite(A.build(C.small_fp64(precision=C.FP32))["transmittance"]).all()

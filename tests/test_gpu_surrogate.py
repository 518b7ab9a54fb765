"""The ray-scatter surrogate: gradients of the GPU's tensor-core forward and
backward passes against a float64 reference, training on the GPU, and what
the trained network gains over the lookup table and over direct quadrature."""
import numpy as np
import pytest

from sfsim_gb300 import config as C
from sfsim_gb300.query import Context
from tests.mlp_reference import forward, loss_and_grads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(C.small_fp64(precision=C.FP32))
    yield c
    c.close()


def test_gradients_match_reference(ctx):
    rng = np.random.default_rng(3)
    n = 2048
    coords = rng.uniform(0, 1, (n, 10)).astype(np.float32)
    targets = rng.normal(0, 0.5, (n, 3)).astype(np.float32)
    params = ctx.surrogate_parameters()
    loss, grads = ctx.surrogate_gradients(coords, targets)
    rloss, rgrads = loss_and_grads(params, coords, targets)
    assert abs(loss - rloss) <= 1e-3 * abs(rloss)
    # per tensor: relative norm of the difference
    from tests.mlp_reference import SHAPES
    o = 0
    for (r, c) in SHAPES:
        for size in (r * c, r):
            g, rg = grads[o:o + size], rgrads[o:o + size]
            o += size
            rel = np.linalg.norm(g - rg) / max(np.linalg.norm(rg), 1e-30)
            assert rel < 2e-2, (r, c, size, rel)
    assert o == grads.size


def random_queries(cfg, n, seed):
    rng = np.random.default_rng(seed)
    h = rng.uniform(0.0, cfg.height, n)

    def unit(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)
    return unit(n) * (cfg.radius + h)[:, None], unit(n), unit(n)


def test_training_reduces_loss_and_surrogate_gains(ctx):
    """Trained on direct-quadrature samples, the corrected lookup is closer to
    the direct quadrature than the table alone; with a threshold the points
    whose predicted error exceeds it are recomputed by quadrature exactly."""
    import torch
    hist = ctx.train_surrogate(steps=600, batch=16384, direct_samples=1 << 18, node_fraction=0.0, lr=2e-3, seed=5)
    assert np.isfinite(hist).all()
    assert hist[-50:].mean() < 0.2 * hist[:10].mean(), (hist[:10].mean(), hist[-50:].mean())
    cfg = ctx.cfg
    x, v, l = random_queries(cfg, 4096, 11)
    xt, vt, lt = (torch.tensor(z, dtype=torch.float64, device="cuda") for z in (x, v, l))
    direct = ctx.direct(xt, vt, lt).cpu().numpy()
    x32, v32, l32 = (torch.tensor(z, dtype=torch.float32, device="cuda") for z in (x, v, l))
    table = ctx.table(4, x32, v32, l32).cpu().numpy()
    sur, nf0 = ctx.surrogate(xt, vt, lt)
    sur = sur.cpu().numpy()
    assert nf0 == 0
    floor = 1e-6 * np.abs(direct).max()

    def err(a):
        return (np.abs(a - direct) / np.maximum(np.abs(direct), floor)).max(axis=1)
    e_table, e_sur = err(table), err(sur)
    assert np.median(e_sur) < np.median(e_table), (np.median(e_sur), np.median(e_table))
    counts = []
    for t in (1.0, 0.3, 0.1, 0.03, 0.01):
        fb, nf = ctx.surrogate(xt, vt, lt, threshold=t)
        e_fb = err(fb.cpu().numpy())
        # flagged points carry the quadrature's value, the others the surrogate's
        assert np.all((e_fb == 0) | (e_fb == e_sur))
        assert np.sum(e_fb == 0) >= nf
        assert np.percentile(e_fb, 90) <= np.percentile(e_sur, 90)
        counts.append(nf)
    # a tighter threshold never flags fewer points, and the estimate separates
    assert all(a <= b for a, b in zip(counts, counts[1:])), counts
    assert any(0 < c < 4096 for c in counts), counts


def test_fused_inference_matches_reference(ctx):
    """The fused tensor-core inference kernel against the float64 forward pass
    at the coordinates the GPU forms for the same queries: the correction it
    applies to the table lookup."""
    import torch
    params = ctx.surrogate_parameters()  # also creates an untrained surrogate when run alone
    cfg = ctx.cfg
    x, v, l = random_queries(cfg, 1000, 21)
    xt, vt, lt = (torch.tensor(z, dtype=torch.float64, device="cuda") for z in (x, v, l))
    coords = ctx.coords(xt, vt, lt).cpu().numpy()
    assert np.all((coords >= 0) & (coords <= 1))
    out, nf = ctx.surrogate(xt, vt, lt)
    x32, v32, l32 = (torch.tensor(z, dtype=torch.float32, device="cuda") for z in (x, v, l))
    table = np.maximum(ctx.table(4, x32, v32, l32).cpu().numpy().astype(np.float64), 0)
    eps = 1e-7
    out = out.cpu().numpy().astype(np.float64)
    r = np.log(out + eps) - np.log(table + eps)
    ref = forward(params, coords)[:, :3]
    mask = out > 1e-5  # well above the offset eps, where the log resolves the correction
    assert mask.sum() > 100
    assert np.abs(r - ref)[mask].max() < 2e-2, float(np.abs(r - ref)[mask].max())

"""The conditioned surrogate (one network for a family of atmospheres, eight
atmosphere inputs in its first layer): gradients against the float64
reference, the fused inference kernel with the inputs folded into its bias,
and what the trained network gains on an atmosphere it was not trained on."""
import numpy as np
import pytest

from sfsim_gb300 import config as C
from sfsim_gb300.query import ConditionedSurrogate, Context, condition_inputs
from tests.mlp_reference import SHAPES, forward, loss_and_grads
from tests.test_gpu_surrogate import random_queries

pytestmark = pytest.mark.gpu


def small_sweep(n, seed):
    return C.parameter_sweep(n, seed=seed, precision=C.FP32, ray_scatter_shape=(8, 16, 8, 4),
                             transmittance_shape=(32, 32), surface_radiance_shape=(16, 32), ray_steps=64,
                             sphere_steps=16, iterations=2)


def test_cond_gradients_match_reference():
    cs = ConditionedSurrogate(seed=3)
    rng = np.random.default_rng(4)
    params = cs.parameters()
    n_plain = sum(r * c + r for (r, c) in SHAPES)
    assert params.size == n_plain + 256 * 8
    assert np.all(params[n_plain:] == 0)
    params[n_plain:] = rng.normal(0, 0.3, 256 * 8)  # exercise the conditioning term
    cs.parameters(set_to=params)
    n, groups = 2048, 5
    coords = rng.uniform(0, 1, (n, 10)).astype(np.float32)
    grp = rng.integers(0, groups, n).astype(np.int32)
    inputs = rng.uniform(-1, 1, (groups, 8)).astype(np.float32)
    targets = rng.normal(0, 0.5, (n, 3)).astype(np.float32)
    loss, grads = cs.gradients(coords, grp, inputs, targets)
    rloss, rgrads = loss_and_grads(params, coords, targets, groups=grp, inputs=inputs)
    assert abs(loss - rloss) <= 1e-3 * abs(rloss)
    assert grads.size == rgrads.size
    o = 0
    sizes = [s for (r, c) in SHAPES for s in (r * c, r)] + [256 * 8]
    for size in sizes:
        g, rg = grads[o:o + size], rgrads[o:o + size]
        o += size
        rel = np.linalg.norm(g - rg) / max(np.linalg.norm(rg), 1e-30)
        assert rel < 2e-2, (size, rel)
    assert o == grads.size
    cs.close()


@pytest.fixture(scope="module")
def family():
    cfgs = small_sweep(7, seed=77)
    ctxs = [Context(c) for c in cfgs]
    yield cfgs, ctxs
    for c in ctxs:
        c.close()


def test_cond_inference_matches_reference(family):
    """Fused inference with the atmosphere's inputs folded into the first-layer
    bias against the float64 forward pass of the conditioned network."""
    import torch
    cfgs, ctxs = family
    cs = ConditionedSurrogate(seed=9)
    rng = np.random.default_rng(6)
    params = cs.parameters()
    n_plain = sum(r * c + r for (r, c) in SHAPES)
    params[n_plain:] = rng.normal(0, 0.3, 256 * 8)
    cs.parameters(set_to=params)
    cfg, ctx = cfgs[0], ctxs[0]
    x, v, l = random_queries(cfg, 1000, 23)
    xt, vt, lt = (torch.tensor(z, dtype=torch.float64, device="cuda") for z in (x, v, l))
    coords = ctx.coords(xt, vt, lt).cpu().numpy()
    out, nf = cs.query(ctx, xt, vt, lt)
    assert nf == 0
    x32, v32, l32 = (torch.tensor(z, dtype=torch.float32, device="cuda") for z in (x, v, l))
    table = np.maximum(ctx.table(4, x32, v32, l32).cpu().numpy().astype(np.float64), 0)
    eps = 1e-7
    out = out.cpu().numpy().astype(np.float64)
    r = np.log(out + eps) - np.log(table + eps)
    ref = forward(params, coords, inputs=condition_inputs(cfg))[:, :3]
    plain = forward(params[:n_plain], coords)[:, :3]
    mask = out > 1e-5
    assert mask.sum() > 100
    assert np.abs(r - ref)[mask].max() < 2e-2, float(np.abs(r - ref)[mask].max())
    # the inputs matter: without them the network gives other corrections
    assert np.abs(plain - ref)[mask].max() > 1e-2
    cs.close()


def test_cond_training_gains_on_held_out_atmosphere(family):
    """Trained on six atmospheres of the sweep, the network corrects the table
    lookup of a seventh that it never saw: its median error is below the
    table's.  Points above a threshold go to that atmosphere's quadrature."""
    import torch
    cfgs, ctxs = family
    cs = ConditionedSurrogate(seed=5)
    hist = cs.train(ctxs[:6], steps=800, batch=16384, direct_samples=1 << 16, node_fraction=0.0, lr=2e-3, seed=7)
    assert np.isfinite(hist).all()
    assert hist[-50:].mean() < 0.25 * hist[:10].mean(), (hist[:10].mean(), hist[-50:].mean())
    cfg, ctx = cfgs[6], ctxs[6]
    x, v, l = random_queries(cfg, 4096, 31)
    xt, vt, lt = (torch.tensor(z, dtype=torch.float64, device="cuda") for z in (x, v, l))
    direct = ctx.direct(xt, vt, lt).cpu().numpy()
    x32, v32, l32 = (torch.tensor(z, dtype=torch.float32, device="cuda") for z in (x, v, l))
    table = ctx.table(4, x32, v32, l32).cpu().numpy()
    sur, nf0 = cs.query(ctx, xt, vt, lt)
    assert nf0 == 0
    floor = 1e-6 * np.abs(direct).max()

    def err(a):
        return (np.abs(a - direct) / np.maximum(np.abs(direct), floor)).max(axis=1)
    e_table, e_sur = err(table), err(sur.cpu().numpy())
    assert np.median(e_sur) < 0.8 * np.median(e_table), (np.median(e_sur), np.median(e_table))
    fb, nf = cs.query(ctx, xt, vt, lt, threshold=0.03)
    e_fb = err(fb.cpu().numpy())
    assert np.all((e_fb == 0) | (e_fb == e_sur))
    assert np.sum(e_fb == 0) >= nf
    cs.close()

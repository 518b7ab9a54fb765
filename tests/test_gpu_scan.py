"""GPU parity of the SCAN_RAYS build mode (view-ray transmittances by one
warp-shuffle prefix scan per ray) against the oracle's restatement of the
same discretisation, and its deviation from the reference's nested
quadrature at production size.

Relative errors as in test_gpu_parity: |gpu - ref| / max(|ref|, 1e-6 max|ref|).
Tolerances: FP64 build 2e-6, FP32 build 1e-4 (the parity-mode bounds).
"""
import numpy as np
import pytest

from oracle import oracle as O
from sfsim_gb300 import _lib
from sfsim_gb300 import atmosphere_lut as A
from sfsim_gb300 import config as C

pytestmark = pytest.mark.gpu

TOL = {C.FP64: 2e-6, C.FP32: 1e-4}


def rel_err(gpu, ref):
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    floor = 1e-6 * max(np.abs(ref).max(), 1e-300)
    err = np.abs(gpu - ref) / np.maximum(np.abs(ref), floor)
    return float(err.max()), float(err.mean())


def assert_close(gpu, ref, tol, name):
    assert np.isfinite(gpu).all(), f"{name}: non-finite values"
    mx, mean = rel_err(gpu, ref)
    assert mx <= tol, f"{name}: max rel err {mx:.3e} (mean {mean:.3e}) > {tol:.1e}"


def scan_config(precision, ray_steps=64, shape=(8, 16, 8, 4)):
    return C.make_config(height=100000.0, transmittance_shape=(32, 32), surface_radiance_shape=(16, 32),
                         ray_scatter_shape=shape, ray_steps=ray_steps, sphere_steps=16, iterations=2,
                         precision=precision, flags=C.SCAN_RAYS)


@pytest.fixture(scope="module")
def scan_oracle():
    return O.build(scan_config(C.FP64), intermediates=True)


@pytest.mark.parametrize("precision", [C.FP64, C.FP32])
def test_scan_build_matches_oracle(scan_oracle, precision):
    """Every intermediate and final table of a 2-iteration scan-mode build."""
    cfg = scan_config(precision)
    gpu = A.build(cfg, intermediates=True)
    tol = TOL[precision]
    for key in ("transmittance_nodes", "surface_base", "rayleigh_first", "mie_first"):
        assert_close(gpu[key], scan_oracle[key], tol, key)
    for it in range(cfg.iterations):
        for key in ("point_scatter", "surface_delta", "ray_scatter_delta"):
            assert_close(gpu[key][it], scan_oracle[key][it], tol, f"{key}[{it}]")
    for key in ("transmittance", "surface_radiance", "ray_scatter", "mie_strength"):
        assert_close(gpu[key], scan_oracle[key], tol, key)


@pytest.mark.parametrize("ray_steps", [4, 21, 32, 70])
def test_scan_ragged_rays(ray_steps):
    """Ray lengths that are below, at and between multiples of the 32 lanes
    of one scan (a partial last chunk, one whole chunk, three chunks)."""
    cfg = scan_config(C.FP64, ray_steps=ray_steps, shape=(5, 9, 7, 5))
    cfg.iterations = 1
    ref = O.build(cfg, intermediates=True)
    gpu = A.build(cfg, intermediates=True)
    for key in ("rayleigh_first", "mie_first"):
        assert_close(gpu[key], ref[key], TOL[C.FP64], key)
    for key in ("ray_scatter", "mie_strength", "surface_radiance"):
        assert_close(gpu[key], ref[key], TOL[C.FP64], key)


def test_scan_batch_and_flag_mix():
    """A batch shares its flags; the scan build of a batch member equals its
    single build, and a batch that mixes flags is refused."""
    a, b = scan_config(C.FP32), scan_config(C.FP32)
    b.radius = 6000000.0
    batch = A.build_batch([a, b])
    single = A.build(b)
    for key in ("ray_scatter", "mie_strength"):
        assert np.array_equal(batch[key][1], single[key])
    c = scan_config(C.FP32)
    c.flags = 0
    with pytest.raises(_lib.AtmoError) as e:
        A.build_batch([a, c])
    assert e.value.code == -1


def test_scan_production_deviation():
    """At production size the scan mode stays within 1e-2 of the nested FP64
    tables (the step error of either quadrature at 128 steps is larger) and
    leaves the transmittance table as the nested FP32 build has it."""
    cfg = C.production()
    cfg.flags = C.SCAN_RAYS
    scan = A.build(cfg)
    nested = A.build(C.production())
    ref = A.build(C.production(precision=C.FP64))
    assert np.array_equal(scan["transmittance"], nested["transmittance"])
    for key in ("surface_radiance", "ray_scatter", "mie_strength"):
        mx, mean = rel_err(scan[key], ref[key])
        assert mx < 1e-2 and mean < 1e-3, (key, mx, mean)

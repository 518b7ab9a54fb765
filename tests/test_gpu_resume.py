"""Iteration states and resume (sfsim_atmo_build_resumable).

A state saved after any iteration resumes a build that ends with exactly the
tables of an uninterrupted build: the state holds the build's own node
values, so nothing is re-rounded.  A callback that stops the build leaves a
state from which the build resumes, through a file.
"""
import numpy as np
import pytest

from sfsim_gb300 import _lib
from sfsim_gb300 import atmosphere_lut as A
from sfsim_gb300 import config as C

pytestmark = pytest.mark.gpu

KEYS = ("transmittance", "surface_radiance", "ray_scatter", "mie_strength")


def resume_config(precision):
    return C.make_config(height=100000.0, transmittance_shape=(17, 33), surface_radiance_shape=(8, 16),
                         ray_scatter_shape=(8, 17, 8, 4), ray_steps=32, sphere_steps=12, iterations=4,
                         precision=precision)


def assert_same(a, b):
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("precision", [C.FP32, C.FP64])
def test_resume_after_every_iteration_matches_uninterrupted(precision):
    cfg = resume_config(precision)
    ref = A.build(cfg)
    states = {}

    def keep(iteration, tables):
        states[iteration] = {k: v.copy() for k, v in tables.items()}
    assert_same(A.build_resumable(cfg, on_iteration=keep), ref)
    assert sorted(states) == list(range(1, cfg.iterations + 1))
    # every iteration changes the sums (they are re-interpolated, not only added to)
    for k in range(2, cfg.iterations + 1):
        assert not np.array_equal(states[k]["ray_scatter_sum"], states[k - 1]["ray_scatter_sum"])
        assert not np.array_equal(states[k]["surface_sum"], states[k - 1]["surface_sum"])
    for k in range(1, cfg.iterations + 1):
        assert_same(A.build_resumable(cfg, resume=(k, states[k])), ref)


def test_stop_then_resume_from_file(tmp_path):
    cfg = resume_config(C.FP32)
    ref = A.build(cfg)
    path = str(tmp_path / "iteration2.npz")

    def stop_after_two(iteration, tables):
        A.save_iteration_state(path, iteration, tables)
        return iteration == 2
    with pytest.raises(_lib.AtmoError) as err:
        A.build_resumable(cfg, on_iteration=stop_after_two)
    assert err.value.code == -9
    iteration, tables = A.load_iteration_state(path)
    assert iteration == 2
    seen = []
    out = A.build_resumable(cfg, resume=(iteration, tables), on_iteration=lambda i, t: seen.append(i))
    assert seen == [3, 4]
    assert_same(out, ref)


def test_callback_exception_stops_the_build():
    cfg = resume_config(C.FP32)

    def boom(iteration, tables):
        raise KeyError("from the callback")
    with pytest.raises(KeyError):
        A.build_resumable(cfg, on_iteration=boom)
    # the library is usable afterwards
    assert_same(A.build_resumable(cfg), A.build(cfg))

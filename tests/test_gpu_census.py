"""The work census (sfsim_atmo_census) that the bench's roofline counts
algorithmic bytes and exponentials with: its point-scatter direction counts
against the oracle's own sphere quadrature and ray geometry
(sphere.clj:62-105, atmosphere.clj:70-111), and the inclusions between its
counts."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from sfsim_gb300 import _lib
from sfsim_gb300 import config as C

pytestmark = pytest.mark.gpu


def oracle_ground_directions(cfg):
    """Per height row: sphere directions whose ray ends on the ground, and
    those of them whose ground point has height coordinate exactly 0 in the
    surface-radiance table."""
    R, H = cfg.radius, cfg.height
    p = O.planet(R, H)
    n0, nE0 = cfg.ray_scatter_shape[0], cfg.surface_radiance_shape[0]
    steps = cfg.sphere_steps
    dirs = []
    for k in range(steps >> 1):
        th = np.pi * (0.5 + k) / (steps >> 1)
        m = int(np.ceil(np.sin(th) * steps))
        for q in range(m):
            ph = 2 * np.pi * (0.5 + q) / m
            dirs.append((np.cos(th), np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph)))
    assert len(dirs) == O.sphere_directions(steps)
    ground = flat = 0
    for i in range(n0):
        r = np.linalg.norm(O.index_to_height(p, n0, i))
        x = np.array([r, 0.0, 0.0])
        n = x / r
        o1 = O.orthogonal(n)
        o2 = np.cross(n, o1)
        for d in dirs:
            g = O.ray_extremity(p, x, n * d[0] + o1 * d[1] + o2 * d[2])
            if O.surface_point(p, g):
                ground += 1
                flat += O.height_to_index(p, nE0, g) == 0.0
    return ground, flat


def test_census_counts():
    cfg = C.small_fp64(precision=C.FP32)
    L = _lib.load()
    counts = (ctypes.c_ulonglong * 10)()
    assert L.sfsim_atmo_census(ctypes.byref(cfg), counts, 10) == 10
    c = list(counts)
    n0, n1, n2, n3 = cfg.ray_scatter_shape
    it = cfg.iterations
    P = O.sphere_directions(cfg.sphere_steps)
    per_height = n1 * n2 * n3
    assert c[3] == n0 * per_height * P * it
    assert c[8] == n0 * per_height * P
    ground, flat = oracle_ground_directions(cfg)
    # the GPU set-up classifies ground ends in FP64 like the oracle; allow a
    # direction of slack per height for rays that graze the horizon
    assert abs(c[7] - ground * per_height * it) <= n0 * per_height * it
    assert 0 < c[9] <= c[7] <= c[3]
    assert abs(c[9] - flat * per_height * it) <= 2 * n0 * per_height * it
    assert c[6] <= c[0] and c[1] == c[0] * cfg.ray_steps

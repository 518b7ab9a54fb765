"""LUT end-to-end pin of the oracle: the reference's shader tests
(test/clj/sfsim/t_atmosphere.clj:569-775) build 12x12 transmittance and 12^4
ray-scatter tables on the CPU with 10 ray steps in a 100 km atmosphere, upload
them as GL textures and query them through the atmosphere shaders.  The GLSL is
restated in FP32 in oracle/atmo_oracle.c; the expected values are the
reference's.  With the 8-bit fixed-point bilinear weights of GL texture
filtering the restatement matches to 1e-6; with exact weights it stays inside
the reference's own 1e-4 tolerance.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sfsim_gb300 import config as C

N = 12


@pytest.fixture(scope="module")
def tables():
    cfg = C.shader_test()
    T = np.zeros((N, N, 3))
    for i in range(N):
        for j in range(N):
            T[i, j] = O.transmittance_node(cfg, i, j)
    S4 = np.zeros((N, N, N, N, 3))
    for i in range(N):
        for j in range(N):
            for k in range(N):
                for a in range(N):
                    # t_atmosphere.clj:174-175: S and M both use the Rayleigh point scatter
                    S4[i, j, k, a] = O.first_order_node(cfg, i, j, k, a)[0]
    # convert-4d-to-2d (image.clj:299-312)
    S2 = S4.transpose(0, 2, 1, 3, 4).reshape(N * N, N * N, 3)
    return dict(transmittance=T, ray_scatter=S2, mie_strength=S2, radius=6378000.0, max_height=100000.0,
                transmittance_shape=(N, N), ray_scatter_shape=(N, N, N, N))


TRACK = [((0, 0, 6478000), (0, 0, 6478000), 1.0),
         ((0, 0, 6378000), (0, 0, 6478000), 0.976549),
         ((6378000, 0, 0), (6378000, 0, 100000), 0.079658)]          # t_atmosphere.clj:629-635
OUTER = [((0, 0, 6478000), (0, 0, 1), 0.976359),
         ((0, 0, 6378000), (0, 0, 1), 0.953463),
         ((0, 0, 6378000), (1, 0, 0), 0.016916)]                     # t_atmosphere.clj:661-667
SCATTER = [((0, 0, 6378000), (0, 0, 6378000), 0.0),
           ((0, 0, 6378000), (0, 0, 6478000), 0.043302),
           ((0, 0, 6378000), (100000, 0, 6378000), 0.008272)]        # t_atmosphere.clj:769-775


@pytest.mark.parametrize("bits,tol", [(8, 2e-6), (0, 1e-4)])
def test_transmittance_track(tables, bits, tol):
    for p, q, r in TRACK:
        assert abs(O.glsl_query(tables, 0, (0, 0, 1), p, q, bits)[0] - r) <= tol


@pytest.mark.parametrize("bits,tol", [(8, 2e-6), (0, 1e-4)])
def test_transmittance_outer(tables, bits, tol):
    for p, d, r in OUTER:
        assert abs(O.glsl_query(tables, 1, (0, 0, 1), p, d, bits)[0] - r) <= tol


@pytest.mark.parametrize("bits,tol", [(8, 2e-6), (0, 1e-4)])
def test_ray_scatter_track(tables, bits, tol):
    for p, q, r in SCATTER:
        assert abs(O.glsl_query(tables, 2, (0, 0, 1), p, q, bits)[2] - r) <= tol

"""The GPU cloud-noise builders (include/sfsim_noise.h) against the FP64
oracle on the same random inputs: Worley and Perlin noise to FP32 accuracy,
blue-noise ranks exactly; plus the reference's own facts
(test/clj/sfsim/t_worley.clj:76-80, t_perlin.clj:143-148,
t_bluenoise.clj:111-124)."""
import numpy as np
import pytest

from oracle import oracle as O
from sfsim_gb300 import noise

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("divisions,size,seed", [(1, 2, 0), (4, 16, 1), (3, 12, 2), (8, 64, 3), (16, 32, 4)])
def test_worley_matches_oracle(divisions, size, seed):
    grid = noise.random_point_grid(divisions, size, np.random.default_rng(seed))
    gpu = noise.worley_noise(divisions, size, grid=grid)
    ref = O.worley(divisions, size, grid)
    assert gpu.shape == ref.shape
    assert np.abs(gpu - ref).max() < 2e-6, float(np.abs(gpu - ref).max())
    assert gpu.min() == pytest.approx(0.0, abs=1e-6) and gpu.max() <= 1.0


def test_worley_fact():
    out = noise.worley_noise(1, 2, grid=np.array([[[[0.5, 0.5, 0.5]]]]))
    assert out[0] == 1.0 and out.size == 8 and out.min() == 0.0


@pytest.mark.parametrize("divisions,size,seed", [(2, 4, 0), (4, 16, 1), (3, 12, 2), (8, 64, 3), (5, 40, 4)])
def test_perlin_matches_oracle(divisions, size, seed):
    grad = noise.random_gradient_grid(divisions, np.random.default_rng(seed))
    gpu = noise.perlin_noise(divisions, size, gradients=grad)
    ref = O.perlin(divisions, size, grad)
    assert np.abs(gpu - ref).max() < 1e-5, float(np.abs(gpu - ref).max())
    assert gpu.min() == 0.0 and gpu.max() == 1.0


def test_perlin_fact():
    from tests.test_noise_oracle import FACT_GRID
    out = noise.perlin_noise(2, 4, gradients=np.array(FACT_GRID))
    assert out[0] == pytest.approx(0.74821, abs=1e-5)
    assert out.size == 64


@pytest.mark.parametrize("m,seed", [(2, 0), (8, 1), (16, 2), (64, 3), (136, 4)])
def test_blue_noise_matches_oracle_exactly(m, seed):
    # 136 x 136 does not fit in shared memory: the global-memory path
    n = max(1, (m * m) // 10)
    pixels = np.random.default_rng(seed).permutation(m * m)[:n]
    gpu = noise.blue_noise(m, sigma=1.5, seed_pixels=pixels)
    ref = O.blue(m, pixels, 1.5)
    np.testing.assert_array_equal(gpu, ref)
    assert sorted(gpu.tolist()) == list(range(m * m))


def test_blue_noise_rejects_bad_seeds():
    from sfsim_gb300 import _lib
    with pytest.raises(_lib.AtmoError):
        noise.blue_noise(8, seed_pixels=np.array([3, 3]))
    with pytest.raises(_lib.AtmoError):
        noise.blue_noise(8, seed_pixels=np.array([], dtype=np.int32))

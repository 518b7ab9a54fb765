"""Cloud-noise table builders on the GPU, the host side of include/sfsim_noise.h.

Mirrors src/clj/sfsim/worley.clj, perlin.clj and bluenoise.clj and the build
tasks `worley`, `perlin` and `bluenoise` of build.clj:34-51: the random
inputs are drawn here on the host with a seeded PCG64 generator (the
reference uses the JVM's rand, rand-nth and shuffle), the per-voxel and
per-pixel work runs in libsfsim_atmo.so.  There is no CPU fallback.
"""
from __future__ import annotations

import os

import numpy as np

from . import _lib
from .atmosphere_lut import spit_floats

WORLEY_SIZE = 16       # sfsim.worley/worley-size and the build task's default size
NOISE_DIVISIONS = 4    # the build tasks' default divisions
BLUE_NOISE_SIZE = 64   # sfsim.bluenoise/noise-size
BLUE_NOISE_SIGMA = 1.5


def random_point_grid(divisions: int, size: int, rng: np.random.Generator) -> np.ndarray:
    """random-point-grid (worley.clj:27-46): grid[k][j][i] = ((i, j, k) + U[0, 1)^3) * size / divisions."""
    cs = size // divisions
    idx = np.indices((divisions, divisions, divisions))  # k, j, i
    base = np.stack([idx[2], idx[1], idx[0]], axis=-1).astype(np.float64) * cs
    return base + rng.random((divisions, divisions, divisions, 3)) * cs


def random_gradient_grid(divisions: int, rng: np.random.Generator) -> np.ndarray:
    """random-gradient-grid (perlin.clj:37-48): indices 0..11 into random-gradient's vectors."""
    return rng.integers(0, 12, size=(divisions, divisions, divisions), dtype=np.int32)


def worley_noise(divisions: int = NOISE_DIVISIONS, size: int = WORLEY_SIZE, grid=None, seed: int = 0) -> np.ndarray:
    """worley-noise (worley.clj:96-109): size^3 float32 in the reference's order."""
    if grid is None:
        grid = random_point_grid(divisions, size, np.random.Generator(np.random.PCG64(seed)))
    g = np.ascontiguousarray(grid, dtype=np.float64)
    out = np.empty(size ** 3, np.float32)
    L = _lib.load()
    _lib.check(L.sfsim_noise_worley(divisions, size, g.ctypes.data, out.ctypes.data), "worley")
    return out


def perlin_noise(divisions: int = NOISE_DIVISIONS, size: int = WORLEY_SIZE, gradients=None, seed: int = 0) -> np.ndarray:
    """perlin-noise (perlin.clj:122-133): size^3 float32 scaled to [0, 1]."""
    if gradients is None:
        gradients = random_gradient_grid(divisions, np.random.Generator(np.random.PCG64(seed)))
    g = np.ascontiguousarray(gradients, dtype=np.int32)
    out = np.empty(size ** 3, np.float32)
    L = _lib.load()
    _lib.check(L.sfsim_noise_perlin(divisions, size, g.ctypes.data, out.ctypes.data), "perlin")
    return out


def blue_noise(m: int = BLUE_NOISE_SIZE, n: int | None = None, sigma: float = BLUE_NOISE_SIGMA, seed_pixels=None,
               seed: int = 0) -> np.ndarray:
    """blue-noise (bluenoise.clj:162-172): the m*m dither ranks; n seed pixels (default m*m/10, as the
    bluenoise build task picks) drawn like pick-n (a shuffle) unless given."""
    if seed_pixels is None:
        n = (m * m) // 10 if n is None else n
        seed_pixels = np.random.Generator(np.random.PCG64(seed)).permutation(m * m)[:n]
    s = np.ascontiguousarray(seed_pixels, dtype=np.int32)
    out = np.empty(m * m, np.int32)
    L = _lib.load()
    _lib.check(L.sfsim_noise_blue(m, len(s), s.ctypes.data, sigma, out.ctypes.data), "blue noise")
    return out


def build_worley(directory: str = "data/clouds", size: int = WORLEY_SIZE, divisions: int = NOISE_DIVISIONS,
                 seed: int = 0) -> list:
    """The `worley` build task (build.clj:34-38): three independent textures."""
    os.makedirs(directory, exist_ok=True)
    paths = []
    for t, name in enumerate(("worley-north.raw", "worley-south.raw", "worley-cover.raw")):
        path = os.path.join(directory, name)
        spit_floats(path, worley_noise(divisions, size, seed=seed + t))
        paths.append(path)
    return paths


def build_perlin(directory: str = "data/clouds", size: int = WORLEY_SIZE, divisions: int = NOISE_DIVISIONS,
                 seed: int = 0) -> str:
    """The `perlin` build task (build.clj:40-43)."""
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, "perlin.raw")
    spit_floats(path, perlin_noise(divisions, size, seed=seed))
    return path


def build_bluenoise(path: str = "data/bluenoise.raw", size: int = BLUE_NOISE_SIZE, seed: int = 0) -> str:
    """The `bluenoise` build task (build.clj:45-51): ranks / size^2 as float32."""
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    dither = blue_noise(size, (size * size) // 10, BLUE_NOISE_SIGMA, seed=seed)
    spit_floats(path, (dither / float(size * size)).astype(np.float32))
    return path

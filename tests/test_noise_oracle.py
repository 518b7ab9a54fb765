"""Known-answer tests that pin the oracle's restatement of the cloud-noise
builders to the reference's own facts:
test/clj/sfsim/t_worley.clj, t_perlin.clj and t_bluenoise.clj (paths in
wedesoft/sfsim).  The reference injects its randomness in these facts; the
oracle takes the random inputs as arguments the same way."""
import math

import numpy as np
import pytest

from oracle import oracle as O


def grid(points):
    """A nested [k][j][i] list of 3-vectors as an array."""
    return np.array(points, dtype=np.float64)


# ---- Worley (t_worley.clj) ------------------------------------------------------------

@pytest.mark.parametrize("g,divisions,size,point,expected", [
    # t_worley.clj:48-59
    ([[[(1, 1, 1)]]], 1, 2, (1, 1, 1), 0.0),
    ([[[(1, 1, 1)]]], 1, 2, (0.5, 1, 1), 0.5),
    ([[[(1, 1, 1), (3, 1, 1)]]], 2, 4, (3, 1, 1), 0.0),
    ([[[(1, 1, 1)], [(1, 3, 1)]]], 2, 4, (1, 3, 1), 0.0),
    ([[[(1, 1, 1)]], [[(1, 1, 3)]]], 2, 4, (1, 1, 3), 0.0),
    ([[[(0.25, 1, 1)]]], 1, 2, (1.75, 1, 1), 0.5),
    ([[[(1.75, 1, 1)]]], 1, 2, (0.25, 1, 1), 0.5),
    ([[[(1, 0.25, 1)]]], 1, 2, (1, 1.75, 1), 0.5),
    ([[[(1, 1.75, 1)]]], 1, 2, (1, 0.25, 1), 0.5),
    ([[[(1, 1, 0.25)]]], 1, 2, (1, 1, 1.75), 0.5),
    ([[[(1, 1, 1.75)]]], 1, 2, (1, 1, 0.25), 0.5),
])
def test_worley_closest_distance(g, divisions, size, point, expected):
    assert O.worley_closest(grid(g), divisions, size, point) == pytest.approx(expected, abs=1e-12)


def test_worley_noise_fact():
    # t_worley.clj:76-80: one point at (0.5, 0.5, 0.5) in a 2^3 texture
    out = O.worley(1, 2, grid([[[(0.5, 0.5, 0.5)]]]))
    assert out[0] == 1.0
    assert out.size == 8
    assert out.min() == 0.0


def test_worley_random_point_grid_layout():
    # t_worley.clj:23-29 with `identity` as the random function: point (i + 1, j + 1, k + 1) * cellsize
    # at grid[k][j][i]; the noise of such a grid is symmetric under any permutation of the axes
    d, size = 2, 8
    cs = size // d
    g = np.array([[[((i + 1) * cs, (j + 1) * cs, (k + 1) * cs) for i in range(d)] for j in range(d)]
                  for k in range(d)], dtype=np.float64)
    assert g[0, 0, 0, 0] == 4.0 and g[0, 0, 1, 0] == 8.0 and g[0, 1, 0, 1] == 8.0 and g[1, 0, 0, 2] == 8.0
    out = O.worley(d, size, g).reshape(size, size, size)
    np.testing.assert_array_equal(out, out.transpose(2, 1, 0))


# ---- Perlin (t_perlin.clj) ------------------------------------------------------------

GRADIENTS = [(1, 1, 0), (-1, 1, 0), (1, -1, 0), (-1, -1, 0), (1, 0, 1), (-1, 0, 1), (1, 0, -1), (-1, 0, -1),
             (0, 1, 1), (0, -1, 1), (0, 1, -1), (0, -1, -1)]

# t_perlin.clj:126-128, as indices into the twelve gradients
FACT_GRID = [[[GRADIENTS.index((1, 1, 0)), GRADIENTS.index((1, 0, -1))],
              [GRADIENTS.index((1, 0, 1)), GRADIENTS.index((-1, -1, 0))]],
             [[GRADIENTS.index((1, 0, 1)), GRADIENTS.index((-1, 0, 1))],
              [GRADIENTS.index((1, 0, -1)), GRADIENTS.index((-1, 0, -1))]]]


@pytest.mark.parametrize("t,expected", [(0.0, 0.0), (1.0, 1.0), (0.5, 0.5), (0.2, 0.05792), (0.8, 0.94208)])
def test_perlin_ease_curve(t, expected):
    # t_perlin.clj:103-110
    assert O.perlin_ease(t) == pytest.approx(expected, abs=1e-4)


@pytest.mark.parametrize("cell,expected", [((0.5, 0.5, 0.5), 0.30273), ((1.5, 0.5, 0.5), -0.21457)])
def test_perlin_sample(cell, expected):
    # t_perlin.clj:138-140
    assert O.perlin_sample(np.array(FACT_GRID), 2, 4, cell) == pytest.approx(expected, abs=1e-5)


def test_perlin_noise_fact():
    # t_perlin.clj:143-148
    out = O.perlin(2, 4, np.array(FACT_GRID))
    assert out[0] == pytest.approx(0.74821, abs=1e-5)
    assert out.size == 64
    assert out.min() == 0.0 and out.max() == 1.0


# ---- blue noise (t_bluenoise.clj) -----------------------------------------------------

@pytest.mark.parametrize("x,m,expected", [(0, 5, 0), (2, 5, 2), (5, 5, 0), (3, 5, -2), (2, 4, -2)])
def test_blue_wrap(x, m, expected):
    # t_bluenoise.clj:74-79
    assert O.blue_wrap(x, m) == expected


def test_blue_density_function():
    # t_bluenoise.clj:44-50 through the weight table
    t = O.blue_table(4, 1.0)
    assert t[0] == pytest.approx(1.0, abs=1e-6)
    assert t[1] == pytest.approx(math.exp(-0.5)) and t[3] == pytest.approx(math.exp(-0.5))
    assert O.blue_table(4, 2.0)[2] == pytest.approx(math.exp(-0.5))


def test_blue_density_array():
    # the density-sample facts (t_bluenoise.clj:82-92) with the Gauss weights: a single set pixel
    # contributes f(0, 0) to itself and f(wrap(dx), wrap(dy)) elsewhere
    d = O.blue_density_array([True, False, False, False], 2, 1.5)
    f = lambda dx, dy: math.exp(-(dx * dx + dy * dy) / (2 * 1.5 * 1.5))  # noqa: E731
    np.testing.assert_allclose(d, [f(0, 0), f(-1, 0), f(0, -1), f(-1, -1)], rtol=1e-15)


@pytest.mark.parametrize("mask,expected", [
    # t_bluenoise.clj:106-108
    ([True, False, False, False], [False, False, False, True]),
    ([True, True, False, False], [True, False, False, True]),
])
def test_blue_seed_pattern(mask, expected):
    assert list(O.blue_seed_pattern(mask, 2, 1.9)) == expected


def test_blue_phase1():
    # t_bluenoise.clj:111-113
    assert list(O.blue_phase(1, [True, False, False, False], 2, 1, 1.5, [0] * 4)[0]) == [0, 0, 0, 0]
    assert list(O.blue_phase(1, [True, False, False, True], 2, 2, 1.5, [0] * 4)[0]) == [0, 0, 0, 1]


def test_blue_phase2():
    # t_bluenoise.clj:116-120
    d, m = O.blue_phase(2, [True, False, False, True], 2, 2, 1.5, [0, 0, 0, 1])
    assert list(d) == [0, 0, 0, 1] and list(m) == [True, False, False, True]
    d, m = O.blue_phase(2, [True, False, False, False], 2, 1, 1.5, [0, 0, 0, 0])
    assert list(d) == [0, 0, 0, 1] and list(m) == [True, False, False, True]


def test_blue_phase3():
    # t_bluenoise.clj:123-124
    d, _ = O.blue_phase(3, [True, False, False, True], 2, 2, 1.5, [0, 0, 0, 1])
    assert list(d) == [0, 3, 2, 1]


def test_blue_noise_is_a_permutation():
    # the dither array of blue-noise ranks every pixel exactly once
    rng = np.random.default_rng(0)
    m = 16
    seed = rng.permutation(m * m)[: (m * m) // 10]
    d = O.blue(m, seed, 1.5)
    assert sorted(d.tolist()) == list(range(m * m))

"""Known-answer tests that pin the FP64 CPU oracle to the reference.

Every expected value below is read from the reference's own test files
(paths inside wedesoft/sfsim, cited per test).  Where a reference test
replaces a callee with `with-redefs`, the test here checks the same call
contract with the real callee instead (constant integrands, zero extinction).
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

R = 6378000.0
H = 100000.0
E = math.e
PI = math.pi

RAY_GRAY = O.comp((5.8e-6, 5.8e-6, 5.8e-6), 8000.0)
EARTH = O.planet(R, H)
SMALL = O.planet(4.0, 1.0)


def close(a, b, tol):
    return np.allclose(np.asarray(a, dtype=float), np.asarray(b, dtype=float), rtol=0, atol=tol)


# --- t_atmosphere.clj:72-100 ---------------------------------------------------

def test_scattering_heights():
    """t_atmosphere.clj:72-78"""
    assert O.scattering(RAY_GRAY, 0.0)[0] == 5.8e-6
    assert close(O.scattering(RAY_GRAY, 8000.0)[0], 5.8e-6 / E, 1e-12)
    assert close(O.scattering(RAY_GRAY, 16000.0)[0], 5.8e-6 / E / E, 1e-12)
    mie = O.comp((2e-5, 2e-5, 2e-5), 1200.0)
    assert close(O.scattering(mie, 1200.0)[0], 2e-5 / E, 1e-12)


def test_extinction():
    """t_atmosphere.clj:81-85"""
    mie = O.comp((2e-5, 2e-5, 2e-5), 1200.0, 0.9)
    assert close(O.extinction(mie, 1200.0)[0], 2e-5 / 0.9 / E, 1e-12)
    assert close(O.extinction(RAY_GRAY, 8000.0)[0], 5.8e-6 / E, 1e-12)


@pytest.mark.parametrize("g,mu,expected", [
    (0.0, 0.0, 3 / (16 * PI)), (0.0, 1.0, 6 / (16 * PI)), (0.0, -1.0, 6 / (16 * PI)),
    (0.5, 0.0, (3 * 0.75) / (8 * PI * 2.25 * 1.25 ** 1.5)),
    (0.5, 1.0, (6 * 0.75) / (8 * PI * 2.25 * 0.25 ** 1.5)),
])
def test_phase(g, mu, expected):
    """t_atmosphere.clj:88-100 (Rayleigh = g 0 and Cornette-Shanks Mie)"""
    assert close(O.phase(g, mu), expected, 1e-12)


# --- t_atmosphere.clj:103-141 --------------------------------------------------

def test_atmosphere_intersection():
    """t_atmosphere.clj:103-111"""
    assert close(O.atmosphere_intersection(EARTH, (R, 0, 0), (1, 0, 0)), (R + H, 0, 0), 1e-6)
    assert close(O.atmosphere_intersection(EARTH, (0, R, 0), (0, 1, 0)), (0, R + H, 0), 1e-6)
    assert close(O.atmosphere_intersection(EARTH, (0, -2 * R, 0), (0, 1, 0)), (0, R + H, 0), 1e-6)


def test_surface_intersection():
    """t_atmosphere.clj:114-121"""
    assert close(O.surface_intersection(EARTH, (R, 0, 0), (-1, 0, 0)), (R, 0, 0), 1e-6)
    assert close(O.surface_intersection(EARTH, (R + 10000, 0, 0), (-1, 0, 0)), (R, 0, 0), 1e-6)
    assert close(O.surface_intersection(EARTH, (R + 100, -1000, 0), (0, 1, 0)), (R + 100, 0, 0), 1e-6)


def test_surface_point():
    """t_atmosphere.clj:124-129"""
    assert O.surface_point(EARTH, (R, 0, 0)) is True
    assert O.surface_point(EARTH, (R + H, 0, 0)) is False


def test_ray_extremity():
    """t_atmosphere.clj:132-141"""
    assert close(O.ray_extremity(EARTH, (R + 10000, 0, 0), (-1, 0, 0)), (R, 0, 0), 1e-6)
    assert close(O.ray_extremity(EARTH, (R + 10000, 0, 0), (1, 0, 0)), (R + 100000, 0, 0), 1e-6)
    assert close(O.ray_extremity(EARTH, (R - 0.1, 0, 0), (1, 0, 0)), (R + 100000, 0, 0), 1e-6)


# --- t_atmosphere.clj:144-172 transmittance ---------------------------------------

def test_transmittance():
    """t_atmosphere.clj:144-172, including the full zenith value 0.932307"""
    ray = O.RAYLEIGH
    mie = O.comp((2e-5, 2e-5, 2e-5), 1200.0, 0.9)
    one = O.comps(ray)
    both = O.comps(ray, mie)
    assert close(O.transmittance(EARTH, one, 50, (0, R, 0), (0, R, 0))[0], 1.0, 1e-6)
    assert close(O.transmittance(EARTH, one, 50, (0, R, 0), (1000, R, 0))[0], math.exp(-1000 * 5.8e-6), 1e-6)
    assert close(O.transmittance(EARTH, one, 50, (0, R + 8000, 0), (1000, R + 8000, 0))[0],
                 math.exp(-(1000 * 5.8e-6) / E), 1e-6)
    assert close(O.transmittance(EARTH, both, 50, (0, R, 0), (1000, R, 0))[0],
                 math.exp(-1000 * (5.8e-6 + 2e-5 / 0.9)), 1e-6)
    # the reference mocks surface-intersection to return (0 R 0); the real one does too
    assert close(O.transmittance_dir(EARTH, one, 50, (-1000, R, 0), (1, 0, 0), False)[0],
                 math.exp(-1000 * 5.8e-6), 1e-6)
    assert close(O.transmittance_dir(EARTH, both, 50, (0, R, 0), (0, 1, 0), True)[0], 0.932307, 1e-6)


def test_surface_radiance_base_contract():
    """t_atmosphere.clj:175-192: E0 = T(x, l, above) * I * max(0, n.l)"""
    cs = O.comps(O.MIE, O.RAYLEIGH)
    I = (1.0, 1.0, 1.0)
    x = (0, R, 0)
    T_up = O.transmittance_dir(EARTH, cs, 10, x, (0, 1, 0), True)
    assert close(O.surface_radiance_base(EARTH, cs, 10, I, x, (1, 0, 0)), (0, 0, 0), 0)
    assert close(O.surface_radiance_base(EARTH, cs, 10, I, x, (0, 1, 0)), T_up, 1e-15)
    assert close(O.surface_radiance_base(EARTH, cs, 10, I, x, (0, -1, 0)), (0, 0, 0), 0)
    moved = O.planet(R, H, centre=(0, 2 * R, 0))
    T_moved = O.transmittance_dir(moved, cs, 10, x, (0, -1, 0), True)
    assert close(O.surface_radiance_base(moved, cs, 10, I, x, (0, -1, 0)), T_moved, 1e-15)


def test_point_scatter_base_contract():
    """t_atmosphere.clj:204-246: J0 = I * beta(x) * phase(v.l) * T(x, l) above the horizon, else 0"""
    cs = O.comps(O.MIE)
    I = (1.0, 1.0, 1.0)
    x = (0, R + 1000, 0)
    v = (0.36, 0.48, 0.8)
    l = (1.0, 0.0, 0.0)
    expected = (O.scattering(O.MIE, 1000.0) * O.phase(0.76, np.dot(v, l))
                * O.transmittance_dir(EARTH, cs, 10, x, l, True))
    assert close(O.single_scatter(EARTH, cs, 0, 2, 10, I, x, v, l), expected, 1e-18)
    # the reference mocks is-above-horizon? to false; a sun straight below is below the horizon
    assert close(O.single_scatter(EARTH, cs, 0, 2, 10, I, x, v, (0.0, -1.0, 0.0)), (0, 0, 0), 0)


def test_ray_scatter_contract():
    """t_atmosphere.clj:249-282: S = integral of T(x,p) J over the ray; with zero
    extinction T = 1 and a constant J gives J * length for both branches"""
    clear = O.comps(O.comp((0, 0, 0), 1200.0, 0.9, 0.76))
    J = (2e-5, 2e-5, 2e-5)
    up = O.ray_scatter_const(EARTH, clear, 10, J, (0, R, 0), (0, 1, 0), (0.36, 0.48, 0.8), True)
    assert close(up, np.array(J) * H, 1e-12)
    # a ground ray from height H straight down has length H as well
    down = O.ray_scatter_const(EARTH, clear, 10, J, (0, R + H, 0), (0, -1, 0), (0.36, 0.48, 0.8), False)
    assert close(down, np.array(J) * H, 1e-12)


def test_single_scatter_components():
    """t_atmosphere.clj:285-296"""
    cs = O.comps(O.MIE, O.RAYLEIGH)
    I = (1, 1, 1)
    x = (R + 1000, 0, 0)
    v = (0, 1, 0)
    l = (0.36, 0.48, 0.8)
    mu = np.dot(v, l)
    psc_mie = O.single_scatter(EARTH, cs, 0, 0, 100, I, x, v, l)
    psc_ray = O.single_scatter(EARTH, cs, 1, 0, 100, I, x, v, l)
    base = O.single_scatter(EARTH, cs, 0, 2, 100, I, x, v, l)
    assert close(psc_mie + psc_ray, base, 1e-12)
    strength = O.single_scatter(EARTH, cs, 0, 1, 100, I, x, v, l)
    assert close(strength * O.phase(0.76, mu), psc_mie, 1e-12)


def test_point_scatter_contract():
    """t_atmosphere.clj:304-361: J integrates beta*phase*(dS + ground) over the
    sphere; a constant dS with no ground light gives beta(x)*dS since the
    Rayleigh phase integrates to 1"""
    cs = O.comps(O.RAYLEIGH)
    x = (0, R + 1200, 0)
    dS = (1.0, 2.0, 3.0)
    J = O.point_scatter_const(EARTH, cs, dS, (0, 0, 0), 64, 10, x, (0, 1, 0), (0.36, 0.48, 0.8))
    expected = O.scattering(O.RAYLEIGH, 1200.0) * np.array(dS)
    assert np.allclose(J, expected, rtol=2e-3)


def test_surface_radiance_contract():
    """t_atmosphere.clj:364-383: E = integral of dS (w.n) over the upper
    hemisphere; a constant dS gives pi * dS"""
    E_ = O.surface_radiance_const(EARTH, (1.0, 2.0, 3.0), 64, (0, R, 0), (0.6, 0.8, 0))
    assert np.allclose(E_, PI * np.array([1.0, 2.0, 3.0]), rtol=2e-3)


# --- t_atmosphere.clj:386-566 horizon and table spaces ------------------------------

def test_is_above_horizon():
    """t_atmosphere.clj:386-393"""
    p = O.planet(R, H)
    assert O.is_above_horizon(p, (R, 0, 0), (1, 0, 0)) is True
    assert O.is_above_horizon(p, (R, 0, 0), (-1, 0, 0)) is False
    assert O.is_above_horizon(p, (R, 0, 0), (-1e-4, 1, 0)) is False
    assert O.is_above_horizon(p, (R + 100000, 0, 0), (-1e-4, 1, 0)) is True
    assert O.is_above_horizon(p, (R + 100000, 0, 0), (-math.sqrt(0.5), math.sqrt(0.5), 0)) is False


def test_horizon_distance():
    """t_atmosphere.clj:396-398"""
    p = O.planet(4.0, 1.0)
    assert O.horizon_distance(p, 4.0) == 0.0
    assert O.horizon_distance(p, 5.0) == 3.0


@pytest.mark.parametrize("size,point,direction,above,expected", [
    (2, (4, 0, 0), (-1, 0, 0), False, 0.5),
    (2, (5, 0, 0), (-1, 0, 0), False, 1 / 3),
    (2, (5, 0, 0), (-math.sqrt(0.5), math.sqrt(0.5), 0), False, 0.223),
    (3, (4, 0, 0), (-1, 0, 0), False, 1.0),
    (2, (5, 0, 0), (-0.6, 0.8, 0), False, 0.0),
    (2, (4, 0, 0), (1, 0, 0), True, 2 / 3),
    (2, (5, 0, 0), (0, 1, 0), True, 0.5),
    (2, (5, 0, 0), (-0.6, 0.8, 0), True, 1.0),
    (2, (4, 0, 0), (0, 1, 0), True, 1.0),
    (3, (4, 0, 0), (0, 1, 0), True, 2.0),
    (2, (5, 0, 0), (-1, 0, 0), True, 1.0),
    (2, (4, 0, 0), (1, 0, 0), False, 0.5),
])
def test_elevation_to_index(size, point, direction, above, expected):
    """t_atmosphere.clj:400-414"""
    assert close(O.elevation_to_index(SMALL, size, point, direction, above), expected, 1e-3)


@pytest.mark.parametrize("size,radius,index,direction,above", [
    (2, 5.0, 1 / 3, (-1, 0, 0), False),
    (3, 5.0, 2 / 3, (-1, 0, 0), None),
    (2, 5.0, 0.222549, (-math.sqrt(0.5), math.sqrt(0.5), 0), None),
    (2, 5.0, 0.4, (-1, 0, 0), None),
    (2, 4.0, 0.4, (0, 1, 0), None),
    (2, 4.0, 2 / 3, (1, 0, 0), True),
    (3, 4.0, 4 / 3, (1, 0, 0), None),
    (2, 4.0, 1.0, (0, 1, 0), None),
    (2, 5.0, 1.0, (-0.6, 0.8, 0), None),
    (2, 5.0, 0.5, (0, 1, 0), True),
    (2, 5.0, 0.5001, (0, 1, 0), None),
    (2, 4.0, 0.5, (0, 1, 0), False),
    (2, 4.0, 0.5001, (1, 0, 0), None),
])
def test_index_to_elevation(size, radius, index, direction, above):
    """t_atmosphere.clj:417-435 (including the tie at index/(size-1) = 0.5)"""
    d, a = O.index_to_elevation(SMALL, size, radius, index)
    assert close(d, direction, 1e-3)
    if above is not None:
        assert a is above


def test_height_to_index():
    """t_atmosphere.clj:438-448"""
    assert O.height_to_index(SMALL, 2, (4, 0, 0)) == 0.0
    assert O.height_to_index(SMALL, 2, (5, 0, 0)) == 1.0
    assert close(O.height_to_index(SMALL, 2, (4.5, 0, 0)), 0.687, 1e-3)
    assert O.height_to_index(SMALL, 17, (5, 0, 0)) == 16.0
    p = O.planet(6378000.0, 35000.0)
    assert close(O.height_to_index(p, 32, (6377999.999549146, -16.87508805500576, 73.93459155883768)), 0.0, 1e-6)


def test_index_to_height():
    """t_atmosphere.clj:451-459"""
    assert close(O.index_to_height(SMALL, 2, 0.0), (4, 0, 0), 0)
    assert close(O.index_to_height(SMALL, 2, 1.0), (5, 0, 0), 0)
    assert close(O.index_to_height(SMALL, 2, 0.68718), (4.5, 0, 0), 1e-3)
    assert close(O.index_to_height(SMALL, 3, 2.0), (5, 0, 0), 0)


def test_transmittance_space():
    """t_atmosphere.clj:462-482"""
    p = O.planet(6378000.0, 35000.0)
    Rr, Hh = 6378000.0, 35000.0
    shape = (15, 17)
    assert close(O.space_forward(p, 0, shape, (Rr, 0, 0), (0, 1, 0), above=True), (0.0, 16.0), 1e-9)
    assert close(O.space_forward(p, 0, shape, (Rr + Hh, 0, 0), (0, 1, 0), above=True), (14.0, 8.0), 1e-9)
    assert close(O.space_forward(p, 0, shape, (Rr, 0, 0), (-1, 0, 0), above=False), (0.0, 8.0), 1e-9)
    pt, d, _, a = O.space_backward(p, 0, shape, (0.0, 16.0))
    assert close(pt, (Rr, 0, 0), 0) and close(d, (0, 1, 0), 1e-6) and a is True
    pt, d, _, a = O.space_backward(p, 0, shape, (14.0, 8.0))
    assert close(pt, (Rr + Hh, 0, 0), 0) and close(d, (0, 1, 0), 0) and a is True
    pt, d, _, a = O.space_backward(p, 0, shape, (0.0, 8.0))
    assert close(d, (0, 1, 0), 0) and a is False


def test_surface_radiance_space():
    """t_atmosphere.clj:485-502"""
    p = O.planet(6378000.0, 35000.0)
    Rr, Hh = 6378000.0, 35000.0
    shape = (15, 17)
    assert close(O.space_forward(p, 1, shape, (Rr, 0, 0), light=(1, 0, 0)), (0.0, 16.0), 1e-9)
    assert close(O.space_forward(p, 1, shape, (Rr + Hh, 0, 0), light=(1, 0, 0)), (14.0, 16.0), 1e-9)
    assert close(O.space_forward(p, 1, shape, (Rr, 0, 0), light=(-1, 0, 0)), (0.0, 0.0), 0)
    assert close(O.space_forward(p, 1, shape, (Rr, 0, 0), light=(-0.2, 0.980, 0)), (0.0, 0.0), 0)
    assert close(O.space_forward(p, 1, shape, (Rr, 0, 0), light=(0, 1, 0)), (0.0, 7.422), 1e-3)
    pt, _, l, _ = O.space_backward(p, 1, shape, (0.0, 16.0))
    assert close(pt, (Rr, 0, 0), 0) and close(l, (1, 0, 0), 1e-6)
    pt, _, l, _ = O.space_backward(p, 1, shape, (14.0, 16.0))
    assert close(pt, (Rr + Hh, 0, 0), 0)
    _, _, l, _ = O.space_backward(p, 1, shape, (14.0, 0.0))
    assert close(l, (-0.2, 0.980, 0), 1e-3)
    _, _, l, _ = O.space_backward(p, 1, shape, (0.0, 7.422))
    assert close(l, (0, 1, 0), 1e-3)


def test_sun_elevation_to_index():
    """t_atmosphere.clj:505-510"""
    assert O.sun_elevation_to_index(2, (4, 0, 0), (1, 0, 0)) == 1.0
    assert close(O.sun_elevation_to_index(2, (4, 0, 0), (0, 1, 0)), 0.464, 1e-3)
    assert O.sun_elevation_to_index(2, (4, 0, 0), (-0.2, 0.980, 0)) == 0.0
    assert O.sun_elevation_to_index(2, (4, 0, 0), (-1, 0, 0)) == 0.0
    assert O.sun_elevation_to_index(17, (4, 0, 0), (1, 0, 0)) == 16.0


def test_index_to_sin_sun_elevation():
    """t_atmosphere.clj:513-518"""
    assert close(O.index_to_sin_sun_elevation(2, 1.0), 1.0, 1e-3)
    assert close(O.index_to_sin_sun_elevation(2, 0.0), -0.2, 1e-3)
    assert close(O.index_to_sin_sun_elevation(2, 0.463863), 0.0, 1e-3)
    assert close(O.index_to_sin_sun_elevation(2, 0.5), 0.022, 1e-3)
    assert close(O.index_to_sin_sun_elevation(3, 1.0), 0.022, 1e-3)


def test_sun_angle_to_index():
    """t_atmosphere.clj:521-525"""
    assert O.sun_angle_to_index(2, (0, 1, 0), (0, 1, 0)) == 1.0
    assert O.sun_angle_to_index(2, (0, 1, 0), (0, -1, 0)) == 0.0
    assert O.sun_angle_to_index(2, (0, 1, 0), (0, 0, 1)) == 0.5
    assert O.sun_angle_to_index(17, (0, 1, 0), (1, 0, 0)) == 8.0


@pytest.mark.parametrize("size,direction,sin_sun,index,expected,tol", [
    (2, (0, 1, 0), 0.0, 1.0, (0, 1, 0), 0),
    (2, (0, 1, 0), 0.0, 0.0, (0, -1, 0), 0),
    (2, (0, 1, 0), 1.0, 0.5, (1, 0, 0), 0),
    (2, (0, 1, 0), 1.00001, 0.5, (1, 0, 0), 1e-3),
    (2, (0, 1, 0), 0.0, 0.5, (0, 0, 1), 0),
    (2, (1, 0, 0), 1.0, 1.0, (1, 0, 0), 0),
    (2, (0, -1, 0), 0.0, 1.0, (0, -1, 0), 0),
    (3, (0, 1, 0), 0.0, 1.0, (0, 0, 1), 0),
])
def test_index_to_sun_direction(size, direction, sin_sun, index, expected, tol):
    """t_atmosphere.clj:528-536"""
    assert close(O.index_to_sun_direction(size, direction, sin_sun, index), expected, tol)


@pytest.mark.parametrize("point,direction,light,above,expected,tol", [
    ((R, 0, 0), (1, 0, 0), (1, 0, 0), True, (0.0, 9.794, 16.0, 14.0), 1e-3),
    ((R + H, 0, 0), (1, 0, 0), (1, 0, 0), True, (20.0, 9.0, 16.0, 14.0), 1e-9),
    ((R, 0, 0), (-1, 0, 0), (1, 0, 0), False, (0.0, 9.0, 16.0, 0.0), 1e-9),
    ((0, R, 0), (0, -1, 0), (0, 1, 0), False, (0.0, 9.0, 16.0, 0.0), 1e-9),
    ((R, 0, 0), (1, 0, 0), (0, 0, 1), True, (0.0, 9.794, 7.422, 7.0), 1e-3),
    ((R, 0, 0), (0, 0, 1), (0, 0, 1), True, (0.0, 18.0, 7.422, 14.0), 1e-3),
    ((R, 0, 0), (0, 0, 1), (0, 0, 1), False, (0.0, 9.0, 7.422, 14.0), 1e-3),
    ((R, 0, 0), (0, 0, 1), (0, -1, 0), True, (0.0, 18.0, 7.422, 7.0), 1e-3),
    ((R, 0, 0), (0, 0, 1), (0, 1, 0), True, (0.0, 18.0, 7.422, 7.0), 1e-3),
    ((R, 0, 0), (0, 1, 0), (0, 1, 0), True, (0.0, 18.0, 7.422, 14.0), 1e-3),
    ((R, 0, 0), (0, 0, 1), (0, 0, -1), True, (0.0, 18.0, 7.422, 0.0), 1e-3),
])
def test_ray_scatter_space_forward(point, direction, light, above, expected, tol):
    """t_atmosphere.clj:539-558"""
    got = O.space_forward(EARTH, 2, (21, 19, 17, 15), point, direction, light, above)
    assert close(got, expected, tol)


def test_ray_scatter_space_backward():
    """t_atmosphere.clj:559-566"""
    shape = (21, 19, 17, 15)
    b = lambda idx: O.space_backward(EARTH, 2, shape, idx)  # noqa: E731
    assert close(b((0.0, 0.0, 0.0, 0.0))[0], (R, 0, 0), 0)
    assert close(b((20.0, 0.0, 0.0, 0.0))[0], (R + H, 0, 0), 1e-9)
    assert close(b((0.0, 9.79376, 0.0, 0.0))[1], (1, 0, 0), 1e-6)
    assert close(b((0.0, 18.0, 0.0, 0.0))[1], (0, 1, 0), 1e-6)
    assert close(b((0.0, 9.7937607, 16.0, 14.0))[2], (1, 0, 0), 1e-3)
    assert close(b((0.0, 9.7937607, 7.421805, 7.0))[2], (0, 0, 1), 1e-3)
    assert close(b((0.0, 18.0, 7.421805, 7.0))[2], (0, 0, 1), 1e-3)
    assert b((0.0, 9.79376, 0.0, 0.0))[3] is True
    assert b((20.0, 8.206, 16.0, 0.0))[3] is False


# --- t_sphere.clj:22-63, t_ray.clj:21-29 ---------------------------------------

def test_height():
    """t_sphere.clj:22-25"""
    assert O.height(O.planet(10.0, 1.0), (10, 0, 0)) == 0.0
    assert O.height(O.planet(10.0, 1.0), (13, 0, 0)) == 3.0
    assert O.height(O.planet(10.0, 1.0, centre=(2, 0, 0)), (13, 0, 0)) == 1.0


@pytest.mark.parametrize("origin,direction,expected", [
    ((-2, 0, 3), (0, 1, 0), (0.0, 0.0)),
    ((-2, 0, 3), (1, 0, 0), (1.0, 2.0)),
    ((0, 0, 3), (1, 0, 0), (0.0, 1.0)),
    ((2, 0, 3), (1, 0, 0), (0.0, 0.0)),
    ((-2, 0, 3), (2, 0, 0), (0.5, 1.0)),
    ((-5, 0, 0), (1, 0, 0), (5.0, 0.0)),
    ((5, 0, 0), (1, 0, 0), (0.0, 0.0)),
])
def test_ray_sphere_intersection(origin, direction, expected):
    """t_sphere.clj:28-43"""
    assert O.ray_sphere_intersection((0, 0, 3), 1.0, origin, direction) == expected


def test_integrate_circle():
    """t_sphere.clj:46-48"""
    assert close(O.integrate_circle(64, (0, 0, 0)), (0, 0, 0), 1e-6)
    assert close(O.integrate_circle(64, (1, 1, 1)), (2 * PI,) * 3, 1e-6)


def test_integral_half_sphere():
    """t_sphere.clj:51-57"""
    left, up = (1, 0, 0), (0, 1, 0)
    assert close(O.integral_sphere(64, left, (0, 0, 0), half=True), (0, 0, 0), 1e-6)
    assert close(O.integral_sphere(64, left, (1, 1, 0), half=True)[:2], (2 * PI, 2 * PI), 1e-6)
    assert close(O.integral_sphere(64, left, (1, 0, 0), (-1, 1, 2), half=True), (2 * PI, 0, 0), 1e-6)
    assert close(O.integral_sphere(64, up, (0, 1, 0), (0, -1, 2), half=True), (0, 2 * PI, 0), 1e-6)


def test_integral_sphere():
    """t_sphere.clj:60-63"""
    left = (1, 0, 0)
    assert close(O.integral_sphere(64, left, (0, 0, 0)), (0, 0, 0), 1e-6)
    assert close(O.integral_sphere(64, left, (1, 1, 0))[:2], (4 * PI, 4 * PI), 1e-6)


def test_sphere_direction_counts():
    """The direction counts that the build relies on (sphere.clj:70-105)."""
    assert O.sphere_directions(15) == 71
    assert O.sphere_directions(16) == 86
    assert O.sphere_directions(32) == 336


def test_integral_ray():
    """t_ray.clj:21-29"""
    assert close(O.integral_ray((2, 3, 5), (1, 0, 0), 10, 0.0, (2, 2, 0)), (0, 0, 0), 1e-6)
    assert close(O.integral_ray((2, 3, 5), (1, 0, 0), 10, 3.0, (2, 2, 0)), (6, 6, 0), 1e-6)
    assert close(O.integral_ray((2, 3, 5), (1, 0, 0), 10, 3.0, (0, 0, 0), (0, 0, -1)), (10.5, 10.5, 0), 1e-6)
    assert close(O.integral_ray((2, 3, 5), (2, 0, 0), 10, 1.5, (0, 0, 0), (0, 0, -1)), (10.5, 10.5, 0), 1e-6)


def test_orthogonal():
    """quaternion.clj:166-171: normal (1,0,0) picks e_y, giving o1 = (0,0,1)."""
    assert close(O.orthogonal((1, 0, 0)), (0, 0, 1), 0)
    o = O.orthogonal((0.36, 0.48, 0.8))
    assert abs(np.dot(o, (0.36, 0.48, 0.8))) < 1e-15 and abs(np.linalg.norm(o) - 1) < 1e-15


# --- t_interpolate.clj:61-109 ------------------------------------------------------

def _lin(x, a, b, n):
    return (x - a) / (b - a) * (n - 1)


@pytest.mark.parametrize("x,expected", [(-3.0, 9.0), (1.5, 2.5), (-5.0, 9.0), (3.0, 4.0)])
def test_interpolation_table_1d(x, expected):
    """t_interpolate.clj:79-85 and :103-109 (linear space [-3, 2] with 6 nodes; clip at both ends)"""
    table = np.array([[v, v, v] for v in (9, 4, 1, 0, 1, 4)], dtype=float)
    assert close(O.interpolate(table, [_lin(x, -3.0, 2.0, 6)])[0], expected, 1e-12)


def test_interpolation_table_vectors():
    """t_interpolate.clj:88-89"""
    table = np.array([[2, 3, 5], [3, 5, 9]], dtype=float)
    assert close(O.interpolate(table, [_lin(0.0, -1.0, 1.0, 2)]), (2.5, 4.0, 7.0), 1e-12)


@pytest.mark.parametrize("y0,x0,y1,x1,y,x,expected", [
    (0.0, 0.0, 1.0, 2.0, 0, 0, 2.0), (0.0, 0.0, 1.0, 2.0, 0, 2, 5.0), (0.0, 0.0, 1.0, 2.0, 0, 1.5, 4.0),
    (0.0, 0.0, 1.0, 2.0, 1, 0, 7.0), (0.0, 0.0, 1.0, 2.0, 0.5, 0, 4.5), (-3.0, 0.0, 1.0, 2.0, -1, 0, 4.5),
])
def test_interpolation_table_2d(y0, x0, y1, x1, y, x, expected):
    """t_interpolate.clj:92-100"""
    data = [[2, 3, 5], [7, 11, 13]]
    table = np.array([[[v, v, v] for v in row] for row in data], dtype=float)
    c = [_lin(y, y0, y1, 2), _lin(x, x0, x1, 3)]
    assert close(O.interpolate(table, c)[0], expected, 1e-12)


def test_clip_and_mix():
    """t_interpolate.clj:61-76 through one-dimensional tables"""
    table = np.array([[v, v, v] for v in range(16)], dtype=float)
    for i, r in [(0.0, 0.0), (15.0, 15.0), (-2.0, 0.0), (16.0, 15.0)]:
        assert O.interpolate(table, [i])[0] == r
    two = np.array([[-2.0] * 3, [4.0] * 3])
    for s, r in [(0.0, -2.0), (1.0, 4.0), (0.5, 1.0), (0.25, -0.5)]:
        assert O.interpolate(two, [s])[0] == r

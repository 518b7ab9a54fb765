"""The oracle's restatement of the SCAN_RAYS build mode (not the reference's
algorithm): view-ray transmittances from one running sum along the ray.

The scan loop is checked against a numpy restatement of the same
discretisation, and the mode against the reference's nested quadrature:
it changes neither the transmittance table nor E0, and its deviation from
the nested tables shrinks as the square of the step size.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sfsim_gb300 import config as C

R = 6378000.0
H = 100000.0
EARTH = O.planet(R, H)


def scan_restated(p, cs, steps, J, x, v, above):
    """sum_n a J exp(-tau_n), tau_n = a (sum_{m<n} ext(p_m) + ext(p_{n+1/4}) / 2)."""
    x = np.asarray(x, float)
    e = O.atmosphere_intersection(p, x, v) if above else O.surface_intersection(p, x, v)
    D = np.asarray(e, float) - x
    a = np.linalg.norm(D) / steps

    def ext(q):
        h = O.height(p, q)
        return sum(O.extinction(c, h) for c in cs)

    depth = np.zeros(3)
    acc = np.zeros(3)
    for n in range(steps):
        pn = x + D * ((0.5 + n) / steps)
        ph = x + D * ((0.25 + n) / steps)
        tau = depth + ext(ph) * (0.5 * a)
        acc += np.asarray(J) * np.exp(-tau) * a
        depth += ext(pn) * a
    return acc


@pytest.mark.parametrize("x,v,above", [
    ((0, R + 2000.0, 0), (0.0, 1.0, 0.0), True),
    ((0, R + 2000.0, 0), (0.999, 0.0447101778, 0.0), True),
    ((0, R + 30000.0, 0), (0.6, -0.8, 0.0), False),
    ((0, R + 500.0, 0), (1.0, 0.0, 0.0), True),
])
def test_scan_loop_restated(x, v, above):
    cs = O.comps(O.MIE, O.RAYLEIGH)
    J = (1e-5, 2e-5, 3e-5)
    got = O.ray_scatter_scan_const(EARTH, cs, 24, J, x, v, (0.0, 1.0, 0.0), above)
    want = scan_restated(EARTH, cs, 24, J, x, v, above)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)


def test_scan_without_extinction_is_the_ray_length():
    """T = 1 everywhere: both quadratures give J times the ray's length."""
    clear = O.comps(O.comp((0, 0, 0), 1200.0, 0.9, 0.76))
    J = (2e-5, 2e-5, 2e-5)
    up = O.ray_scatter_scan_const(EARTH, clear, 10, J, (0, R, 0), (0, 1, 0), (0.36, 0.48, 0.8), True)
    np.testing.assert_allclose(up, np.array(J) * H, rtol=1e-12)


def tiny(steps, flags):
    return C.make_config(height=100000.0, transmittance_shape=(6, 6), surface_radiance_shape=(4, 6),
                         ray_scatter_shape=(4, 6, 4, 3), ray_steps=steps, sphere_steps=8, iterations=1,
                         precision=C.FP64, flags=flags)


def rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-6 * np.abs(b).max())


def test_scan_mode_tables():
    """T and E0 do not depend on the view-ray quadrature; every 4-D table
    does, by less than the nested quadrature's own step error."""
    nested = O.build(tiny(32, 0), intermediates=True)
    scan = O.build(tiny(32, C.SCAN_RAYS), intermediates=True)
    assert np.array_equal(nested["transmittance"], scan["transmittance"])
    assert np.array_equal(nested["surface_base"], scan["surface_base"])
    for k in ("rayleigh_first", "mie_first", "ray_scatter", "mie_strength", "surface_radiance"):
        e = rel(scan[k], nested[k])
        assert 0 < e.max() < 0.1, (k, e.max())


def test_scan_deviation_is_second_order():
    """Halving the step size cuts the scan's deviation from the nested
    quadrature about fourfold (both are midpoint rules)."""
    dev = []
    for steps in (16, 32, 64):
        n = O.build(tiny(steps, 0), intermediates=True)
        s = O.build(tiny(steps, C.SCAN_RAYS), intermediates=True)
        dev.append(max(rel(s[k], n[k]).max() for k in ("rayleigh_first", "mie_first")))
    assert dev[0] / dev[1] > 3.0 and dev[1] / dev[2] > 3.0, dev

"""Configuration records of the atmosphere lookup-table build.

`AtmoConfig` is the ctypes mirror of `sfsim_atmo_config` in include/sfsim_atmo.h.
The planet and scattering-component values mirror the maps that
src/clj/sfsim/atmosphere_lut.clj:20-40 defines (`earth`, `mie`, `rayleigh`);
shapes, steps and iterations mirror atmosphere_lut.clj:47-61.

Named workloads:
  reference_production()  the reference's own settings (35 km atmosphere,
                          T 64x255, E 16x63, S 32x127x32x8, 100 ray steps,
                          15 sphere steps, 5 iterations)
  small_fp64()            FP64 case: 100 km atmosphere, T 32x32, E 16x32,
                          S 8x16x8x4, 2 iterations, 64 ray steps, sphere steps 16
  production()            FP32 case: T 255x255, E 16x64, S 32x255x32x8,
                          5 iterations, 128 ray steps, sphere steps 32
  parameter_sweep(n, seed) n atmospheres with physical parameters drawn
                          uniformly (Rayleigh scale height 6-10 km, Mie scale
                          height 0.8-2 km, g in [0.6, 0.85], each beta scaled
                          log-uniformly in [0.5, 2], radius 3000-7000 km);
                          S 16x128x16x8, 4 iterations
  shader_test()           the 12x12 / 12^4 tables with 10 ray steps of
                          test/clj/sfsim/t_atmosphere.clj:44-69,569-578
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

FP32 = 0
FP64 = 1

# flag bits of AtmoConfig.flags (sfsim_atmo.h SFSIM_ATMO_*); 0 follows the reference
SCAN_RAYS = 1  # view-ray transmittances by one prefix scan per ray, not the nested quadrature


class Component(ctypes.Structure):
    """sfsim_atmo_component; mirrors the `scatter` schema, atmosphere.clj:35-39."""

    _fields_ = [
        ("scatter_base", ctypes.c_double * 3),
        ("scatter_scale", ctypes.c_double),
        ("scatter_quotient", ctypes.c_double),
        ("scatter_g", ctypes.c_double),
    ]


class AtmoConfig(ctypes.Structure):
    """sfsim_atmo_config of include/sfsim_atmo.h."""

    _fields_ = [
        ("radius", ctypes.c_double),
        ("height", ctypes.c_double),
        ("brightness", ctypes.c_double * 3),
        ("intensity", ctypes.c_double * 3),
        ("mie", Component),
        ("rayleigh", Component),
        ("transmittance_shape", ctypes.c_int * 2),
        ("surface_radiance_shape", ctypes.c_int * 2),
        ("ray_scatter_shape", ctypes.c_int * 4),
        ("ray_steps", ctypes.c_int),
        ("sphere_steps", ctypes.c_int),
        ("iterations", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("flags", ctypes.c_int),
    ]

    # -- convenience -------------------------------------------------------
    def copy(self) -> "AtmoConfig":
        c = AtmoConfig()
        ctypes.pointer(c)[0] = self
        return c

    def shapes(self):
        return (tuple(self.transmittance_shape), tuple(self.surface_radiance_shape),
                tuple(self.ray_scatter_shape))

    def table_sizes(self):
        """Float counts of the four output tables (RGB included)."""
        t, e, s = self.shapes()
        n_t = 3 * t[0] * t[1]
        n_e = 3 * e[0] * e[1]
        n_s = 3 * s[0] * s[1] * s[2] * s[3]
        return n_t, n_e, n_s, n_s

    def describe(self) -> dict:
        t, e, s = self.shapes()
        return {
            "radius": self.radius, "height": self.height,
            "transmittance": list(t), "surface_radiance": list(e), "ray_scatter": list(s),
            "ray_steps": self.ray_steps, "sphere_steps": self.sphere_steps,
            "iterations": self.iterations,
            "precision": "fp64" if self.precision == FP64 else "fp32",
        }


def component(base, scale, quotient=1.0, g=0.0) -> Component:
    c = Component()
    for i in range(3):
        c.scatter_base[i] = float(base[i])
    c.scatter_scale = float(scale)
    c.scatter_quotient = float(quotient)
    c.scatter_g = float(g)
    return c


def mie_component() -> Component:
    """atmosphere_lut.clj:31-35"""
    return component((2e-5, 2e-5, 2e-5), 1200.0, 0.9, 0.76)


def rayleigh_component() -> Component:
    """atmosphere_lut.clj:38-40"""
    return component((5.8e-6, 13.5e-6, 33.1e-6), 8000.0)


def make_config(radius=6378000.0, height=35000.0, brightness=(0.3, 0.3, 0.3), intensity=(1.0, 1.0, 1.0),
                mie=None, rayleigh=None, transmittance_shape=(64, 255), surface_radiance_shape=(16, 63),
                ray_scatter_shape=(32, 127, 32, 8), ray_steps=100, sphere_steps=15, iterations=5,
                precision=FP32, flags=0) -> AtmoConfig:
    c = AtmoConfig()
    c.radius = float(radius)
    c.height = float(height)
    for i in range(3):
        c.brightness[i] = float(brightness[i])
        c.intensity[i] = float(intensity[i])
    c.mie = mie if mie is not None else mie_component()
    c.rayleigh = rayleigh if rayleigh is not None else rayleigh_component()
    for i in range(2):
        c.transmittance_shape[i] = int(transmittance_shape[i])
        c.surface_radiance_shape[i] = int(surface_radiance_shape[i])
    for i in range(4):
        c.ray_scatter_shape[i] = int(ray_scatter_shape[i])
    c.ray_steps = int(ray_steps)
    c.sphere_steps = int(sphere_steps)
    c.iterations = int(iterations)
    c.precision = int(precision)
    c.flags = int(flags)
    return c


def reference_production() -> AtmoConfig:
    """The reference's own build settings, atmosphere_lut.clj:20-63."""
    return make_config()


def small_fp64(precision=FP64) -> AtmoConfig:
    """Small case that the reference's CPU path finishes quickly."""
    return make_config(height=100000.0, transmittance_shape=(32, 32), surface_radiance_shape=(16, 32),
                       ray_scatter_shape=(8, 16, 8, 4), ray_steps=64, sphere_steps=16, iterations=2,
                       precision=precision)


def production(precision=FP32) -> AtmoConfig:
    """Production-size build on one GPU."""
    return make_config(height=100000.0, transmittance_shape=(255, 255), surface_radiance_shape=(16, 64),
                       ray_scatter_shape=(32, 255, 32, 8), ray_steps=128, sphere_steps=32, iterations=5,
                       precision=precision)


def shader_test() -> AtmoConfig:
    """Tables of the reference's LUT shader tests, t_atmosphere.clj:44-69."""
    return make_config(height=100000.0, transmittance_shape=(12, 12), surface_radiance_shape=(12, 12),
                       ray_scatter_shape=(12, 12, 12, 12), ray_steps=10, sphere_steps=16, iterations=0,
                       precision=FP64)


SWEEP_SEED = 20261203


def parameter_sweep(n=64, seed=SWEEP_SEED, precision=FP32, ray_scatter_shape=(16, 128, 16, 8),
                    transmittance_shape=(255, 255), surface_radiance_shape=(16, 64), ray_steps=128,
                    sphere_steps=32, iterations=4):
    """`n` atmospheres drawn with numpy's PCG64 from `seed`."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        h_r = rng.uniform(6000.0, 10000.0)
        h_m = rng.uniform(800.0, 2000.0)
        g = rng.uniform(0.6, 0.85)
        s_r = math.exp(rng.uniform(math.log(0.5), math.log(2.0)))
        s_m = math.exp(rng.uniform(math.log(0.5), math.log(2.0)))
        radius = rng.uniform(3000e3, 7000e3)
        ray = component(tuple(s_r * b for b in (5.8e-6, 13.5e-6, 33.1e-6)), h_r)
        mie = component(tuple(s_m * b for b in (2e-5, 2e-5, 2e-5)), h_m, 0.9, g)
        out.append(make_config(radius=radius, height=100000.0, mie=mie, rayleigh=ray,
                               transmittance_shape=transmittance_shape,
                               surface_radiance_shape=surface_radiance_shape,
                               ray_scatter_shape=ray_scatter_shape, ray_steps=ray_steps,
                               sphere_steps=sphere_steps, iterations=iterations, precision=precision))
    return out


def config_array(cfgs):
    arr = (AtmoConfig * len(cfgs))()
    for i, c in enumerate(cfgs):
        arr[i] = c
    return arr

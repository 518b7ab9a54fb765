"""ctypes wrapper of the FP64 CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  The shared library is built by oracle/Makefile into
oracle/_build/libatmo_oracle.so.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from sfsim_gb300.config import AtmoConfig

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libatmo_oracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


class Planet(ctypes.Structure):
    _fields_ = [("centre", ctypes.c_double * 3), ("radius", ctypes.c_double), ("height", ctypes.c_double),
                ("brightness", ctypes.c_double * 3)]


class Comp(ctypes.Structure):
    _fields_ = [("base", ctypes.c_double * 3), ("scale", ctypes.c_double), ("quotient", ctypes.c_double),
                ("g", ctypes.c_double)]


class Intermediates(ctypes.Structure):
    _fields_ = [(n, _dp) for n in ("transmittance_nodes", "surface_base", "rayleigh_first", "mie_first",
                                   "point_scatter", "surface_delta", "ray_scatter_delta")]


class GlslTables(ctypes.Structure):
    _fields_ = [("radius", ctypes.c_float), ("max_height", ctypes.c_float),
                ("t_height_size", ctypes.c_int), ("t_elevation_size", ctypes.c_int),
                ("height_size", ctypes.c_int), ("elevation_size", ctypes.c_int),
                ("light_elevation_size", ctypes.c_int), ("heading_size", ctypes.c_int),
                ("transmittance", _fp), ("ray_scatter", _fp), ("mie_strength", _fp),
                ("weight_bits", ctypes.c_int)]


def build_library(force: bool = False) -> str:
    # make is incremental: it rebuilds only when a source changed
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_library()
        _lib = ctypes.CDLL(_LIB_PATH)
        L = _lib
        L.oracle_phase.restype = ctypes.c_double
        L.oracle_phase.argtypes = [ctypes.c_double, ctypes.c_double]
        for name in ("oracle_height", "oracle_horizon_distance", "oracle_elevation_to_index",
                     "oracle_height_to_index", "oracle_sun_elevation_to_index",
                     "oracle_index_to_sin_sun_elevation", "oracle_sun_angle_to_index", "oracle_limit_quot"):
            getattr(L, name).restype = ctypes.c_double
    return _lib


def _v(x):
    return (ctypes.c_double * 3)(*[float(t) for t in x])


def _out3():
    return (ctypes.c_double * 3)()


def planet(radius=6378000.0, height=100000.0, centre=(0, 0, 0), brightness=(0.3, 0.3, 0.3)) -> Planet:
    p = Planet()
    p.centre[:] = [float(t) for t in centre]
    p.radius = float(radius)
    p.height = float(height)
    p.brightness[:] = [float(t) for t in brightness]
    return p


def comp(base, scale, quotient=1.0, g=0.0) -> Comp:
    c = Comp()
    c.base[:] = [float(t) for t in base]
    c.scale = float(scale)
    c.quotient = float(quotient)
    c.g = float(g)
    return c


def comps(*cs):
    arr = (Comp * len(cs))()
    for i, c in enumerate(cs):
        arr[i] = c
    return arr


MIE = comp((2e-5, 2e-5, 2e-5), 1200.0, 0.9, 0.76)
RAYLEIGH = comp((5.8e-6, 13.5e-6, 33.1e-6), 8000.0)


# --- unit functions -----------------------------------------------------------

def phase(g, mu):
    return lib().oracle_phase(float(g), float(mu))


def scattering(c, h):
    o = _out3()
    lib().oracle_scattering(ctypes.byref(c), ctypes.c_double(h), o)
    return np.array(o[:])


def extinction(c, h):
    o = _out3()
    lib().oracle_extinction(ctypes.byref(c), ctypes.c_double(h), o)
    return np.array(o[:])


def height(p, point):
    return lib().oracle_height(ctypes.byref(p), _v(point))


def ray_sphere_intersection(centre, radius, origin, direction):
    o = (ctypes.c_double * 2)()
    lib().oracle_ray_sphere_intersection(_v(centre), ctypes.c_double(radius), _v(origin), _v(direction), o)
    return o[0], o[1]


def atmosphere_intersection(p, origin, direction):
    o = _out3()
    lib().oracle_atmosphere_intersection(ctypes.byref(p), _v(origin), _v(direction), o)
    return np.array(o[:])


def surface_intersection(p, origin, direction):
    o = _out3()
    lib().oracle_surface_intersection(ctypes.byref(p), _v(origin), _v(direction), o)
    return np.array(o[:])


def surface_point(p, point):
    return bool(lib().oracle_surface_point(ctypes.byref(p), _v(point)))


def is_above_horizon(p, point, direction):
    return bool(lib().oracle_is_above_horizon(ctypes.byref(p), _v(point), _v(direction)))


def ray_extremity(p, origin, direction):
    o = _out3()
    lib().oracle_ray_extremity(ctypes.byref(p), _v(origin), _v(direction), o)
    return np.array(o[:])


def transmittance(p, cs, steps, x, x0):
    o = _out3()
    lib().oracle_transmittance(ctypes.byref(p), cs, len(cs), steps, _v(x), _v(x0), o)
    return np.array(o[:])


def transmittance_dir(p, cs, steps, x, v, above):
    o = _out3()
    lib().oracle_transmittance_dir(ctypes.byref(p), cs, len(cs), steps, _v(x), _v(v), int(above), o)
    return np.array(o[:])


def surface_radiance_base(p, cs, steps, intensity, x, light):
    o = _out3()
    lib().oracle_surface_radiance_base(ctypes.byref(p), cs, len(cs), steps, _v(intensity), _v(x), _v(light), o)
    return np.array(o[:])


def single_scatter(p, cs, component, kind, steps, intensity, x, v, l):
    """kind 0 point-scatter-component, 1 strength-component, 2 point-scatter-base"""
    o = _out3()
    lib().oracle_single_scatter(ctypes.byref(p), cs, len(cs), component, kind, steps, _v(intensity), _v(x), _v(v),
                                _v(l), o)
    return np.array(o[:])


def ray_scatter_single(p, cs, component, kind, steps, intensity, x, v, l, above):
    o = _out3()
    lib().oracle_ray_scatter_single(ctypes.byref(p), cs, len(cs), component, kind, steps, _v(intensity), _v(x),
                                    _v(v), _v(l), int(above), o)
    return np.array(o[:])


def ray_scatter_const(p, cs, steps, J, x, v, l, above):
    o = _out3()
    lib().oracle_ray_scatter_const(ctypes.byref(p), cs, len(cs), steps, _v(J), _v(x), _v(v), _v(l), int(above), o)
    return np.array(o[:])


def ray_scatter_scan_const(p, cs, steps, J, x, v, l, above):
    """ray_scatter_const with the scan-mode transmittances (SCAN_RAYS)."""
    o = _out3()
    lib().oracle_ray_scatter_scan_const(ctypes.byref(p), cs, len(cs), steps, _v(J), _v(x), _v(v), _v(l), int(above),
                                        o)
    return np.array(o[:])


def point_scatter_const(p, cs, dS, dE, sphere_steps, ray_steps, x, v, l):
    o = _out3()
    lib().oracle_point_scatter_const(ctypes.byref(p), cs, len(cs), _v(dS), _v(dE), sphere_steps, ray_steps, _v(x),
                                     _v(v), _v(l), o)
    return np.array(o[:])


def surface_radiance_const(p, dS, steps, x, l):
    o = _out3()
    lib().oracle_surface_radiance_const(ctypes.byref(p), _v(dS), steps, _v(x), _v(l), o)
    return np.array(o[:])


def integral_ray(origin, direction, steps, distance, const=(0, 0, 0), select=(-1, -1, -1)):
    o = _out3()
    lib().oracle_integral_ray(_v(origin), _v(direction), steps, ctypes.c_double(distance), _v(const),
                              (ctypes.c_int * 3)(*select), o)
    return np.array(o[:])


def integral_sphere(steps, normal, const=(0, 0, 0), select=(-1, -1, -1), half=False):
    o = _out3()
    lib().oracle_integral_sphere(int(half), steps, _v(normal), _v(const), (ctypes.c_int * 3)(*select), o)
    return np.array(o[:])


def integrate_circle(steps, const):
    o = _out3()
    lib().oracle_integrate_circle(steps, _v(const), o)
    return np.array(o[:])


def sphere_directions(steps, half=False):
    return lib().oracle_sphere_directions(int(half), steps)


def orthogonal(n):
    o = _out3()
    lib().oracle_orthogonal(_v(n), o)
    return np.array(o[:])


def horizon_distance(p, radius):
    return lib().oracle_horizon_distance(ctypes.byref(p), ctypes.c_double(radius))


def elevation_to_index(p, size, point, direction, above):
    return lib().oracle_elevation_to_index(ctypes.byref(p), size, _v(point), _v(direction), int(above))


def index_to_elevation(p, size, radius, index):
    o = _out3()
    above = lib().oracle_index_to_elevation(ctypes.byref(p), size, ctypes.c_double(radius), ctypes.c_double(index),
                                            o)
    return np.array(o[:]), bool(above)


def height_to_index(p, size, point):
    return lib().oracle_height_to_index(ctypes.byref(p), size, _v(point))


def index_to_height(p, size, index):
    o = _out3()
    lib().oracle_index_to_height(ctypes.byref(p), size, ctypes.c_double(index), o)
    return np.array(o[:])


def sun_elevation_to_index(size, point, light):
    return lib().oracle_sun_elevation_to_index(size, _v(point), _v(light))


def index_to_sin_sun_elevation(size, index):
    return lib().oracle_index_to_sin_sun_elevation(size, ctypes.c_double(index))


def sun_angle_to_index(size, direction, light):
    return lib().oracle_sun_angle_to_index(size, _v(direction), _v(light))


def index_to_sun_direction(size, direction, sin_sun, index):
    o = _out3()
    lib().oracle_index_to_sun_direction(size, _v(direction), ctypes.c_double(sin_sun), ctypes.c_double(index), o)
    return np.array(o[:])


def space_forward(p, space, shape, point, direction=(0, 0, 0), light=(0, 0, 0), above=True):
    n = len(shape)
    o = (ctypes.c_double * n)()
    lib().oracle_space_forward(ctypes.byref(p), space, (ctypes.c_int * n)(*shape), _v(point), _v(direction),
                               _v(light), int(above), o)
    return list(o[:])


def space_backward(p, space, shape, idx):
    n = len(shape)
    pt, d, l = _out3(), _out3(), _out3()
    above = lib().oracle_space_backward(ctypes.byref(p), space, (ctypes.c_int * n)(*shape),
                                        (ctypes.c_double * n)(*[float(t) for t in idx]), pt, d, l)
    return np.array(pt[:]), np.array(d[:]), np.array(l[:]), bool(above)


def interpolate(table, coords):
    table = np.ascontiguousarray(table, dtype=np.float64)
    shape = table.shape[:-1]
    o = _out3()
    lib().oracle_interpolate(len(shape), (ctypes.c_int * len(shape))(*shape), table.ctypes.data_as(_dp),
                             (ctypes.c_double * len(coords))(*[float(c) for c in coords]), o)
    return np.array(o[:])


# --- whole build and single nodes ---------------------------------------------

def _dptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def build(cfg: AtmoConfig, nthreads: int | None = None, intermediates: bool = False):
    """Runs the whole reference build; returns a dict of float64 arrays."""
    t, e, s = cfg.shapes()
    nthreads = nthreads or os.cpu_count() or 1
    T = np.zeros(t + (3,))
    E = np.zeros(e + (3,))
    S = np.zeros((s[0] * s[2], s[1] * s[3], 3))
    M = np.zeros_like(S)
    inter = None
    out = {"transmittance": T, "surface_radiance": E, "ray_scatter": S, "mie_strength": M}
    if intermediates:
        it = cfg.iterations
        d = {
            "transmittance_nodes": np.zeros(t + (3,)),
            "surface_base": np.zeros(e + (3,)),
            "rayleigh_first": np.zeros(s + (3,)),
            "mie_first": np.zeros(s + (3,)),
            "point_scatter": np.zeros((it,) + s + (3,)),
            "surface_delta": np.zeros((it,) + e + (3,)),
            "ray_scatter_delta": np.zeros((it,) + s + (3,)),
        }
        inter = Intermediates(*[_dptr(d[n]) for n, _ in Intermediates._fields_])
        out.update(d)
    rc = lib().oracle_build(ctypes.byref(cfg), int(nthreads), _dptr(T), _dptr(E), _dptr(S), _dptr(M),
                            ctypes.byref(inter) if inter is not None else None)
    assert rc == 0
    return out


def transmittance_node(cfg, i, j):
    o = _out3()
    lib().oracle_transmittance_node(ctypes.byref(cfg), i, j, o)
    return np.array(o[:])


def surface_base_node(cfg, i, k):
    o = _out3()
    lib().oracle_surface_base_node(ctypes.byref(cfg), i, k, o)
    return np.array(o[:])


def first_order_node(cfg, i, j, k, a):
    r, m = _out3(), _out3()
    lib().oracle_first_order_node(ctypes.byref(cfg), i, j, k, a, r, m)
    return np.array(r[:]), np.array(m[:])


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def point_scatter_node(cfg, dS, dE, i, j, k, a, mie_first=None):
    o = _out3()
    dS, dE = _c64(dS), _c64(dE)
    mf = _c64(mie_first) if mie_first is not None else None
    lib().oracle_point_scatter_node(ctypes.byref(cfg), _dptr(dS), _dptr(mf), _dptr(dE), i, j, k, a, o)
    return np.array(o[:])


def ray_scatter_node(cfg, J, i, j, k, a):
    o = _out3()
    J = _c64(J)
    lib().oracle_ray_scatter_node(ctypes.byref(cfg), _dptr(J), i, j, k, a, o)
    return np.array(o[:])


def surface_radiance_node(cfg, dS, i, k, mie_first=None):
    o = _out3()
    dS = _c64(dS)
    mf = _c64(mie_first) if mie_first is not None else None
    lib().oracle_surface_radiance_node(ctypes.byref(cfg), _dptr(dS), _dptr(mf), i, k, o)
    return np.array(o[:])


def remap4_node(cfg, table, i, j, k, a):
    o = _out3()
    table = _c64(table)
    lib().oracle_remap4_node(ctypes.byref(cfg), _dptr(table), i, j, k, a, o)
    return np.array(o[:])


def rendered_inscatter(cfg, x, v, l, jsum=None):
    o = _out3()
    js = _c64(jsum) if jsum is not None else None
    lib().oracle_rendered_inscatter(ctypes.byref(cfg), _dptr(js), _v(x), _v(v), _v(l), o)
    return np.array(o[:])


# --- GLSL consumer restatement --------------------------------------------------

def glsl_query(tables: dict, kind: int, light, p, q, weight_bits: int = 0):
    """kind 0 transmittance_track, 1 transmittance_outer, 2 ray_scatter_track, 3 ray_scatter_outer,
    4 in-scatter at (p, direction q) with the horizon test choosing the table half."""
    T = np.ascontiguousarray(tables["transmittance"], dtype=np.float32)
    S = np.ascontiguousarray(tables["ray_scatter"], dtype=np.float32)
    M = np.ascontiguousarray(tables["mie_strength"], dtype=np.float32)
    t = GlslTables()
    t.radius = tables["radius"]
    t.max_height = tables["max_height"]
    t.t_height_size, t.t_elevation_size = tables["transmittance_shape"]
    (t.height_size, t.elevation_size, t.light_elevation_size, t.heading_size) = tables["ray_scatter_shape"]
    t.transmittance = T.ctypes.data_as(_fp)
    t.ray_scatter = S.ctypes.data_as(_fp)
    t.mie_strength = M.ctypes.data_as(_fp)
    t.weight_bits = weight_bits
    o = (ctypes.c_float * 3)()
    f3 = lambda x: (ctypes.c_float * 3)(*[float(v) for v in x])  # noqa: E731
    lib().oracle_glsl_query(ctypes.byref(t), kind, f3(light), f3(p), f3(q), o)
    return np.array(o[:], dtype=np.float64)


def glsl_query_batch(tables: dict, kind: int, light, p, q, weight_bits: int = 0):
    """glsl_query over n queries at once.  light, p and q are [n][3] arrays
    that are rounded to float32 first (the inputs the CUDA lookups receive);
    returns (float32 [n][3] results, bool [n] is-above-horizon of each query)."""
    T = np.ascontiguousarray(tables["transmittance"], dtype=np.float32)
    S = np.ascontiguousarray(tables["ray_scatter"], dtype=np.float32)
    M = np.ascontiguousarray(tables["mie_strength"], dtype=np.float32)
    t = GlslTables()
    t.radius = tables["radius"]
    t.max_height = tables["max_height"]
    t.t_height_size, t.t_elevation_size = tables["transmittance_shape"]
    (t.height_size, t.elevation_size, t.light_elevation_size, t.heading_size) = tables["ray_scatter_shape"]
    t.transmittance = T.ctypes.data_as(_fp)
    t.ray_scatter = S.ctypes.data_as(_fp)
    t.mie_strength = M.ctypes.data_as(_fp)
    t.weight_bits = weight_bits
    f32 = [np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, 3)) for a in (light, p, q)]
    n = f32[1].shape[0]
    out = np.empty((n, 3), dtype=np.float32)
    above = np.empty(n, dtype=np.int32)
    L = lib()
    L.oracle_glsl_query_batch.argtypes = [ctypes.POINTER(GlslTables), ctypes.c_int, ctypes.c_long, _fp, _fp, _fp,
                                          _fp, _ip]
    L.oracle_glsl_query_batch(ctypes.byref(t), kind, n, *[a.ctypes.data_as(_fp) for a in f32],
                              out.ctypes.data_as(_fp), above.ctypes.data_as(_ip))
    return out, above.astype(bool)


def glsl_attenuation_batch(tables: dict, kind: int, light, p, d=None, s=None, incoming=None,
                           amplification: float = 1.0, weight_bits: int = 0):
    """n attenuation queries (atmo_oracle.c oracle_glsl_attenuation_batch):
    kind 0 attenuation_outer(light, p, d, s[0], incoming.rgb), 1
    attenuation_track(light, p, d, s, incoming), 2 attenuation_point(p,
    incoming) with the eye d, 3 transmittance_point(p).  Inputs are rounded to
    float32 first; returns float32 [n][4]."""
    T = np.ascontiguousarray(tables["transmittance"], dtype=np.float32)
    S = np.ascontiguousarray(tables["ray_scatter"], dtype=np.float32)
    M = np.ascontiguousarray(tables["mie_strength"], dtype=np.float32)
    t = GlslTables()
    t.radius = tables["radius"]
    t.max_height = tables["max_height"]
    t.t_height_size, t.t_elevation_size = tables["transmittance_shape"]
    (t.height_size, t.elevation_size, t.light_elevation_size, t.heading_size) = tables["ray_scatter_shape"]
    t.transmittance = T.ctypes.data_as(_fp)
    t.ray_scatter = S.ctypes.data_as(_fp)
    t.mie_strength = M.ctypes.data_as(_fp)
    t.weight_bits = weight_bits

    def f32(a, w):
        return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, w))
    lt, pt, dt, st, it = f32(light, 3), f32(p, 3), f32(d, 3), f32(s, 2), f32(incoming, 4)
    n = pt.shape[0]
    out = np.empty((n, 4), dtype=np.float32)
    ptr = lambda a: None if a is None else a.ctypes.data_as(_fp)  # noqa: E731
    L = lib()
    L.oracle_glsl_attenuation_batch.argtypes = [ctypes.POINTER(GlslTables), ctypes.c_int, ctypes.c_long, _fp, _fp,
                                                _fp, _fp, _fp, ctypes.c_float, _fp]
    L.oracle_glsl_attenuation_batch(ctypes.byref(t), kind, n, ptr(lt), ptr(pt), ptr(dt), ptr(st), ptr(it),
                                    amplification, out.ctypes.data_as(_fp))
    return out


# --- cloud-noise builders (noise_oracle.c) ----------------------------------------

def worley(divisions: int, size: int, grid):
    """worley-noise (worley.clj:96-109) for a given point grid [d][d][d][3]."""
    g = np.ascontiguousarray(grid, dtype=np.float64)
    assert g.shape == (divisions, divisions, divisions, 3)
    out = np.zeros(size ** 3, np.float64)
    lib().noise_worley(divisions, size, g.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
    return out


def worley_closest(grid, divisions: int, size: int, point):
    """closest-distance-to-point-in-grid on a grid [nk][nj][ni][3]."""
    g = np.ascontiguousarray(grid, dtype=np.float64)
    f = lib().noise_worley_closest_grid
    f.restype = ctypes.c_double
    return f(g.ctypes.data_as(_dp), g.shape[0], g.shape[1], g.shape[2], divisions, size, _v(point))


def perlin(divisions: int, size: int, gradients):
    """perlin-noise (perlin.clj:122-133) for gradient indices [d][d][d] into the twelve vectors."""
    g = np.ascontiguousarray(gradients, dtype=np.int32)
    assert g.shape == (divisions, divisions, divisions)
    out = np.zeros(size ** 3, np.float64)
    lib().noise_perlin(divisions, size, g.ctypes.data_as(_ip), out.ctypes.data_as(_dp))
    return out


def perlin_sample(gradients, divisions: int, size: int, cell):
    g = np.ascontiguousarray(gradients, dtype=np.int32)
    f = lib().noise_perlin_sample
    f.restype = ctypes.c_double
    return f(g.ctypes.data_as(_ip), divisions, size, _v(cell))


def perlin_ease(t: float) -> float:
    f = lib().noise_perlin_ease
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double]
    return f(t)


def blue(m: int, seed_indices, sigma: float):
    """blue-noise (bluenoise.clj:162-172) from the given seed pixels; returns m*m ranks."""
    seed = np.ascontiguousarray(seed_indices, dtype=np.int32)
    out = np.zeros(m * m, np.int32)
    f = lib().noise_blue
    f.argtypes = [ctypes.c_int, ctypes.c_int, _ip, ctypes.c_double, _ip]
    assert f(m, len(seed), seed.ctypes.data_as(_ip), sigma, out.ctypes.data_as(_ip)) == 0
    return out


def blue_table(m: int, sigma: float):
    t = np.zeros((m // 2 + 1) ** 2, np.float64)
    f = lib().noise_blue_table
    f.argtypes = [ctypes.c_int, ctypes.c_double, _dp]
    f(m, sigma, t.ctypes.data_as(_dp))
    return t


def blue_density_array(mask, m: int, sigma: float):
    msk = np.ascontiguousarray(mask, dtype=np.uint8)
    t = blue_table(m, sigma)
    out = np.zeros(m * m, np.float64)
    lib().noise_blue_density_array(msk.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), m, t.ctypes.data_as(_dp),
                                   out.ctypes.data_as(_dp))
    return out


def blue_seed_pattern(mask, m: int, sigma: float):
    msk = np.array(mask, dtype=np.uint8)
    t = blue_table(m, sigma)
    lib().noise_blue_seed_pattern(msk.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), m, t.ctypes.data_as(_dp))
    return msk.astype(bool)


def blue_wrap(x: int, m: int) -> int:
    return lib().noise_blue_wrap(x, m)


def blue_phase(phase: int, mask, m: int, n: int, sigma: float, dither):
    """dither-phase1/2/3 (bluenoise.clj:127-169) from a mask; returns (dither, mask after the phase)."""
    msk = np.array(mask, dtype=np.uint8)
    d = np.array(dither, dtype=np.int32)
    f = lib().noise_blue_phase
    f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_ubyte), ctypes.c_int, ctypes.c_int, ctypes.c_double, _ip]
    f(phase, msk.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), m, n, sigma, d.ctypes.data_as(_ip))
    return d, msk.astype(bool)

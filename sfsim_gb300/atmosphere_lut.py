"""Atmosphere lookup-table build on the GPU; the drop-in for
src/clj/sfsim/atmosphere_lut.clj (generate-atmosphere-luts).

`generate_atmosphere_luts()` writes the same four files as the reference
(atmosphere_lut.clj:102-105) in the same layout: little-endian float32, RGB
interleaved, no header; the 4-D tables tiled 2-D as convert-4d-to-2d does
(image.clj:299-312).  The tables come from libsfsim_atmo.so.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from .config import AtmoConfig, config_array, reference_production

FILES = ("transmittance.scatter", "surface-radiance.scatter", "ray-scatter.scatter", "mie-strength.scatter")


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def table_shapes(cfg: AtmoConfig):
    """numpy shapes of the four outputs in the .scatter layout."""
    t, e, s = cfg.shapes()
    four = (s[0] * s[2], s[1] * s[3], 3)
    return (t[0], t[1], 3), (e[0], e[1], 3), four, four


def build(cfg: AtmoConfig | None = None, intermediates: bool = False):
    """Builds the four tables; returns a dict of float32 arrays (and the
    intermediate tables in plain [..][3] order when `intermediates`)."""
    cfg = cfg if cfg is not None else reference_production()
    L = _lib.load()
    _lib.check(L.sfsim_atmo_validate(ctypes.byref(cfg)), "sfsim_atmo_validate")
    sT, sE, sS, sM = table_shapes(cfg)
    out = {"transmittance": np.empty(sT, np.float32), "surface_radiance": np.empty(sE, np.float32),
           "ray_scatter": np.empty(sS, np.float32), "mie_strength": np.empty(sM, np.float32)}
    args = [ctypes.byref(cfg)] + [_fptr(out[k]) for k in ("transmittance", "surface_radiance", "ray_scatter",
                                                          "mie_strength")]
    if not intermediates:
        _lib.check(L.sfsim_atmo_build(*args), "sfsim_atmo_build")
        return out
    t, e, s = cfg.shapes()
    it = cfg.iterations
    inter = {
        "transmittance_nodes": np.zeros(t + (3,), np.float32),
        "surface_base": np.zeros(e + (3,), np.float32),
        "rayleigh_first": np.zeros(s + (3,), np.float32),
        "mie_first": np.zeros(s + (3,), np.float32),
        "point_scatter": np.zeros((it,) + s + (3,), np.float32),
        "surface_delta": np.zeros((it,) + e + (3,), np.float32),
        "ray_scatter_delta": np.zeros((it,) + s + (3,), np.float32),
    }
    st = _lib.Intermediates(*[_fptr(inter[n]) if inter[n].size else None for n, _ in _lib.Intermediates._fields_])
    _lib.check(L.sfsim_atmo_build_debug(*args, ctypes.byref(st)), "sfsim_atmo_build_debug")
    out.update(inter)
    return out


STATE_TABLES = ("ray_scatter_delta", "surface_delta", "ray_scatter_sum", "surface_sum")


def empty_iteration_state(cfg: AtmoConfig) -> dict:
    """Host buffers of one iteration state (sfsim_atmo_iteration_state): node
    records of four values in the build's precision, 4-D tables
    [h][el][sun el][heading][4], 2-D tables [h][sun el][4]."""
    from .config import FP64
    dt = np.float64 if cfg.precision == FP64 else np.float32
    _, e, s = cfg.shapes()
    return {"ray_scatter_delta": np.zeros(s + (4,), dt), "surface_delta": np.zeros(e + (4,), dt),
            "ray_scatter_sum": np.zeros(s + (4,), dt), "surface_sum": np.zeros(e + (4,), dt)}


def _state_struct(iteration: int, tables: dict) -> "_lib.IterationState":
    return _lib.IterationState(iteration, *[tables[k].ctypes.data for k in STATE_TABLES])


def build_resumable(cfg: AtmoConfig, resume: tuple | None = None, on_iteration=None):
    """Builds the four tables with a state after every iteration
    (sfsim_atmo_build_resumable).  `resume`: (iteration, tables) saved from
    an earlier build of the same config; the build continues after that
    iteration.  `on_iteration(iteration, tables)` sees each iteration's state
    (arrays the next iteration overwrites: copy what you keep) and stops the
    build by returning True (AtmoError with code SFSIM_ATMO_ESTOPPED); an
    exception it raises stops the build and is raised again here."""
    L = _lib.load()
    _lib.check(L.sfsim_atmo_validate(ctypes.byref(cfg)), "sfsim_atmo_validate")
    sT, sE, sS, sM = table_shapes(cfg)
    out = {"transmittance": np.empty(sT, np.float32), "surface_radiance": np.empty(sE, np.float32),
           "ray_scatter": np.empty(sS, np.float32), "mie_strength": np.empty(sM, np.float32)}
    rs = None
    if resume is not None:
        iteration, tables = resume
        want = empty_iteration_state(cfg)
        tables = {k: np.ascontiguousarray(tables[k], dtype=want[k].dtype) for k in STATE_TABLES}
        for k in STATE_TABLES:
            if tables[k].shape != want[k].shape:
                raise ValueError(f"resume table {k} has shape {tables[k].shape}, the config needs {want[k].shape}")
        rs = _state_struct(int(iteration), tables)
    state_tables = empty_iteration_state(cfg) if on_iteration is not None else None
    st = _state_struct(0, state_tables) if state_tables is not None else None
    raised = []

    def hook(p, _user):
        try:
            return 1 if on_iteration(p.contents.iteration, state_tables) else 0
        except BaseException as e:  # it cannot cross the C ABI: stop the build, raise it below
            raised.append(e)
            return 1
    fn = _lib.ITERATION_FN(hook) if on_iteration is not None else _lib.ITERATION_FN()
    rc = L.sfsim_atmo_build_resumable(ctypes.byref(cfg), ctypes.byref(rs) if rs is not None else None,
                                      ctypes.byref(st) if st is not None else None, fn, None,
                                      *[_fptr(out[k]) for k in ("transmittance", "surface_radiance",
                                                                "ray_scatter", "mie_strength")])
    if raised:
        raise raised[0]
    _lib.check(rc, "sfsim_atmo_build_resumable")
    return out


def save_iteration_state(path: str, iteration: int, tables: dict) -> None:
    """Writes an iteration state to an .npz file."""
    np.savez(path, iteration=np.int64(iteration), **{k: tables[k] for k in STATE_TABLES})


def load_iteration_state(path: str) -> tuple:
    """Reads an iteration state written by save_iteration_state: (iteration, tables)."""
    with np.load(path) as z:
        return int(z["iteration"]), {k: z[k].copy() for k in STATE_TABLES}


def build_batch(cfgs):
    """Builds len(cfgs) atmospheres sharing shapes and steps in one batched pass."""
    L = _lib.load()
    n = len(cfgs)
    arr = config_array(cfgs)
    sT, sE, sS, sM = table_shapes(cfgs[0])
    out = {"transmittance": np.empty((n,) + sT, np.float32), "surface_radiance": np.empty((n,) + sE, np.float32),
           "ray_scatter": np.empty((n,) + sS, np.float32), "mie_strength": np.empty((n,) + sM, np.float32)}
    _lib.check(L.sfsim_atmo_build_batch(arr, n, *[_fptr(out[k]) for k in ("transmittance", "surface_radiance",
                                                                           "ray_scatter", "mie_strength")]),
               "sfsim_atmo_build_batch")
    return out


def build_device(cfg: AtmoConfig, tensors=None, stream=None):
    """Builds into torch CUDA tensors (allocated when `tensors` is None) on
    `stream` (torch.cuda.Stream, default: the current stream)."""
    import torch
    L = _lib.load()
    if tensors is None:
        tensors = [torch.empty(s, dtype=torch.float32, device="cuda") for s in table_shapes(cfg)]
    st = stream if stream is not None else torch.cuda.current_stream()
    _lib.check(L.sfsim_atmo_build_device(ctypes.byref(cfg), *[t.data_ptr() for t in tensors],
                                         ctypes.c_void_p(st.cuda_stream)), "sfsim_atmo_build_device")
    return tensors


class Plan:
    """A build prepared once (sfsim_atmo_plan_*): `build(tensors, stream)`
    only launches kernels, so it can be captured into a torch CUDA graph and
    replayed."""

    def __init__(self, cfg: AtmoConfig):
        self.cfg = cfg.copy()
        self._L = _lib.load()
        self._ptr = ctypes.c_void_p()
        _lib.check(self._L.sfsim_atmo_plan_create(ctypes.byref(self.cfg), ctypes.byref(self._ptr)), "plan_create")

    def build(self, tensors=None, stream=None):
        import torch
        if tensors is None:
            tensors = [torch.empty(s, dtype=torch.float32, device="cuda") for s in table_shapes(self.cfg)]
        st = stream if stream is not None else torch.cuda.current_stream()
        _lib.check(self._L.sfsim_atmo_plan_build(self._ptr, *[t.data_ptr() for t in tensors],
                                                 ctypes.c_void_p(st.cuda_stream)), "plan_build")
        return tensors

    def close(self):
        if self._ptr:
            self._L.sfsim_atmo_plan_destroy(self._ptr)
            self._ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def spit_floats(path: str, data: np.ndarray) -> None:
    """util.clj:236-240: raw little-endian float32."""
    np.ascontiguousarray(data, dtype="<f4").tofile(path)


def generate_atmosphere_luts(out_dir: str = "data/atmosphere", cfg: AtmoConfig | None = None) -> dict:
    """Program to generate lookup tables for atmospheric scattering
    (atmosphere_lut.clj:43-105).  Returns the written paths."""
    tables = build(cfg)
    os.makedirs(out_dir, exist_ok=True)
    paths = {}
    for key, name in zip(("transmittance", "surface_radiance", "ray_scatter", "mie_strength"), FILES):
        p = os.path.join(out_dir, name)
        spit_floats(p, tables[key])
        paths[key] = p
    return paths


def stage_timings(enabled: bool = True):
    """Enables per-stage CUDA-event timing; returns a reader of the last build's timings."""
    L = _lib.load()
    L.sfsim_atmo_set_timing(1 if enabled else 0)

    def read():
        ms = (ctypes.c_double * 10)()
        n = L.sfsim_atmo_last_timings(ms, 10)
        names = ("setup", "transmittance", "surface_base", "first_order", "reserved", "point_scatter",
                 "surface_radiance", "ray_scatter", "accumulate", "output")
        return {names[i]: ms[i] for i in range(max(n, 0))}

    return read


def last_launch_count() -> int:
    return int(_lib.load().sfsim_atmo_last_launch_count())

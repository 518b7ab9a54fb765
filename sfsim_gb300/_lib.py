"""ctypes binding of libsfsim_atmo.so, the C ABI declared in include/sfsim_atmo.h.

The library is the only compute path: when it cannot be loaded every entry
point raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from .config import AtmoConfig

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsfsim_atmo.so")

_fp = ctypes.POINTER(ctypes.c_float)
_cfgp = ctypes.POINTER(AtmoConfig)

# every exported symbol of include/sfsim_atmo.h
EXPORTS = (
    "sfsim_atmo_default_config", "sfsim_atmo_validate", "sfsim_atmo_table_sizes", "sfsim_atmo_build",
    "sfsim_atmo_build_device", "sfsim_atmo_build_batch", "sfsim_atmo_build_debug", "sfsim_atmo_set_timing",
    "sfsim_atmo_last_timings", "sfsim_atmo_last_launch_count", "sfsim_atmo_release", "sfsim_atmo_strerror",
    "sfsim_atmo_last_error", "sfsim_atmo_version", "sfsim_atmo_census", "sfsim_atmo_sfu_peak",
    "sfsim_atmo_build_static", "sfsim_atmo_context_create", "sfsim_atmo_context_destroy",
    "sfsim_atmo_context_tables", "sfsim_atmo_context_point_scatter_sum", "sfsim_atmo_query_table",
    "sfsim_atmo_query_direct", "sfsim_atmo_gemm_bf16", "sfsim_atmo_surrogate_train",
    "sfsim_atmo_surrogate_parameters", "sfsim_atmo_surrogate_gradients", "sfsim_atmo_query_surrogate",
    "sfsim_atmo_query_coords", "sfsim_atmo_smem_peak", "sfsim_noise_worley", "sfsim_noise_perlin", "sfsim_noise_blue",
    "sfsim_atmo_condition_inputs", "sfsim_atmo_cond_surrogate_create", "sfsim_atmo_cond_surrogate_destroy",
    "sfsim_atmo_cond_surrogate_train", "sfsim_atmo_cond_surrogate_parameters", "sfsim_atmo_cond_surrogate_gradients",
    "sfsim_atmo_query_cond_surrogate", "sfsim_atmo_plan_create", "sfsim_atmo_plan_build", "sfsim_atmo_plan_destroy",
    "sfsim_atmo_set_wait_limit", "sfsim_atmo_wait_selftest", "sfsim_atmo_last_transfer_bytes",
    "sfsim_atmo_iteration_state_bytes", "sfsim_atmo_build_resumable", "sfsim_atmo_query_attenuation",
)


class SurrogateConfig(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("batch", ctypes.c_int), ("direct_samples", ctypes.c_longlong),
                ("node_fraction", ctypes.c_float), ("lr", ctypes.c_float), ("seed", ctypes.c_ulonglong),
                ("huber_delta", ctypes.c_float)]


class Intermediates(ctypes.Structure):
    _fields_ = [(n, _fp) for n in ("transmittance_nodes", "surface_base", "rayleigh_first", "mie_first",
                                   "point_scatter", "surface_delta", "ray_scatter_delta")]


class IterationState(ctypes.Structure):
    """sfsim_atmo_iteration_state: the four tables carried from one iteration to the next."""
    _fields_ = [("iteration", ctypes.c_int), ("ray_scatter_delta", ctypes.c_void_p), ("surface_delta", ctypes.c_void_p),
                ("ray_scatter_sum", ctypes.c_void_p), ("surface_sum", ctypes.c_void_p)]


ITERATION_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(IterationState), ctypes.c_void_p)


class AtmoError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str):
        super().__init__(f"{where} failed with {code}: {detail}")
        self.code = code


_lib = None


def load(build: bool = False):
    """Loads the library (building it first when `build`); raises when absent."""
    global _lib
    if _lib is not None:
        return _lib
    if build:
        from .build import build_library
        build_library()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run `python -m sfsim_gb300.build` (needs nvcc)")
    L = ctypes.CDLL(LIB_PATH)
    L.sfsim_atmo_default_config.argtypes = [_cfgp]
    L.sfsim_atmo_default_config.restype = None
    L.sfsim_atmo_validate.argtypes = [_cfgp]
    L.sfsim_atmo_table_sizes.argtypes = [_cfgp] + [ctypes.POINTER(ctypes.c_size_t)] * 4
    L.sfsim_atmo_build.argtypes = [_cfgp, _fp, _fp, _fp, _fp]
    L.sfsim_atmo_build_device.argtypes = [_cfgp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
    L.sfsim_atmo_build_static.argtypes = [_cfgp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
    L.sfsim_atmo_build_batch.argtypes = [_cfgp, ctypes.c_int, _fp, _fp, _fp, _fp]
    L.sfsim_atmo_build_debug.argtypes = [_cfgp, _fp, _fp, _fp, _fp, ctypes.POINTER(Intermediates)]
    L.sfsim_atmo_set_timing.argtypes = [ctypes.c_int]
    L.sfsim_atmo_last_timings.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    L.sfsim_atmo_last_launch_count.argtypes = []
    L.sfsim_atmo_release.argtypes = []
    L.sfsim_atmo_strerror.argtypes = [ctypes.c_int]
    L.sfsim_atmo_strerror.restype = ctypes.c_char_p
    L.sfsim_atmo_last_error.argtypes = []
    L.sfsim_atmo_last_error.restype = ctypes.c_char_p
    L.sfsim_atmo_census.argtypes = [_cfgp, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]
    L.sfsim_atmo_sfu_peak.argtypes = [ctypes.POINTER(ctypes.c_double)]
    L.sfsim_atmo_smem_peak.argtypes = [ctypes.POINTER(ctypes.c_double)]
    vp = ctypes.c_void_p
    L.sfsim_atmo_context_create.argtypes = [_cfgp, ctypes.POINTER(vp)]
    L.sfsim_atmo_context_destroy.argtypes = [vp]
    L.sfsim_atmo_context_tables.argtypes = [vp] + [ctypes.POINTER(vp)] * 4
    L.sfsim_atmo_context_point_scatter_sum.argtypes = [vp, ctypes.POINTER(vp)]
    L.sfsim_atmo_query_table.argtypes = [vp, ctypes.c_int, ctypes.c_longlong, vp, vp, vp, vp, ctypes.c_int, vp]
    L.sfsim_atmo_query_direct.argtypes = [vp, ctypes.c_longlong, vp, vp, vp, vp, vp]
    L.sfsim_atmo_query_attenuation.argtypes = [vp, ctypes.c_int, ctypes.c_longlong, vp, vp, vp, vp, vp,
                                               ctypes.c_float, vp, ctypes.c_int, vp]
    L.sfsim_atmo_gemm_bf16.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_longlong, ctypes.c_int, vp]
    L.sfsim_atmo_surrogate_train.argtypes = [vp, ctypes.POINTER(SurrogateConfig), vp]
    L.sfsim_atmo_surrogate_parameters.argtypes = [vp, vp, vp, ctypes.POINTER(ctypes.c_longlong)]
    L.sfsim_atmo_surrogate_gradients.argtypes = [vp, ctypes.c_longlong, vp, vp, vp, vp]
    L.sfsim_atmo_query_surrogate.argtypes = [vp, ctypes.c_longlong, vp, vp, vp, vp, ctypes.c_float,
                                             ctypes.POINTER(ctypes.c_longlong), vp]
    L.sfsim_atmo_query_coords.argtypes = [vp, ctypes.c_longlong, vp, vp, vp, vp, vp]
    L.sfsim_atmo_condition_inputs.argtypes = [_cfgp, vp]
    L.sfsim_atmo_plan_create.argtypes = [_cfgp, ctypes.POINTER(vp)]
    L.sfsim_atmo_plan_build.argtypes = [vp, vp, vp, vp, vp, vp]
    L.sfsim_atmo_plan_destroy.argtypes = [vp]
    L.sfsim_atmo_cond_surrogate_create.argtypes = [ctypes.c_ulonglong, ctypes.POINTER(vp)]
    L.sfsim_atmo_cond_surrogate_destroy.argtypes = [vp]
    L.sfsim_atmo_cond_surrogate_train.argtypes = [vp, vp, ctypes.c_int, ctypes.POINTER(SurrogateConfig), vp]
    L.sfsim_atmo_cond_surrogate_parameters.argtypes = [vp, vp, vp, ctypes.POINTER(ctypes.c_longlong)]
    L.sfsim_atmo_cond_surrogate_gradients.argtypes = [vp, ctypes.c_longlong, vp, vp, ctypes.c_int, vp, vp, vp, vp]
    L.sfsim_atmo_query_cond_surrogate.argtypes = [vp, vp, ctypes.c_longlong, vp, vp, vp, vp, ctypes.c_float,
                                                  ctypes.POINTER(ctypes.c_longlong), vp]
    L.sfsim_noise_worley.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp]
    L.sfsim_noise_perlin.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp]
    L.sfsim_noise_blue.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_double, vp]
    L.sfsim_atmo_set_wait_limit.argtypes = [ctypes.c_longlong]
    L.sfsim_atmo_set_wait_limit.restype = ctypes.c_longlong
    L.sfsim_atmo_wait_selftest.argtypes = [ctypes.c_int]
    L.sfsim_atmo_last_transfer_bytes.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)] * 2
    L.sfsim_atmo_iteration_state_bytes.argtypes = [_cfgp, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    L.sfsim_atmo_build_resumable.argtypes = [_cfgp, ctypes.POINTER(IterationState), ctypes.POINTER(IterationState), ITERATION_FN,
                                          ctypes.c_void_p, _fp, _fp, _fp, _fp]
    L.sfsim_atmo_version.argtypes = []
    L.sfsim_atmo_version.restype = ctypes.c_char_p
    _lib = L
    return L


def check(rc: int, where: str) -> None:
    if rc < 0:
        L = load()
        detail = (L.sfsim_atmo_last_error() or b"").decode() or L.sfsim_atmo_strerror(rc).decode()
        raise AtmoError(rc, where, detail)

"""sfsim_gb300: GB300 (sm_103a) build of sfsim's atmosphere lookup tables.

The compute path is libsfsim_atmo.so (CUDA, C ABI in include/sfsim_atmo.h);
this package holds its ctypes binding, the configuration records and the
`generate_atmosphere_luts` entry point that mirrors
src/clj/sfsim/atmosphere_lut.clj.
"""
from .config import AtmoConfig, Component, FP32, FP64  # noqa: F401

__version__ = "0.1.0"

"""CPU checks of the C ABI: the library loads, exports every function that
include/sfsim_atmo.h declares, validates configurations and reports errors
without touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from sfsim_gb300 import _lib, config as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    return _lib.load(build=True)


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            names.update(re.findall(r"\b(sfsim_atmo_\w+)\s*\(", text))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(_lib.EXPORTS) | set(names)


def test_default_config_matches_reference(lib):
    c = C.AtmoConfig()
    lib.sfsim_atmo_default_config(ctypes.byref(c))
    ref = C.reference_production()
    assert bytes(c) == bytes(ref)


def test_table_sizes(lib):
    c = C.production()
    n = [ctypes.c_size_t() for _ in range(4)]
    assert lib.sfsim_atmo_table_sizes(ctypes.byref(c), *[ctypes.byref(x) for x in n]) == 0
    assert [x.value for x in n] == list(c.table_sizes())
    assert n[2].value == 3 * 32 * 255 * 32 * 8


@pytest.mark.parametrize("field,value,code", [
    ("radius", -1.0, -1), ("height", 0.0, -1), ("ray_steps", 0, -1), ("iterations", -1, -1),
    ("precision", 7, -1), ("flags", 2, -1), ("flags", -1, -1), ("sphere_steps", 1, -1),
])
def test_validate_rejects(lib, field, value, code):
    c = C.production()
    setattr(c, field, value)
    assert lib.sfsim_atmo_validate(ctypes.byref(c)) == code
    assert lib.sfsim_atmo_last_error()


def test_validate_accepts_scan_rays(lib):
    c = C.production()
    c.flags = C.SCAN_RAYS
    assert lib.sfsim_atmo_validate(ctypes.byref(c)) == 0


def test_validate_shapes(lib):
    c = C.production()
    c.ray_scatter_shape[1] = 1
    assert lib.sfsim_atmo_validate(ctypes.byref(c)) == -5
    c = C.production()
    c.mie.scatter_g = 1.0
    assert lib.sfsim_atmo_validate(ctypes.byref(c)) == -1


def test_validate_limits(lib):
    """The remaining configuration checks, all on the host: a ray-scatter table
    over 2^31 nodes, non-finite or negative physical values, surface radiance
    without its ray_steps/4 rings, and the step limits."""
    def code(**kw):
        c = C.production()
        for k, v in kw.items():
            if k == "shape":
                for i, x in enumerate(v):
                    c.ray_scatter_shape[i] = x
            elif k in ("mie_base", "ray_scale"):
                if k == "mie_base":
                    c.mie.scatter_base[0] = v
                else:
                    c.rayleigh.scatter_scale = v
            else:
                setattr(c, k, v)
        return lib.sfsim_atmo_validate(ctypes.byref(c))
    assert code() == 0
    assert code(shape=(2048, 1024, 32, 33)) == -7          # 2^31 + 2^26 nodes
    assert code(shape=(2048, 1024, 32, 32)) == 0           # exactly 2^31
    assert code(radius=float("nan")) == -1
    assert code(height=float("inf")) == -1
    assert code(mie_base=-1e-6) == -1
    assert code(ray_scale=0.0) == -1
    assert code(ray_steps=3) == -1                         # iterations > 0 need 4 rings' worth
    assert code(ray_steps=3, iterations=0) == 0
    assert code(ray_steps=4097) == -1
    assert code(sphere_steps=1025) == -1
    assert code(sphere_steps=1) == -1                      # iterations need a sphere
    assert code(sphere_steps=0, iterations=0) == 0         # a first-order build needs none
    assert code(sphere_steps=1 << 20, iterations=0) == -1  # bounded even when unused
    assert code(sphere_steps=-2, iterations=0) == -1
    assert code(iterations=65) == -1


def test_batch_size_limits(lib):
    """Batches of 0 or of more than 65535 atmospheres are refused before any
    device work (each atmosphere is one grid row of the batched kernels)."""
    cfgs = (C.AtmoConfig * 65536)()
    out = (ctypes.c_float * 4)()
    assert lib.sfsim_atmo_build_batch(cfgs, 0, out, out, out, out) == -1
    assert lib.sfsim_atmo_build_batch(cfgs, 65536, out, out, out, out) == -7


def test_null_outputs(lib):
    c = C.small_fp64()
    assert lib.sfsim_atmo_build(ctypes.byref(c), None, None, None, None) == -6


def test_iteration_state_bytes(lib):
    c = C.production()
    s, e = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.sfsim_atmo_iteration_state_bytes(ctypes.byref(c), ctypes.byref(s), ctypes.byref(e)) == 0
    assert s.value == 4 * 4 * 32 * 255 * 32 * 8 and e.value == 4 * 4 * 16 * 64
    c.precision = C.FP64
    assert lib.sfsim_atmo_iteration_state_bytes(ctypes.byref(c), ctypes.byref(s), ctypes.byref(e)) == 0
    assert s.value == 8 * 4 * 32 * 255 * 32 * 8


def test_build_resumable_rejects_bad_states(lib):
    """Resume states are checked on the host before any device work: an
    iteration outside [1, iterations] and a missing table are refused."""
    c = C.small_fp64()
    buf = (ctypes.c_double * 16)()
    full = lambda it: _lib.IterationState(it, *[ctypes.addressof(buf)] * 4)
    outs = [(ctypes.c_float * 4)() for _ in range(4)]
    fp = [ctypes.cast(o, ctypes.POINTER(ctypes.c_float)) for o in outs]
    none = _lib.ITERATION_FN()
    for it in (0, -1, c.iterations + 1):
        st = full(it)
        assert lib.sfsim_atmo_build_resumable(ctypes.byref(c), ctypes.byref(st), None, none, None, *fp) == -1
    st = full(1)
    st.surface_sum = None
    assert lib.sfsim_atmo_build_resumable(ctypes.byref(c), ctypes.byref(st), None, none, None, *fp) == -6
    assert lib.sfsim_atmo_build_resumable(ctypes.byref(c), None, ctypes.byref(st), none, None, *fp) == -6
    assert lib.sfsim_atmo_build_resumable(ctypes.byref(c), None, None, none, None, fp[0], None, fp[2], fp[3]) == -6


def test_strerror(lib):
    for code in range(0, -10, -1):
        assert lib.sfsim_atmo_strerror(code)
    assert lib.sfsim_atmo_version().startswith(b"sfsim-atmo-gb300")


def test_no_gpu_reports_enodev(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    c = C.small_fp64()
    a = np.zeros(c.table_sizes()[2], np.float32)
    p = a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert lib.sfsim_atmo_build(ctypes.byref(c), p, p, p, p) == -4


def test_batch_layout_mismatch_rejected(lib):
    a, b = C.small_fp64(), C.small_fp64()
    b.ray_steps = 32
    arr = C.config_array([a, b])
    x = np.zeros(10, np.float32)
    p = x.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert lib.sfsim_atmo_build_batch(arr, 2, p, p, p, p) == -1


def test_condition_inputs(lib):
    """The conditioned surrogate's atmosphere inputs (host-only): Earth's
    coefficients give 0 in the coefficient inputs, the sweep's ranges map to
    about [-1, 1]."""
    from sfsim_gb300.query import condition_inputs
    g = condition_inputs(C.production())
    assert g.shape == (8,)
    np.testing.assert_allclose(g[:4], 0.0, atol=1e-6)
    np.testing.assert_allclose(g[4:], [0.0, (1200.0 - 1400.0) / 600.0, (0.76 - 0.725) / 0.125,
                                       (6378e3 - 5e6) / 2e6], rtol=1e-6, atol=1e-6)
    for cfg in C.parameter_sweep(64):
        g = condition_inputs(cfg)
        assert np.all(np.abs(g) <= 1.0 + 1e-5), g
        ref = [np.log2(cfg.rayleigh.scatter_base[0] / 5.8e-6), np.log2(cfg.mie.scatter_base[0] / 2e-5),
               (cfg.radius - 5e6) / 2e6]
        np.testing.assert_allclose([g[0], g[3], g[7]], ref, rtol=1e-5, atol=1e-6)
    assert lib.sfsim_atmo_condition_inputs(None, None) == -6


def test_no_gpu_new_entry_points_report_enodev(lib):
    """Plans and conditioned surrogates report ENODEV without a GPU, like the
    builds, and leave their out-pointer NULL."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    c = C.small_fp64()
    p = ctypes.c_void_p(1)
    assert lib.sfsim_atmo_plan_create(ctypes.byref(c), ctypes.byref(p)) == -4
    assert not p.value
    q = ctypes.c_void_p(1)
    assert lib.sfsim_atmo_cond_surrogate_create(1, ctypes.byref(q)) == -4
    assert not q.value
    assert lib.sfsim_atmo_plan_build(None, None, None, None, None, None) == -6
    assert lib.sfsim_atmo_plan_destroy(None) == 0
    assert lib.sfsim_atmo_cond_surrogate_destroy(None) == 0


@pytest.mark.gpu
def test_native_caller_matches_python(tmp_path):
    """tests/abi_build.c, compiled against include/sfsim_atmo.h and linked with
    the library the way a native host would, builds the small FP32 tables;
    they equal the tables built through the Python binding bit for bit."""
    import shutil
    import subprocess

    from sfsim_gb300 import atmosphere_lut as A
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lib_dir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "abi_build")
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_build.c"), "-L", lib_dir, "-lsfsim_atmo",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    out = str(tmp_path / "tables.bin")
    r = subprocess.run([exe, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    native = np.fromfile(out, dtype=np.float32)
    ref = A.build(C.small_fp64(precision=C.FP32))
    py = np.concatenate([ref[k].ravel() for k in ("transmittance", "surface_radiance", "ray_scatter",
                                                  "mie_strength")])
    assert native.shape == py.shape
    assert np.array_equal(native, py)

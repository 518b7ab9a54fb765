"""The .scatter reader and validator on CPU with synthetic files."""
import numpy as np
import pytest

from sfsim_gb300 import config as C
from sfsim_gb300 import scatter_io as io


def _write(tmp_path, cfg, seed=0, corrupt=None):
    shapes = io.expected_shapes(cfg)
    rng = np.random.default_rng(seed)
    tables = {}
    for key, name in io.FILES.items():
        a = rng.uniform(0, 1, shapes[key]).astype("<f4")
        if corrupt == key:
            a.flat[5] = np.nan
            a.flat[7] = -1.0
        a.tofile(tmp_path / name)
        tables[key] = a
    return tables


def test_round_trip_and_validation(tmp_path):
    cfg = C.small_fp64()
    written = _write(tmp_path, cfg)
    got = io.load_atmosphere_luts(str(tmp_path), cfg)
    for key in written:
        assert np.array_equal(got[key], written[key])
    assert io.validate_tables(got) == {}


def test_reports_bad_values(tmp_path):
    cfg = C.small_fp64()
    _write(tmp_path, cfg, corrupt="ray_scatter")
    probs = io.validate_tables(io.load_atmosphere_luts(str(tmp_path), cfg))
    assert probs == {"ray_scatter": {"non_finite": 1, "negative": 1}}


def test_size_mismatch_raises(tmp_path):
    cfg = C.small_fp64()
    _write(tmp_path, cfg)
    (tmp_path / "mie-strength.scatter").write_bytes(b"\0" * 12)
    with pytest.raises(io.ScatterFileError):
        io.load_atmosphere_luts(str(tmp_path), cfg)


def test_runtime_shapes_are_the_reference_production_shapes():
    """atmosphere.clj:572-579 against atmosphere_lut.clj:47-57."""
    ref = C.reference_production()
    assert io.expected_shapes(None) == io.expected_shapes(ref)


def test_tiled_to_4d_inverts_convert_4d_to_2d():
    s = (3, 5, 2, 4)
    four = np.arange(np.prod(s) * 3, dtype=np.float32).reshape(s + (3,))
    tiled = four.transpose(0, 2, 1, 3, 4).reshape(s[0] * s[2], s[1] * s[3], 3)
    assert np.array_equal(io.tiled_to_4d(tiled, s), four)

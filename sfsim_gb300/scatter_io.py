"""Reading and validating `.scatter` lookup-table files.

`load_atmosphere_luts` mirrors make-atmosphere-luts (src/clj/sfsim/atmosphere.clj:
587-619): it reads the four files that generate-atmosphere-luts writes
(atmosphere_lut.clj:102-105) with slurp-floats semantics (raw little-endian
float32, util.clj), checks their sizes against the table shapes the runtime
expects (atmosphere.clj:572-579, or a configuration's shapes), and returns the
tables as arrays in the layout the runtime uploads:
  transmittance     [height][elevation][3]         2-D texture (width elevation)
  surface_radiance  [height][sun elevation][3]     2-D texture
  ray_scatter, mie_strength  4-D texture stored as 2-D tiles
                    [height * sun elevation][elevation * heading][3]
`validate_tables` reports non-finite and negative values and transmittance
outside [0, 1].
"""
from __future__ import annotations

import os

import numpy as np

from .config import AtmoConfig

FILES = {"transmittance": "transmittance.scatter", "surface_radiance": "surface-radiance.scatter",
         "ray_scatter": "ray-scatter.scatter", "mie_strength": "mie-strength.scatter"}

# the shapes the reference runtime expects, atmosphere.clj:572-579
RUNTIME_SHAPES = {"transmittance": (64, 255), "surface_radiance": (16, 63), "ray_scatter": (32, 127, 32, 8)}


class ScatterFileError(ValueError):
    pass


def slurp_floats(path: str) -> np.ndarray:
    """Raw little-endian float32 values of a file (util.clj slurp-floats)."""
    size = os.path.getsize(path)
    if size % 4:
        raise ScatterFileError(f"{path}: {size} bytes is not a whole number of float32 values")
    return np.fromfile(path, dtype="<f4")


def expected_shapes(cfg: AtmoConfig | None = None) -> dict:
    if cfg is None:
        t, e, s = RUNTIME_SHAPES["transmittance"], RUNTIME_SHAPES["surface_radiance"], RUNTIME_SHAPES["ray_scatter"]
    else:
        t, e, s = cfg.shapes()
    tiled = (s[0] * s[2], s[1] * s[3], 3)
    return {"transmittance": tuple(t) + (3,), "surface_radiance": tuple(e) + (3,), "ray_scatter": tiled,
            "mie_strength": tiled, "_4d": tuple(s)}


def load_atmosphere_luts(directory: str = "data/atmosphere", cfg: AtmoConfig | None = None) -> dict:
    """Reads and shapes the four tables; raises ScatterFileError on a size mismatch."""
    shapes = expected_shapes(cfg)
    out = {}
    for key, name in FILES.items():
        path = os.path.join(directory, name)
        data = slurp_floats(path)
        want = int(np.prod(shapes[key]))
        if data.size != want:
            raise ScatterFileError(f"{path}: {data.size} floats, expected {want} for shape {shapes[key]}")
        out[key] = data.reshape(shapes[key])
    return out


def tiled_to_4d(tiled: np.ndarray, shape4) -> np.ndarray:
    """Inverse of convert-4d-to-2d (image.clj:299-312): [h*se][e*a][3] -> [h][e][se][a][3]."""
    n0, n1, n2, n3 = shape4
    return tiled.reshape(n0, n2, n1, n3, 3).transpose(0, 2, 1, 3, 4)


def validate_tables(tables: dict) -> dict:
    """Counts of problems per table; an empty dict means every check passed."""
    problems = {}
    for key, arr in tables.items():
        if key.startswith("_"):
            continue
        p = {}
        nonfinite = int((~np.isfinite(arr)).sum())
        negative = int((arr < 0).sum())
        if nonfinite:
            p["non_finite"] = nonfinite
        if negative:
            p["negative"] = negative
        if key == "transmittance":
            above = int((arr > 1.0 + 1e-6).sum())
            if above:
                p["above_one"] = above
        if p:
            problems[key] = p
    return problems

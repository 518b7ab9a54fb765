"""Byte layout of sfsim_atmo_config across the C ABI, without a JVM.

tests/abi_layout.c is compiled against include/sfsim_atmo.h and prints every
field's offset and size.  Three layouts must equal it:
  * the coffi `config-struct` / `component-struct` binding of the
    integration guide at the repository root (the binding a sfsim
    maintainer would add next to src/clj/sfsim/jolt.clj:35-55), laid out by
    C's alignment rules with its explicit padding members;
  * that guide's offset table;
  * the Python ctypes mirror, sfsim_gb300.config.AtmoConfig.
"""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from sfsim_gb300 import config as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INTEGRATION = os.path.join(ROOT, "INTEGRATION.md")


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("abi") / "abi_layout")
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_layout.c"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    fields, sizes = [], {}
    for line in out:
        parts = line.split()
        if len(parts) == 3:
            fields.append((parts[0], int(parts[1]), int(parts[2])))
        elif len(parts) == 2:
            sizes[parts[0]] = int(parts[1])
    return fields, sizes


# coffi member types -> (size, alignment); arrays and padding handled below
_SCALARS = {"::mem/double": (8, 8), "::mem/int": (4, 4), "::mem/float": (4, 4), "::mem/long": (8, 8)}
_MEMBER = re.compile(r"\[:([\w-]+)\s+(::mem/\w+|\[::mem/array\s+(::mem/\w+)\s+(\d+)\]|\[::mem/padding\s+(\d+)\]|"
                     r"[\w-]+-struct)\]")


def _struct_members(text, name):
    m = re.search(r"\(def " + re.escape(name) + r"\s+\[::mem/struct\s+\[(.*?)\]\]\)", text, re.S)
    assert m, f"{name} not found in the integration guide"
    return _MEMBER.findall(m.group(1))


def _layout(text, name, base=0, prefix=""):
    """Flattened (path, offset, size) of a coffi struct under C's rules
    (each member at a multiple of its alignment, the size a multiple of the
    largest alignment), plus the struct's size and alignment."""
    fields, off, align = [], 0, 1
    for member, typ, elem, count, pad in _struct_members(text, name):
        path = prefix + member.replace("-", "_")
        if pad:
            off += int(pad)
            continue
        if typ.endswith("-struct"):
            sub, size, a = _layout(text, typ, 0, path + ".")
            off = (off + a - 1) // a * a
            fields += [(p, base + off + o, s) for p, o, s in sub]
        elif elem:
            es, a = _SCALARS[elem]
            size = es * int(count)
            off = (off + a - 1) // a * a
            fields.append((path, base + off, size))
        else:
            size, a = _SCALARS[typ]
            off = (off + a - 1) // a * a
            fields.append((path, base + off, size))
        off += size
        align = max(align, a)
    return fields, (off + align - 1) // align * align, align


def test_coffi_binding_matches_header(c_layout):
    fields, sizes = c_layout
    text = open(INTEGRATION).read()
    coffi, size, _ = _layout(text, "config-struct")
    assert coffi == fields
    assert size == sizes["sizeof"] == 216
    # without C alignment (a packed layout) the explicit tail padding must
    # still give C's size, so arrays of configs keep C's stride
    packed = sum(int(p) if p else 0 for *_, p in _struct_members(text, "config-struct"))
    assert fields[-1][1] + fields[-1][2] + packed == sizes["sizeof"]


def test_offset_table_matches_header(c_layout):
    fields, sizes = c_layout
    rows = re.findall(r"^\| `([\w.]+)` \| (\d+) \| (\d+) \|$", open(INTEGRATION).read(), re.M)
    assert [(n, int(o), int(s)) for n, o, s in rows] == fields
    m = re.search(r"^\| `sizeof\(sfsim_atmo_config\)` \| \| (\d+) \|$", open(INTEGRATION).read(), re.M)
    assert m and int(m.group(1)) == sizes["sizeof"]


def test_ctypes_mirror_matches_header(c_layout):
    fields, sizes = c_layout
    assert ctypes.sizeof(C.AtmoConfig) == sizes["sizeof"]
    assert ctypes.sizeof(C.Component) == sizes["component_sizeof"]
    for path, off, size in fields:
        if "." in path:
            outer, inner = path.split(".")
            o = getattr(C.AtmoConfig, outer).offset + getattr(C.Component, inner).offset
            s = getattr(C.Component, inner).size
        else:
            o, s = getattr(C.AtmoConfig, path).offset, getattr(C.AtmoConfig, path).size
        assert (o, s) == (off, size), path

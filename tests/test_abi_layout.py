"""The Python mirror's ctypes structures against the C ABI of include/wedg.h, on the CPU.

A field whose offset or size differs between include/wedg.h and edg_westervelt_gb300/_lib.py
would make every call that passes the structure read the wrong bytes without an error. A small C
program compiled with gcc against the header prints sizeof and offsetof of every field of every
structure the Python side builds; they must equal ctypes' figures field by field.
"""
import ctypes
import os
import subprocess

import pytest

from edg_westervelt_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {"wedg_config": L.Config, "wedg_pre": L.Pre, "wedg_stats": L.Stats, "wedg_face_values": L.FaceValues,
           "wedg_cell_table": L.CellTable, "wedg_points": L.Points, "wedg_batch_shape": L.BatchShape,
           "wedg_source_run": L.SourceRun, "wedg_norm_args": L.NormArgs}


def _c_layout(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "wedg.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'  printf("{cname} . %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        layout[(cname, field)] = int(value)
    return layout


def test_ctypes_structures_match_the_header(tmp_path):
    try:
        layout = _c_layout(tmp_path)
    except (OSError, subprocess.CalledProcessError) as e:   # no gcc, or the header does not compile as C
        pytest.fail(f"the layout probe did not build or run: {e}")
    for cname, py in STRUCTS.items():
        assert ctypes.sizeof(py) == layout[(cname, ".")], cname
        for field, _ in py._fields_:
            assert getattr(py, field).offset == layout[(cname, field)], (cname, field)


def _prototypes():
    """name -> list of parameter types of every function declared in include/wedg.h."""
    import re
    src = open(os.path.join(ROOT, "include", "wedg.h")).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    protos = {}
    for m in re.finditer(r"\b(wedg_[a-z0-9_]+)\s*\(([^;{}()]*)\)\s*;", src):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        protos[m.group(1)] = params
    return protos


def _kind_c(param):
    """The ABI class of a C parameter declaration: pointer, double, int32, int64 or size_t."""
    import re
    t = re.sub(r"\[[^\]]*\]", "*", param)          # an array parameter is a pointer
    if "*" in t:
        return "pointer"
    t = re.sub(r"\bconst\b", "", t).split()
    base = " ".join(t[:-1]) if len(t) > 1 else t[0]
    return {"double": "double", "int": "int32", "int32_t": "int32", "int64_t": "int64", "size_t": "size_t"}[base]


def _kind_py(t):
    if t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(t, ctypes._Pointer)):
        return "pointer"
    return {ctypes.c_double: "double", ctypes.c_int: "int32", ctypes.c_int32: "int32", ctypes.c_int64: "int64",
            ctypes.c_size_t: "size_t"}[t]


def test_ctypes_argument_lists_match_the_prototypes(wedg_lib):
    """Every function the Python side declares argtypes for takes, parameter by parameter, the
    pointer / double / 32-bit / 64-bit / size_t arguments of its prototype in include/wedg.h."""
    protos = _prototypes()
    assert sorted(protos) == L.exported_symbols()          # every declared function was parsed
    undeclared = []
    for name, params in protos.items():
        argtypes = getattr(wedg_lib, name).argtypes
        if argtypes is None:
            undeclared.append(name)
            continue
        assert [_kind_py(t) for t in argtypes] == [_kind_c(p) for p in params], name
    assert undeclared == ["wedg_version"]                  # it takes no arguments

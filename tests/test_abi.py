"""The C ABI library loads without a GPU and exports every function that
include/xtg.h declares; the ctypes structs have the C layout."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

import xtensor_gb300 as xg
from xtensor_gb300 import _ffi

ROOT = Path(__file__).resolve().parent.parent


def declared_functions() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\**\s+\**(xtg_\w+)\s*\(", text, re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_library_loads_and_exports_every_declared_symbol():
    L = xg.lib()
    names = declared_functions()
    assert len(names) >= 35, names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"declared in include/xtg.h but not exported: {missing}"
    assert b"sm_103a" in L.xtg_version()


def test_status_strings():
    L = xg.lib()
    for code, text in _ffi.STATUS.items():
        assert L.xtg_status_string(code).decode() == text


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "xtg.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(xtg_node), sizeof(xtg_array),"
        " sizeof(xtg_expr), sizeof(xtg_reduce_desc), offsetof(xtg_reduce_desc, initial),"
        " offsetof(xtg_reduce_desc, ddof), offsetof(xtg_expr, leaves), sizeof(xtg_jit_stats)); return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [C.sizeof(_ffi.Node), C.sizeof(_ffi.Array), C.sizeof(_ffi.Expr), C.sizeof(_ffi.ReduceDesc),
            _ffi.ReduceDesc.initial.offset, _ffi.ReduceDesc.ddof.offset, _ffi.Expr.leaves.offset, C.sizeof(_ffi.JitStats)]
    assert got == want


def test_options_roundtrip():
    xg.set_option("assign.unroll", 4)
    v = C.c_int64()
    xg.check(xg.lib().xtg_get_option(b"assign.unroll", C.byref(v)))
    assert v.value == 4
    xg.set_option("assign.unroll", -1)
    assert xg.lib().xtg_get_option(b"assign.unroll", C.byref(v)) == 13


def test_invalid_arguments_fail_without_gpu():
    L = xg.lib()
    assert L.xtg_assign(None, None, None) == 1
    ex = _ffi.Expr()
    ex.n_nodes = 0
    r = C.c_int32()
    sh = (C.c_int64 * 8)()
    assert L.xtg_broadcast_shape(C.byref(ex), C.byref(r), sh) == 1
    assert L.xtg_last_error()

"""The ctypes mirror of the C ABI has the header's struct layouts.

Every structure that bfs_simd_benchmarks_gb300/_native.py declares is
compiled here from include/bfs_gb300.h with the host C compiler; its size and
every field's offset must equal the ctypes ones, so that a field added to one
side only (or in another order) fails here instead of corrupting calls.
CPU only: no library call is made.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# ctypes mirror -> C typedef
STRUCTS = {
    "GraphInfo": "bfs_graph_info",
    "Options": "bfs_options",
    "Stats": "bfs_stats",
    "BatchStats": "bfs_batch_stats",
    "BcStats": "bfs_bc_stats",
    "TuneTrial": "bfs_tune_trial",
    "TuneResult": "bfs_tune_result",
    "ServerOptions": "bfs_server_options",
    "QueryResult": "bfs_query_result",
    "ServerStats": "bfs_server_stats",
    "RmatParams": "bfs_rmat_params",
}


def _c_layouts(tmp_path):
    from bfs_simd_benchmarks_gb300 import _native as N
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "bfs_gb300.h"', "int main(void) {"]
    for py, c in STRUCTS.items():
        cls = getattr(N, py)
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for name, _ in cls._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        py, name, val = line.split()
        got[(py, name)] = int(val)
    return got


def test_ctypes_structs_match_the_header(tmp_path):
    from bfs_simd_benchmarks_gb300 import _native as N
    got = _c_layouts(tmp_path)
    for py in STRUCTS:
        cls = getattr(N, py)
        assert got[(py, "size")] == C.sizeof(cls), f"{py}: C size {got[(py, 'size')]} vs ctypes {C.sizeof(cls)}"
        for name, _ in cls._fields_:
            off = getattr(cls, name).offset
            assert got[(py, name)] == off, f"{py}.{name}: C offset {got[(py, name)]} vs ctypes {off}"


def test_ctypes_signatures_have_the_header_arity():
    """Every function the ctypes mirror declares takes as many arguments as its
    prototype in include/bfs_gb300.h."""
    import re
    from bfs_simd_benchmarks_gb300 import _native as N
    text = open(os.path.join(ROOT, "include", "bfs_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(bfs_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        args = m.group(2).strip()
        protos[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    for name, _, argtypes in N._SIGNATURES:
        assert name in protos, f"{name} has no prototype in the header"
        assert len(argtypes) == protos[name], f"{name}: {len(argtypes)} ctypes arguments, {protos[name]} in the header"

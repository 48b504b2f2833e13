"""Python face of the CPU oracle (bfs_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker that the GPU product is compared
against, and the CPU baseline bench.py times.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline / reference legs import
this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_lib = None


def reference_dir() -> str | None:
    """The reference checkout named by BFS_REFERENCE_DIR, if it holds the sources."""
    d = os.environ.get("BFS_REFERENCE_DIR", "")
    return d if d and os.path.isdir(os.path.join(d, "apps")) else None


def build(with_reference: bool = True) -> None:
    """Compiles liboracle.so and, where the reference sources exist (BFS_REFERENCE_DIR), oracle/_ref."""
    subprocess.run(["make", "-s", "-C", HERE, "lib"], check=True, capture_output=True)
    ref = reference_dir()
    if with_reference and ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True, capture_output=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(with_reference=False)
        L = C.CDLL(LIB)
        sig = {
            "orc_csr_order": [C.c_uint, C.c_uint, _u32p, _u32p, _u32p, _u32p, _u32p],
            "orc_coo_tile_order": [C.c_uint, C.c_uint, _u32p, _u32p, C.c_uint, _u32p, _u32p, _u32p],
            "orc_col_major_order": [C.c_uint, C.c_uint, _u32p, _u32p, _u32p, C.c_uint, C.c_uint, _u32p, _u32p, _u32p],
            "orc_vertex_remap_map": [C.c_uint, _u32p, _u32p, _u32p, _u32p],
            "orc_write_split": [C.c_char_p, C.c_uint, C.c_uint, _u32p, _u32p, _u32p],
            "orc_write_lines": [C.c_char_p, _u32p, C.c_size_t],
            "orc_write_edge_list": [C.c_char_p, C.c_uint, C.c_uint, _u32p, _u32p, _u32p],
            "orc_read_header": [C.c_char_p, _u32p, _u32p],
            "orc_read_split": [C.c_char_p, C.c_uint, _u32p, _u32p, C.c_int],
            "orc_read_lines": [C.c_char_p, _u32p, C.c_size_t],
            "orc_write_path_dump": [C.c_char_p, C.c_uint, _i32p],
            "orc_read_path_dump": [C.c_char_p, C.c_uint, _i32p],
            "orc_tool_csr_tiling": [C.c_char_p, C.c_int],
            "orc_tool_coo_tiling": [C.c_char_p, C.c_uint],
            "orc_tool_column_major": [C.c_char_p, C.c_uint, C.c_uint],
            "orc_tool_vertex_remap": [C.c_char_p],
            "orc_bfs_hybrid": [C.c_uint, C.c_uint, _u32p, _u32p, _u32p, _u32p, _u32p, _u32p, C.c_uint, C.c_uint,
                               C.c_uint, C.c_uint, C.c_int, _i32p, _u32p, C.POINTER(C.c_uint8), C.c_uint, _u32p,
                               C.POINTER(C.c_double)],
            "orc_bfs_levels": [C.c_uint, _u32p, _u32p, _u32p, C.c_uint, _i32p],
            "orc_check_parents": [C.c_uint, _u32p, _u32p, _u32p, C.c_uint, _i32p, _u32p],
            "orc_bc_single": [C.c_uint, _u32p, _u32p, _u32p, C.c_uint, _u32p, C.POINTER(C.c_float), _i32p,
                              C.POINTER(C.c_double)],
            "orc_max_threads": [],
            "orc_gen_rmat": [C.c_uint, C.c_ulonglong, C.c_double, C.c_double, C.c_double, C.c_ulonglong, C.c_uint,
                             _u32p, _u32p],
            "orc_check_levels": [C.c_uint, C.c_ulonglong, _u32p, _u32p, C.c_uint, _i32p],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_ulonglong if name in ("orc_check_parents", "orc_check_levels") else C.c_int
        _lib = L
    return _lib


def _u(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_i32p if a.dtype == np.int32 else _u32p)


def _ok(st: int, what: str) -> None:
    if st != 0:
        raise RuntimeError(f"oracle {what} failed with status {st}")


def side_length(n: int, w: int) -> int:
    return n // w + (1 if n % w else 0)


# ---- in-memory tool orders ------------------------------------------------
def csr_order(n: int, src, dst):
    s, d = _u(src), _u(dst)
    cs, cd, deg = np.empty_like(s), np.empty_like(d), np.empty(n, dtype=np.uint32)
    _ok(lib().orc_csr_order(n, s.size, _p(s), _p(d), _p(cs), _p(cd), _p(deg)), "csr_order")
    return cs, cd, deg


def coo_tile_order(n: int, src, dst, w: int):
    s, d = _u(src), _u(dst)
    side = side_length(n, w)
    ts, td, off = np.empty_like(s), np.empty_like(d), np.empty(side * side, dtype=np.uint32)
    _ok(lib().orc_coo_tile_order(n, s.size, _p(s), _p(d), w, _p(ts), _p(td), _p(off)), "coo_tile_order")
    return ts, td, off


def col_major_order(n: int, src, dst, offsets, w: int, s_len: int):
    s, d, off = _u(src), _u(dst), _u(offsets)
    hs, tl, noff = np.empty_like(s), np.empty_like(d), np.empty_like(off)
    _ok(lib().orc_col_major_order(n, s.size, _p(s), _p(d), _p(off), w, s_len, _p(hs), _p(tl), _p(noff)),
        "col_major_order")
    return hs, tl, noff


def arrays_from_edges(n: int, src, dst, w: int, s_len: int) -> dict:
    """The arrays graph_input would read after csr_tiling -> coo_tiling -> column_major_tile."""
    cs, cd, deg = csr_order(n, src, dst)
    ts, td, off = coo_tile_order(n, cs, cd, w)
    hs, tl, noff = col_major_order(n, ts, td, off, w, s_len)
    row = np.zeros(n, dtype=np.uint32)
    if n > 1:
        row[1:] = np.cumsum(deg[:-1], dtype=np.uint64).astype(np.uint32)
    return {"n": n, "m": int(cs.size), "w": w, "s": s_len, "degrees": deg, "row_start": row,
            "csr_src": cs, "csr_dst": cd, "heads": hs, "tails": tl, "tile_offsets": noff}


def csr_arrays(n: int, src, dst) -> dict:
    """Only the CSR arrays (what bfs_levels, check_parents and bc_single read):
    cheaper than arrays_from_edges on large graphs."""
    cs, cd, deg = csr_order(n, src, dst)
    del cs
    row = np.zeros(n, dtype=np.uint32)
    if n > 1:
        row[1:] = np.cumsum(deg[:-1], dtype=np.uint64).astype(np.uint32)
    return {"n": n, "m": int(cd.size), "degrees": deg, "row_start": row, "csr_dst": cd}


# ---- traversal -------------------------------------------------------------
def bfs_hybrid(arr: dict, source: int, t_ratio: int = 20, threads: int = 0, trace_cap: int = 256):
    """Levels, parents, direction trace and seconds of the restated graph_prepare."""
    n = arr["n"]
    cost = np.empty(n, dtype=np.int32)
    par = np.empty(n, dtype=np.uint32)
    trace = (C.c_uint8 * trace_cap)()
    steps = C.c_uint(0)
    secs = C.c_double(0)
    _ok(lib().orc_bfs_hybrid(n, arr["m"], _p(arr["row_start"]), _p(arr["degrees"]), _p(arr["csr_dst"]),
                             _p(arr["heads"]), _p(arr["tails"]), _p(arr["tile_offsets"]), arr["w"], arr["s"],
                             int(source), t_ratio, threads, _p(cost), _p(par), trace, trace_cap,
                             C.byref(steps), C.byref(secs)), "bfs_hybrid")
    return cost, par, list(trace[: min(steps.value, trace_cap)]), secs.value


def bfs_levels(arr: dict, source: int) -> np.ndarray:
    cost = np.empty(arr["n"], dtype=np.int32)
    _ok(lib().orc_bfs_levels(arr["n"], _p(arr["row_start"]), _p(arr["degrees"]), _p(arr["csr_dst"]),
                             int(source), _p(cost)), "bfs_levels")
    return cost


def check_parents(arr: dict, source: int, cost, parents) -> int:
    c = np.ascontiguousarray(cost, dtype=np.int32)
    p = _u(parents)
    return int(lib().orc_check_parents(arr["n"], _p(arr["row_start"]), _p(arr["degrees"]), _p(arr["csr_dst"]),
                                       int(source), _p(c), _p(p)))


def bc_single(arr: dict, source: int):
    """Path counts (uint32), float dependencies, levels and per-vertex error
    scale of one source: the reference's BC() restated (bfs_oracle.c)."""
    n = arr["n"]
    sigma = np.empty(n, dtype=np.uint32)
    dep = np.empty(n, dtype=np.float32)
    cost = np.empty(n, dtype=np.int32)
    scale = np.empty(n, dtype=np.float64)
    _ok(lib().orc_bc_single(n, _p(arr["row_start"]), _p(arr["degrees"]), _p(arr["csr_dst"]), int(source),
                            _p(sigma), dep.ctypes.data_as(C.POINTER(C.c_float)), _p(cost),
                            scale.ctypes.data_as(C.POINTER(C.c_double))), "bc_single")
    return sigma, dep, cost, scale


def check_levels(n: int, src, dst, source: int, cost) -> int:
    """Violations of the BFS-level certificate (orc_check_levels): 0 when cost
    are exactly the BFS levels from source in the edge list src -> dst."""
    s, d = _u(src), _u(dst)
    c = np.ascontiguousarray(cost, dtype=np.int32)
    return int(lib().orc_check_levels(n, s.size, _p(s), _p(d), int(source), _p(c)))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def gen_rmat(num_vertices: int, num_edges: int, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1, dedup: bool = True, no_self_loops: bool = True, permute: bool = False):
    """The bench's seeded R-MAT edge list generated on the checker's side
    (bfs_oracle.c orc_gen_rmat): the same list as the product's generator,
    without loading the product library."""
    src = np.empty(num_edges, dtype=np.uint32)
    dst = np.empty(num_edges, dtype=np.uint32)
    flags = (1 if no_self_loops else 0) | (2 if dedup else 0) | (4 if permute else 0)
    _ok(lib().orc_gen_rmat(num_vertices, num_edges, a, b, c, seed, flags, _p(src), _p(dst)), "gen_rmat")
    return src, dst


# ---- files -------------------------------------------------------------------
def write_edge_list(path: str, n: int, src, dst, weights=None) -> None:
    s, d = _u(src), _u(dst)
    w = None if weights is None else _u(weights)
    _ok(lib().orc_write_edge_list(path.encode(), n, s.size, _p(s), _p(d), None if w is None else _p(w)),
        "write_edge_list")


def tool_csr_tiling(path: str, weighted: bool = False) -> None:
    _ok(lib().orc_tool_csr_tiling(path.encode(), 1 if weighted else 0), "csr_tiling")


def tool_coo_tiling(base: str, w: int) -> None:
    _ok(lib().orc_tool_coo_tiling(base.encode(), w), "coo_tiling")


def tool_column_major(base: str, w: int, s_len: int) -> None:
    _ok(lib().orc_tool_column_major(base.encode(), w, s_len), "column_major")


def vertex_remap_map(arr: dict) -> np.ndarray:
    """tools/vertex_id_remap's map (BFS from vertex 0), map[old] = new."""
    out = np.empty(arr["n"], dtype=np.uint32)
    _ok(lib().orc_vertex_remap_map(arr["n"], _p(arr["row_start"]), _p(arr["degrees"]), _p(arr["csr_dst"]), _p(out)),
        "vertex_remap_map")
    return out


def tool_vertex_remap(base: str) -> None:
    _ok(lib().orc_tool_vertex_remap(base.encode()), "vertex_remap")


def read_path_dump(directory: str, n: int) -> np.ndarray:
    cost = np.empty(n, dtype=np.int32)
    _ok(lib().orc_read_path_dump(directory.encode(), n, _p(cost)), "read_path_dump")
    return cost


def write_path_dump(directory: str, cost) -> None:
    c = np.ascontiguousarray(cost, dtype=np.int32)
    _ok(lib().orc_write_path_dump(directory.encode(), c.size, _p(c)), "write_path_dump")


def read_colmajor_files(base: str, w: int, s_len: int, weighted: bool = False) -> dict:
    """Restated graph_input (apps/bfs_simd/bfs.cpp:968-1118) on the text files of <base>."""
    L = lib()
    prefix = f"{base}_col-{s_len}-coo-tiled-{w}"
    n, m = C.c_uint(), C.c_uint()
    _ok(L.orc_read_header(f"{prefix}-0".encode(), C.byref(n), C.byref(m)), "read_header")
    n, m = n.value, m.value
    side = side_length(n, w)
    off = np.empty(side * side, dtype=np.uint32)
    _ok(L.orc_read_lines(f"{prefix}-offsets".encode(), _p(off), off.size), "read offsets")
    hs, tl = np.empty(m, dtype=np.uint32), np.empty(m, dtype=np.uint32)
    _ok(L.orc_read_split(prefix.encode(), m, _p(hs), _p(tl), 1 if weighted else 0), "read col-major")
    deg = np.empty(n, dtype=np.uint32)
    _ok(L.orc_read_lines(f"{base}_untiled-nneibor".encode(), _p(deg), n), "read nneibor")
    cs, cd = np.empty(m, dtype=np.uint32), np.empty(m, dtype=np.uint32)
    _ok(L.orc_read_split(f"{base}_untiled".encode(), m, _p(cs), _p(cd), 1 if weighted else 0), "read untiled")
    row = np.zeros(n, dtype=np.uint32)
    if n > 1:
        row[1:] = np.cumsum(deg[:-1], dtype=np.uint64).astype(np.uint32)
    return {"n": n, "m": m, "w": w, "s": s_len, "degrees": deg, "row_start": row, "csr_src": cs,
            "csr_dst": cd, "heads": hs, "tails": tl, "tile_offsets": off}


def reference_binary(name: str) -> str:
    """Path of a reference program compiled into oracle/_ref (present only where it was built)."""
    return os.path.join(REF_DIR, name)

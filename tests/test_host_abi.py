"""Host side of the product on CPU: the C ABI library, its tools, loader and
generator.  No test here launches a kernel."""
from __future__ import annotations

import hashlib
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_case_names, load_case

CASES = golden_case_names()


def _sha(paths):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _fam(prefix):
    return [f"{prefix}-{t}" for t in range(64)]


def header_symbols():
    text = open(os.path.join(ROOT, "include", "bfs_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bfs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(native, s), f"{s} declared in include/bfs_gb300.h but not exported"
    from bfs_simd_benchmarks_gb300 import _native
    assert set(_native.exported_names()) <= set(syms)


def test_status_strings(native):
    assert native.bfs_status_string(0) == b"ok"
    assert b"open" in native.bfs_status_string(1)


@pytest.mark.parametrize("name", CASES)
def test_product_tools_byte_identical_to_reference(native, name, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    files = c["meta"]["files"]
    g = str(tmp_path / "h")
    w, s = c["w"], c["s"]
    B.write_edge_list(g, c["n"], c["src"], c["dst"])
    B.tool_csr_tiling(g)
    assert _sha(_fam(g + "_untiled") + [g + "_untiled-nneibor"]) == files["untiled"]
    B.tool_coo_tiling(g, w, w)
    assert _sha(_fam(f"{g}_coo-tiled-{w}") + [f"{g}_coo-tiled-{w}-offsets", f"{g}_coo-tiled-{w}-nneibor"]) == files["coo"]
    B.tool_column_major(g, w, s, s)
    col = f"{g}_col-{s}-coo-tiled-{w}"
    assert _sha(_fam(col) + [col + "-offsets", col + "-nneibor"]) == files["col"]
    B.tool_vertex_remap(g)
    assert _sha([g + "_reorder"]) == files["reorder"]


def test_product_weighted_csr_tiling(native, golden_summary, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    z = np.load(os.path.join(ROOT, "tests", "golden", "weighted_csr.npz"))
    g = str(tmp_path / "wg")
    oracle.write_edge_list(g, int(z["n"]), z["src"], z["dst"], z["wts"])
    B.tool_csr_tiling(g, weighted=True)
    assert _sha(_fam(g + "_untiled") + [g + "_untiled-nneibor"]) == golden_summary["weighted_csr"]["digest"]


def test_tool_sweeps_write_every_width_and_stripe(native, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    g = str(tmp_path / "g")
    s, d = B.gen_rmat(256, 2000, seed=3)
    B.write_edge_list(g, 256, s, d)
    B.tool_csr_tiling(g)
    B.tool_coo_tiling(g, 16, 64)          # 16, 32, 64 (tools/coo_tiling/page_rank.cpp:399)
    for w in (16, 32, 64):
        assert os.path.exists(f"{g}_coo-tiled-{w}-offsets")
    B.tool_column_major(g, 32, 2, 8)      # 2, 4, 8
    for st in (2, 4, 8):
        assert os.path.exists(f"{g}_col-{st}-coo-tiled-32-offsets")


@pytest.mark.parametrize("name", CASES)
def test_loader_host_only_matches_oracle_arrays(native, oracle, name, tmp_path):
    """bfs_graph_load parses and validates the reference files (no GPU needed)."""
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    g = str(tmp_path / "h")
    w, s = c["w"], c["s"]
    oracle.write_edge_list(g, c["n"], c["src"], c["dst"])
    oracle.tool_csr_tiling(g)
    oracle.tool_coo_tiling(g, w)
    oracle.tool_column_major(g, w, s)
    gr = B.Graph.load(g, w, s, host_only=True)
    info = gr.info()
    assert info["num_vertices"] == c["n"] and info["num_edges"] == len(c["src"])
    assert info["base"] == g and info["used_reorder"] == 0
    np.testing.assert_array_equal(gr.degrees(), np.bincount(c["src"], minlength=c["n"]))
    gr.close()


def test_loader_prefers_plain_then_reorder_names(native, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    s, d = B.gen_rmat(128, 900, seed=5)
    base = str(tmp_path / "out.x")
    reo = base + "_reorder"
    oracle.write_edge_list(reo, 128, s, d)
    oracle.tool_csr_tiling(reo)
    oracle.tool_coo_tiling(reo, 16)
    oracle.tool_column_major(reo, 16, 2)
    gr = B.Graph.load(base, 16, 2, host_only=True)    # only the bfs_simd (_reorder) names exist
    assert gr.info()["used_reorder"] == 1 and gr.info()["base"] == reo
    gr.close()


def _make_files(oracle, g, n=200, m=1500, w=16, s=3, seed=9):
    import bfs_simd_benchmarks_gb300 as B
    src, dst = B.gen_rmat(n, m, seed=seed)
    oracle.write_edge_list(g, n, src, dst)
    oracle.tool_csr_tiling(g)
    oracle.tool_coo_tiling(g, w)
    oracle.tool_column_major(g, w, s)
    return f"{g}_col-{s}-coo-tiled-{w}"


def test_loader_missing_file_is_eio(native, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    with pytest.raises(B.BfsError) as e:
        B.Graph.load(str(tmp_path / "nothing"), 1024, 16, host_only=True)
    assert e.value.status == 1


def test_loader_truncated_edge_file_is_eformat(native, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    g = str(tmp_path / "g")
    col = _make_files(oracle, g)
    with open(col + "-63") as f:
        lines = f.readlines()
    with open(col + "-63", "w") as f:
        f.writelines(lines[: len(lines) // 2])
    with pytest.raises(B.BfsError) as e:
        B.Graph.load(g, 16, 3, host_only=True)
    assert e.value.status == 2


def test_loader_garbled_and_out_of_range_ids_are_eformat(native, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    g = str(tmp_path / "g")
    col = _make_files(oracle, g)
    with open(col + "-10") as f:
        lines = f.readlines()
    bad = list(lines)
    bad[0] = "7 xyz\n"
    with open(col + "-10", "w") as f:
        f.writelines(bad)
    with pytest.raises(B.BfsError) as e:
        B.Graph.load(g, 16, 3, host_only=True)
    assert e.value.status == 2
    bad[0] = "1 100000\n"   # id > N
    with open(col + "-10", "w") as f:
        f.writelines(bad)
    with pytest.raises(B.BfsError):
        B.Graph.load(g, 16, 3, host_only=True)


def test_loader_non_monotone_offsets_are_eformat(native, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    g = str(tmp_path / "g")
    col = _make_files(oracle, g)
    offs = open(col + "-offsets").read().split()
    offs[5], offs[6] = offs[6], str(int(offs[6]) + 1000)
    with open(col + "-offsets", "w") as f:
        f.write("\n".join(offs) + "\n")
    with pytest.raises(B.BfsError) as e:
        B.Graph.load(g, 16, 3, host_only=True)
    assert e.value.status == 2


def test_loader_edges_out_of_tile_order_are_eformat(native, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    g = str(tmp_path / "g")
    col = _make_files(oracle, g)
    # swap two edge files' contents: the order is then no longer column-major
    a, b = open(col + "-1").read(), open(col + "-40").read()
    open(col + "-1", "w").write(b)
    open(col + "-40", "w").write(a)
    with pytest.raises(B.BfsError) as e:
        B.Graph.load(g, 16, 3, host_only=True)
    assert e.value.status == 2


def test_weighted_files_load_with_w_flag(native, oracle, tmp_path):
    """-w: 3-column files, weights dropped (same graph as the unweighted files)."""
    import bfs_simd_benchmarks_gb300 as B
    n, w, s = 300, 32, 4
    src, dst = B.gen_rmat(n, 2500, seed=11)
    arr = oracle.arrays_from_edges(n, src, dst, w, s)
    wts = (np.arange(len(src)) % 97 + 1).astype(np.uint32)
    base = str(tmp_path / "wg")
    L = oracle.lib()
    import ctypes as C
    def u(a):
        a = np.ascontiguousarray(a, dtype=np.uint32)
        return a, a.ctypes.data_as(C.POINTER(C.c_uint32))
    h, hp = u(arr["heads"]); t, tp = u(arr["tails"]); cs, csp = u(arr["csr_src"]); cd, cdp = u(arr["csr_dst"])
    ww, wp = u(wts)
    assert L.orc_write_split(f"{base}_col-{s}-coo-tiled-{w}".encode(), n, len(src), hp, tp, wp) == 0
    off, offp = u(arr["tile_offsets"])
    assert L.orc_write_lines(f"{base}_col-{s}-coo-tiled-{w}-offsets".encode(), offp, off.size) == 0
    assert L.orc_write_split(f"{base}_untiled".encode(), n, len(src), csp, cdp, wp) == 0
    dg, dgp = u(arr["degrees"])
    assert L.orc_write_lines(f"{base}_untiled-nneibor".encode(), dgp, n) == 0
    with pytest.raises(B.BfsError):
        B.Graph.load(base, w, s, host_only=True)          # without -w the third column is misread
    gr = B.Graph.load(base, w, s, weighted=True, host_only=True)
    np.testing.assert_array_equal(gr.degrees(), arr["degrees"])
    gr.close()


def test_from_arrays_validates(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n, w, s = 500, 32, 3
    src, dst = B.gen_rmat(n, 4000, seed=12)
    arr = oracle.arrays_from_edges(n, src, dst, w, s)
    gr = B.Graph.from_arrays(n, arr["degrees"], arr["csr_dst"], arr["heads"], arr["tails"], arr["tile_offsets"],
                             w, s, host_only=True)
    gr.close()
    bad = arr["heads"].copy()
    bad[[0, -1]] = bad[[-1, 0]]
    with pytest.raises(B.BfsError):
        B.Graph.from_arrays(n, arr["degrees"], arr["csr_dst"], bad, arr["tails"], None, w, s, host_only=True)


def test_rmat_is_deterministic_and_clean(native):
    import bfs_simd_benchmarks_gb300 as B
    s1, d1 = B.gen_rmat(5000, 60000, seed=42, permute=True)
    s2, d2 = B.gen_rmat(5000, 60000, seed=42, permute=True)
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(d1, d2)
    assert len(s1) == 60000 and (s1 != d1).all() and s1.max() < 5000 and d1.max() < 5000
    key = s1.astype(np.uint64) << np.uint64(32) | d1.astype(np.uint64)
    assert np.unique(key).size == key.size
    s3, _ = B.gen_rmat(5000, 60000, seed=43)
    assert not np.array_equal(s1, s3)


def test_level_dump_matches_oracle_bytes(native, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    lev = np.random.default_rng(1).integers(-1, 9, 1000).astype(np.int32)
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir(); b.mkdir()
    B.write_level_dump(str(a), lev)
    oracle.write_path_dump(str(b), lev)
    for t in range(64):
        assert (a / f"path{t}.txt").read_bytes() == (b / f"path{t}.txt").read_bytes()


def test_cli_usage_and_missing_files(native, tmp_path):
    import subprocess
    from bfs_simd_benchmarks_gb300 import build
    r = subprocess.run([build.CLI], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.startswith("Usage: ./bfs <data> <tile_width> <stripe_length>")
    r = subprocess.run([build.CLI, str(tmp_path / "none"), "1024", "16"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open file" in r.stderr


def test_server_option_errors_without_device(native):
    """Invalid server options are refused before any device work; with no GPU
    the server reports BFS_ENODEV instead of failing later."""
    import bfs_simd_benchmarks_gb300 as B
    from conftest import gpu_available
    with pytest.raises(B.BfsError) as ei:
        B.Server(max_batch=0)
    assert ei.value.status == 4
    with pytest.raises(B.BfsError) as ei:
        B.Server(num_slots=17)
    assert ei.value.status == 4
    with pytest.raises(B.BfsError) as ei:
        B.Server(budget_bytes=1 << 20, slot_bytes=1 << 20, num_slots=2)
    assert ei.value.status == 5
    if not gpu_available():
        with pytest.raises(B.BfsError) as ei:
            B.Server()
        assert ei.value.status == 9


def test_autotune_argument_errors(native):
    import bfs_simd_benchmarks_gb300 as B
    src, dst = np.array([0, 1], np.uint32), np.array([1, 2], np.uint32)
    with pytest.raises(B.BfsError) as ei:
        B.autotune(3, src, dst, [5])                 # source out of range
    assert ei.value.status == 4
    with pytest.raises(B.BfsError) as ei:
        B.autotune(3, src, dst, [0], single=False)   # nothing to tune
    assert ei.value.status == 4


def test_binary_load_errors(native, tmp_path):
    """bfs_graph_load_binary refuses missing, foreign and empty files before any device work."""
    import bfs_simd_benchmarks_gb300 as B
    with pytest.raises(B.BfsError) as ei:
        B.Graph.load_binary(str(tmp_path / "missing.bin"))
    assert ei.value.status == 1
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"not a graph file at all" * 8)
    with pytest.raises(B.BfsError) as ei:
        B.Graph.load_binary(str(bad))
    assert ei.value.status == 2
    (tmp_path / "empty.bin").write_bytes(b"")
    with pytest.raises(B.BfsError) as ei:
        B.Graph.load_binary(str(tmp_path / "empty.bin"), host_only=True)
    assert ei.value.status == 2


def test_tile_size_range_matches_reference_tool(native):
    """bfs_tile_size_range against the reference's tile-size-computer outputs
    (tests/golden/tile_size.json, made by its own binary)."""
    import json
    import bfs_simd_benchmarks_gb300 as B
    with open(os.path.join(ROOT, "tests", "golden", "tile_size.json")) as f:
        cases = json.load(f)
    assert len(cases) >= 10
    for c in cases:
        assert B.tile_size_range(c["vertices"], c["edges"]) == (c["min_tile_size"], c["max_tile_size"]), c
    with pytest.raises(B.BfsError):
        B.tile_size_range(10, 3)   # too few edges for any width

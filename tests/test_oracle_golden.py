"""The oracle (oracle/bfs_oracle.c) pinned against the reference's own outputs.

The golden fixtures were produced by running the reference's tools and
apps/bfs_simd (-DONEDEBUG level dump) on these inputs (tests/golden/make_golden.py).
"""
from __future__ import annotations

import hashlib
import os

import numpy as np
import pytest

from conftest import golden_case_names, load_case

CASES = golden_case_names()


def _sha(paths):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _fam(prefix):
    return [f"{prefix}-{t}" for t in range(64)]


@pytest.mark.parametrize("name", CASES)
def test_oracle_hybrid_levels_match_reference(oracle, name):
    c = load_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    for i, src in enumerate(c["sources"]):
        cost, par, trace, _ = oracle.bfs_hybrid(arr, int(src))
        np.testing.assert_array_equal(cost, c["levels"][i], err_msg=f"{name} source {src}")
        assert oracle.check_parents(arr, int(src), cost, par) == 0
        np.testing.assert_array_equal(oracle.bfs_levels(arr, int(src)), cost)
        assert trace[0] == 0  # the first step is always top-down (bfs.cpp:807)


@pytest.mark.parametrize("name", CASES)
def test_oracle_tools_byte_identical_to_reference(oracle, name, tmp_path):
    c = load_case(name)
    files = c["meta"]["files"]
    g = str(tmp_path / "h")
    w, s = c["w"], c["s"]
    oracle.write_edge_list(g, c["n"], c["src"], c["dst"])
    oracle.tool_csr_tiling(g)
    assert _sha(_fam(g + "_untiled") + [g + "_untiled-nneibor"]) == files["untiled"]
    oracle.tool_coo_tiling(g, w)
    assert _sha(_fam(f"{g}_coo-tiled-{w}") + [f"{g}_coo-tiled-{w}-offsets", f"{g}_coo-tiled-{w}-nneibor"]) == files["coo"]
    oracle.tool_column_major(g, w, s)
    col = f"{g}_col-{s}-coo-tiled-{w}"
    assert _sha(_fam(col) + [col + "-offsets", col + "-nneibor"]) == files["col"]
    oracle.tool_vertex_remap(g)
    assert _sha([g + "_reorder"]) == files["reorder"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_reader_roundtrip(oracle, name, tmp_path):
    """graph_input restated on the files equals the in-memory tool orders."""
    c = load_case(name)
    g = str(tmp_path / "h")
    w, s = c["w"], c["s"]
    oracle.write_edge_list(g, c["n"], c["src"], c["dst"])
    oracle.tool_csr_tiling(g)
    oracle.tool_coo_tiling(g, w)
    oracle.tool_column_major(g, w, s)
    arr_f = oracle.read_colmajor_files(g, w, s)
    arr_m = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], w, s)
    for k in ("degrees", "csr_dst", "heads", "tails", "tile_offsets", "row_start"):
        np.testing.assert_array_equal(arr_f[k], arr_m[k], err_msg=k)


def test_oracle_weighted_csr_tiling_matches_reference(oracle, golden_summary, tmp_path):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "weighted_csr.npz"))
    g = str(tmp_path / "wg")
    oracle.write_edge_list(g, int(z["n"]), z["src"], z["dst"], z["wts"])
    oracle.tool_csr_tiling(g, weighted=True)
    assert _sha(_fam(g + "_untiled") + [g + "_untiled-nneibor"]) == golden_summary["weighted_csr"]["digest"]


def test_oracle_path_dump_roundtrip(oracle, tmp_path):
    cost = np.array([0, 1, -1, 2] * 40 + [3], dtype=np.int32)
    oracle.write_path_dump(str(tmp_path), cost)
    np.testing.assert_array_equal(oracle.read_path_dump(str(tmp_path), cost.size), cost)
    with open(tmp_path / "path0.txt") as f:
        assert f.readline() == "0) cost:0\n"


def test_oracle_switch_rule_goes_dense_on_big_frontier(oracle):
    c = load_case("rmat16_w1024_s16")
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    _, _, trace, _ = oracle.bfs_hybrid(arr, int(c["sources"][0]))
    assert 1 in trace, "an R-MAT scale-16 traversal must take at least one bottom-up step"
    _, _, trace_td, _ = oracle.bfs_hybrid(arr, int(c["sources"][0]), t_ratio=1)
    # frontier + out_degree > E never holds: every step is top-down
    assert set(trace_td) == {0}


@pytest.mark.parametrize("n,m,permute,dedup,loops", [(1 << 10, 16 << 10, False, True, False),
                                                     (3000, 40000, True, True, False),
                                                     (1 << 12, 1 << 16, True, False, True),
                                                     (5, 20, False, True, False)])
def test_oracle_generator_equals_product_generator(native, oracle, n, m, permute, dedup, loops):
    """The checker's R-MAT generator (used where the product library must not
    be loaded) gives the product generator's edge list, element for element."""
    import bfs_simd_benchmarks_gb300 as B
    a = oracle.gen_rmat(n, m, seed=77, permute=permute, dedup=dedup, no_self_loops=not loops)
    b = B.gen_rmat(n, m, seed=77, permute=permute, dedup=dedup, no_self_loops=not loops)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_level_certificate_accepts_bfs_levels_and_rejects_others(oracle):
    """orc_check_levels (the full-size check of the bench's large graph)
    against the oracle's BFS on R-MAT graphs, and on planted mistakes."""
    import bfs_simd_benchmarks_gb300 as B
    rng = np.random.default_rng(3)
    for n, m, perm in ((1 << 12, 1 << 16, False), (3000, 30000, True)):
        src, dst = oracle.gen_rmat(n, m, seed=31, permute=perm)
        arr = oracle.csr_arrays(n, src, dst)
        for s in B.pick_sources(arr["degrees"], 3, seed=8):
            lev = oracle.bfs_levels(arr, int(s))
            assert oracle.check_levels(n, src, dst, int(s), lev) == 0
            reached = np.flatnonzero(lev > 0)
            for mutate in range(4):
                bad = lev.copy()
                v = int(rng.choice(reached))
                if mutate == 0:
                    bad[v] += 1            # too deep
                elif mutate == 1:
                    bad[v] = max(1, bad[v] - 1) if bad[v] > 1 else 2
                elif mutate == 2:
                    bad[v] = -1            # dropped a reached vertex
                else:
                    bad[int(s)] = 1        # wrong source
                assert oracle.check_levels(n, src, dst, int(s), bad) > 0

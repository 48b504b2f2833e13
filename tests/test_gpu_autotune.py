"""The autotuner: options and tile shapes chosen by measurement leave the
levels unchanged, the tuned options are applied to the graph, and a second
bfs_autotune on the same graph is answered from the cache file."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_options_keeps_levels(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 14
    src, dst = B.gen_rmat(n, 16 * n, seed=55, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, 1024, 16)
    srcs = B.pick_sources(arr["degrees"], 40, seed=5)
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        r = g.tune(srcs, single=True, batch=True)
        assert r["single_gteps"] > 0 and r["batch_gteps"] > 0
        assert r["single_gteps"] >= r["default_single_gteps"] * 0.99 or r["num_trials"] > 1
        assert r["num_trials"] >= 10 and {t["kind"] for t in r["trials"]} == {1, 2}
        opts = g.options()
        for k in ("to_dense_ratio", "to_sparse_ratio", "bottom_up", "batch_push_div"):
            assert opts[k] == r["options"][k]
        for s in srcs[:6]:
            lev, par, _ = g.run(int(s))
            np.testing.assert_array_equal(lev, oracle.bfs_levels(arr, int(s)))
            assert oracle.check_parents(arr, int(s), lev, par) == 0
        lev, st = g.run_batch(srcs)
        got = lev.cpu().numpy()
        for i, s in enumerate(srcs[:6]):
            ref = oracle.bfs_levels(arr, int(s))
            np.testing.assert_array_equal(got[i], np.where(ref < 0, 255, ref).astype(np.uint8))


def test_autotune_shapes_and_cache(native, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 13
    src, dst = B.gen_rmat(n, 16 * n, seed=66)
    arr = oracle.arrays_from_edges(n, src, dst, 512, 8)
    srcs = B.pick_sources(arr["degrees"], 8, seed=1)
    cache = str(tmp_path / "tune.txt")
    r1 = B.autotune(n, src, dst, srcs, tile_widths=(512, 2048), stripe_lengths=(8, 32), cache_path=cache)
    assert r1["from_cache"] == 0 and r1["tile_width"] in (512, 2048) and r1["stripe_length"] in (8, 32)
    shapes = {(t["tile_width"], t["stripe_length"]) for t in r1["trials"]}
    assert shapes == {(512, 8), (512, 32), (2048, 8), (2048, 32)}
    r2 = B.autotune(n, src, dst, srcs, tile_widths=(512, 2048), stripe_lengths=(8, 32), cache_path=cache)
    assert r2["from_cache"] == 1
    assert (r2["tile_width"], r2["stripe_length"]) == (r1["tile_width"], r1["stripe_length"])
    assert r2["options"] == r1["options"]
    # the tuned shape and options give the reference's levels
    with B.Graph.from_edges(n, src, dst, r1["tile_width"], r1["stripe_length"]) as g:
        g.set_options(**{k: v for k, v in r1["options"].items()})
        for s in srcs:
            lev, _, _ = g.run(int(s))
            np.testing.assert_array_equal(lev, oracle.bfs_levels(arr, int(s)))


def test_autotune_default_widths_from_tile_size_range(native, oracle):
    """With no tile widths, bfs_autotune searches the powers of two of the
    tile-size computer's range (capped at what the packing holds)."""
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 13
    src, dst = B.gen_rmat(n, 16 * n, seed=67)
    srcs = B.pick_sources(np.bincount(src, minlength=n), 4, seed=2)
    lo, hi = B.tile_size_range(n, src.size)
    r = B.autotune(n, src, dst, srcs, tile_widths=None, stripe_lengths=(16,))
    widths = {t["tile_width"] for t in r["trials"]}
    expect = set()
    w = lo
    while w <= max(lo, hi) and w <= 8192:
        expect.add(w)
        w *= 2
    assert widths == expect and r["tile_width"] in expect


@pytest.mark.parametrize("device_build", [False, True])
def test_degree_ordered_layout_keeps_callers_ids(native, oracle, device_build):
    """BFS_LOAD_DEGREE_ORDER (tools/vertex_id_reorder_to_degrees' layout with
    this library's tie-break): sources, levels, parents and out-degrees stay in
    the caller's ids, bit-exact against the oracle on the original graph, in
    both execution modes; the batched, betweenness and save paths refuse it."""
    import bfs_simd_benchmarks_gb300 as B
    n = 20000
    src, dst = B.gen_rmat(n, 12 * n, seed=515, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, 256, 8)
    with B.Graph.from_edges(n, src, dst, 256, 8, device_build=device_build, degree_order=True) as g:
        np.testing.assert_array_equal(g.degrees(), arr["degrees"])
        for mode in ("persistent", "stepwise"):
            g.set_options(mode=mode)
            for s in B.pick_sources(arr["degrees"], 4, seed=3):
                lev, par, st = g.run(int(s))
                np.testing.assert_array_equal(lev, oracle.bfs_levels(arr, int(s)))
                assert oracle.check_parents(arr, int(s), lev, par) == 0
        for call in (lambda: g.run_batch([0, 1, 2, 3, 4, 5]), lambda: g.bc(0)):
            with pytest.raises(B.BfsError) as e:
                call()
            assert e.value.status == 8


def test_autotune_searches_layouts(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 14
    src, dst = B.gen_rmat(n, 16 * n, seed=516, permute=True)
    srcs = B.pick_sources(np.bincount(src, minlength=n), 4, seed=1)
    r = B.autotune(n, src, dst, srcs, tile_widths=(512,), stripe_lengths=(8,), device_build=True, layouts=True)
    assert {t["load_flags"] for t in r["trials"]} == {0, B._native.BFS_LOAD_DEGREE_ORDER}
    assert r["load_flags"] in (0, B._native.BFS_LOAD_DEGREE_ORDER)

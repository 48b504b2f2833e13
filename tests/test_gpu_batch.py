"""Parity of the batched traversal (bfs_run_batch, through the C ABI).

Every source's row of the batched uint8 levels must equal that source's
single-source levels (the reference's h_cost, -1 shown as 255): against the
reference's own golden levels where the fixtures hold them, against the
oracle elsewhere.  The cases cover a partial last 64-source word, repeated
sources, 4096 sources (64 words per vertex), push levels with vertices of
degree above the grid-spread threshold, pull-only traversals, traversals
deeper than the level planes (early output passes) and the 254-level limit.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_case_names, load_case

pytestmark = pytest.mark.gpu


def _expect(oracle, arr, sources):
    out = np.empty((len(sources), arr["n"]), dtype=np.uint8)
    for i, s in enumerate(sources):
        lev = oracle.bfs_levels(arr, int(s))
        out[i] = np.where(lev < 0, 255, lev).astype(np.uint8)
    return out


def _check(oracle, arr, g, sources, expect=None):
    lev, st = g.run_batch(sources)
    got = lev.cpu().numpy()
    if expect is None:
        expect = _expect(oracle, arr, sources)
    for i, s in enumerate(sources):
        np.testing.assert_array_equal(got[i], expect[i], err_msg=f"row {i} (source {s})")
    assert st["status"] == 0
    deg = arr["degrees"].astype(np.uint64)
    assert st["edges_traversed"] == int(sum(deg[expect[i] != 255].sum() for i in range(len(sources))))
    assert st["depth"] == int(expect[expect != 255].max()) + 1
    assert st["num_sources"] == len(sources)
    return got, st


@pytest.mark.parametrize("single_max", [0, 4])
@pytest.mark.parametrize("name", [c for c in golden_case_names() if not c.startswith("chain")])
def test_golden_sources_batched(native, oracle, name, single_max):
    """single_max 0: the bit-sliced kernel even for 4 sources; 4: the
    back-to-back single-source path that small batches take."""
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    exp = np.where(c["levels"] < 0, 255, c["levels"]).astype(np.uint8)
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        g.set_options(batch_single_max=single_max)
        _, st = _check(oracle, arr, g, [int(x) for x in c["sources"]], exp)
        assert st["single_source_runs"] == (len(c["sources"]) if len(c["sources"]) <= single_max else 0)


def test_partial_word_and_repeated_sources(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 14
    src, dst = B.gen_rmat(n, 16 * n, seed=141, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, 1024, 16)
    srcs = B.pick_sources(arr["degrees"], 130, seed=3).tolist()
    srcs[7] = srcs[100] = srcs[129]          # the same source in three words
    srcs[64] = int(np.flatnonzero(arr["degrees"] == 0)[0]) if (arr["degrees"] == 0).any() else srcs[64]
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        _check(oracle, arr, g, srcs)
        # a smaller batch next on the same buffers, then a bigger one (reallocation)
        _check(oracle, arr, g, srcs[:1])
        big = B.pick_sources(arr["degrees"], 700, seed=4)
        _check(oracle, arr, g, big)


def test_4096_sources(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 12
    src, dst = B.gen_rmat(n, 16 * n, seed=412, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, 256, 4)
    srcs = B.pick_sources(arr["degrees"], 4096, seed=12)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        _, st = _check(oracle, arr, g, srcs)
        assert st["words_per_vertex"] == 64
        assert st["push_levels"] < st["depth"], "a frontier this large should be pulled"


def test_push_with_high_degree_vertices(native, oracle):
    """Hubs of out-degree above the grid-spread threshold in push levels."""
    import bfs_simd_benchmarks_gb300 as B
    rng = np.random.default_rng(8)
    n = 60000
    s1, d1 = B.gen_rmat(1 << 15, 4 * (1 << 15), seed=88)
    hubs = [0, 1, 2]
    src = [s1, np.repeat(np.array(hubs, np.uint32), 5000)]
    dst = [d1, rng.integers(0, n, 15000).astype(np.uint32)]
    src = np.concatenate(src).astype(np.uint32)
    dst = np.concatenate(dst).astype(np.uint32)
    arr = oracle.arrays_from_edges(n, src, dst, 1024, 16)
    srcs = hubs + B.pick_sources(arr["degrees"], 40, seed=2).tolist()
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        _, st = _check(oracle, arr, g, srcs)
        assert st["push_levels"] >= 1


def test_deeper_than_planes_and_vertex_tails(native, oracle):
    """A long chain with a few branches: 180 levels through 2 and 3 planes
    (many early output passes); N = 1003 so that rows are written bytewise."""
    import bfs_simd_benchmarks_gb300 as B
    n = 1003
    chain = np.arange(180, dtype=np.uint32)
    rng = np.random.default_rng(1)
    br_src = rng.integers(0, 180, 600).astype(np.uint32)
    br_dst = rng.integers(181, n, 600).astype(np.uint32)
    src = np.concatenate([chain, br_src])
    dst = np.concatenate([chain + 1, br_dst])
    arr = oracle.arrays_from_edges(n, src, dst, 64, 3)
    srcs = [0, 5, 90, 179, 180, 500] + list(range(10, 80))
    exp = _expect(oracle, arr, srcs)
    with B.Graph.from_edges(n, src, dst, 64, 3) as g:
        for planes in (2, 3, 0):
            g.set_options(batch_planes=planes)
            _, st = _check(oracle, arr, g, srcs, exp)
            if planes:
                assert st["spills"] > 0 and st["planes"] == planes


def test_aligned_rows_vector_path_and_offset_output(native, oracle):
    """N a multiple of 16 (16-byte row stores) and the same output at an odd address."""
    torch = pytest.importorskip("torch")
    import bfs_simd_benchmarks_gb300 as B
    n = 4096
    src, dst = B.gen_rmat(n, 8 * n, seed=21)
    arr = oracle.arrays_from_edges(n, src, dst, 128, 4)
    srcs = B.pick_sources(arr["degrees"], 200, seed=5)
    exp = _expect(oracle, arr, srcs)
    with B.Graph.from_edges(n, src, dst, 128, 4) as g:
        _check(oracle, arr, g, srcs, exp)
        buf = torch.full((len(srcs) * n + 1,), 7, dtype=torch.uint8, device="cuda")
        st = g.run_batch_device(srcs, buf.data_ptr() + 1, torch.cuda.current_stream().cuda_stream, stats=True)
        got = buf.cpu().numpy()
        assert got[0] == 7 and st["status"] == 0
        np.testing.assert_array_equal(got[1:].reshape(len(srcs), n), exp)


@pytest.mark.parametrize("single_max", [0, 4])
def test_levels_above_254_are_refused(native, oracle, single_max):
    import bfs_simd_benchmarks_gb300 as B
    n = 300
    src = np.arange(299, dtype=np.uint32)
    with B.Graph.from_edges(n, src, src + 1, 32, 2) as g:
        g.set_options(batch_single_max=single_max)
        with pytest.raises(B.BfsError) as ei:
            g.run_batch([0, 1])
        assert ei.value.status == 8  # BFS_EUNSUPPORTED
        # a source whose levels stay within 254 works on the same graph
        lev, st = g.run_batch([100])
        exp = np.full(n, 255, np.uint8)
        exp[100:] = np.arange(200)
        np.testing.assert_array_equal(lev.cpu().numpy()[0], exp)


def test_argument_errors(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    src, dst = B.gen_rmat(1024, 4096, seed=2)
    with B.Graph.from_edges(1024, src, dst, 64, 2) as g:
        with pytest.raises(B.BfsError):
            g.run_batch([1024])                     # out of range
        with pytest.raises(B.BfsError):
            g.run_batch(np.zeros(4097, np.uint32))  # too many sources
        with pytest.raises(B.BfsError):
            g.set_options(batch_planes=1)


def test_many_in_edge_destinations(native, oracle):
    """Destinations with thousands of in-edges: their in-edges are cut into
    chunks that warps across the grid gather and combine."""
    import bfs_simd_benchmarks_gb300 as B
    rng = np.random.default_rng(17)
    n = 20000
    s1, d1 = B.gen_rmat(1 << 14, 8 * (1 << 14), seed=171, permute=True)
    sinks = np.array([19990, 19991, 19992, 5, 77], np.uint32)
    src = [s1, rng.integers(0, n, 5 * 3000).astype(np.uint32), np.repeat(sinks[:3], 40)]
    dst = [d1, np.repeat(sinks, 3000), rng.integers(0, n, 120).astype(np.uint32)]
    src = np.concatenate(src).astype(np.uint32)
    dst = np.concatenate(dst).astype(np.uint32)
    arr = oracle.arrays_from_edges(n, src, dst, 512, 8)
    srcs = B.pick_sources(arr["degrees"], 500, seed=9)
    with B.Graph.from_edges(n, src, dst, 512, 8) as g:
        _, st = _check(oracle, arr, g, srcs)
        assert 0 in st["level_push"], "expected pull levels"


@pytest.mark.parametrize("planes", [2, 0])
@pytest.mark.parametrize("n", [2050, 1028, 1001])
def test_row_alignments_and_merges(native, oracle, n, planes):
    """Rows of N bytes start at every alignment (N = 2 mod 4: 2-byte stores,
    N = 4 mod 16: 4-byte stores, odd N: bytes); with 2 planes the output is
    written in several segments merged by a byte-wise minimum."""
    import bfs_simd_benchmarks_gb300 as B
    rng = np.random.default_rng(n)
    chain = np.arange(40, dtype=np.uint32)
    s1, d1 = B.gen_rmat(n, 6 * n, seed=n + 1)
    src = np.concatenate([chain, s1, rng.integers(0, 40, 200).astype(np.uint32)])
    dst = np.concatenate([chain + 1, d1, rng.integers(41, n, 200).astype(np.uint32)])
    arr = oracle.arrays_from_edges(n, src, dst, 64, 4)
    srcs = [0, 3, 17] + B.pick_sources(arr["degrees"], 67, seed=n).tolist()
    with B.Graph.from_edges(n, src, dst, 64, 4) as g:
        g.set_options(batch_planes=planes)
        _, st = _check(oracle, arr, g, srcs)
        if planes:
            assert st["spills"] > 0


def test_device_sources_and_cuda_graph(native, oracle):
    """bfs_run_batch_device and a captured CUDA graph launched twice with new
    source values in the same device buffer: the rows equal bfs_run_batch's."""
    torch = pytest.importorskip("torch")
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 13
    src, dst = B.gen_rmat(n, 16 * n, seed=913, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, 256, 8)
    s1 = B.pick_sources(arr["degrees"], 150, seed=1)
    s2 = B.pick_sources(arr["degrees"], 150, seed=2)
    with B.Graph.from_edges(n, src, dst, 256, 8) as g:
        d_src = torch.tensor(s1.astype(np.int64), dtype=torch.int32, device="cuda")
        out = torch.empty((150, n), dtype=torch.uint8, device="cuda")
        g.run_batch_sources_device(d_src.data_ptr(), 150, out.data_ptr())
        st = g.last_batch_stats()
        assert st["status"] == 0
        np.testing.assert_array_equal(out.cpu().numpy(), _expect(oracle, arr, s1))
        with g.batch_graph(d_src.data_ptr(), 150, out.data_ptr()) as bg:
            for srcs in (s2, s1):
                d_src.copy_(torch.tensor(srcs.astype(np.int64), dtype=torch.int32))
                out.fill_(7)
                torch.cuda.synchronize()
                bg.launch()
                st = g.last_batch_stats()
                assert st["status"] == 0 and st["num_sources"] == 150
                np.testing.assert_array_equal(out.cpu().numpy(), _expect(oracle, arr, srcs))
        # a source out of range is reported by the device
        d_src[3] = n
        with pytest.raises(B.BfsError) as ei:
            g.run_batch_sources_device(d_src.data_ptr(), 150, out.data_ptr())
            g.last_batch_stats()
        assert ei.value.status == 4


@pytest.mark.timeout(900)
def test_rmat22_4096_sources_against_the_oracle(native, oracle):
    """The batched configuration at full size: R-MAT scale 22 (4,194,304
    vertices, 67,108,864 edges), 4096 seeded sources in one launch (64 words
    per vertex); 12 rows spread over the batch (first and last words
    included) bit-exact against the oracle."""
    torch = pytest.importorskip("torch")
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import workloads
    wl = workloads.get("rmat22")
    src, dst = wl.edges()
    arr = oracle.csr_arrays(wl.n, src, dst)
    with B.Graph.from_edges(wl.n, src, dst, wl.w, wl.s, device_build=True) as g:
        del src, dst
        sources = wl.sources(g.degrees(), 4096)
        out = torch.empty((4096, wl.n), dtype=torch.uint8, device="cuda")
        st = g.run_batch_device(sources, out.data_ptr(), torch.cuda.current_stream().cuda_stream, stats=True)
        assert st["status"] == 0 and st["words_per_vertex"] == 64
        for i in (0, 1, 63, 64, 1000, 2047, 2048, 3000, 4031, 4032, 4094, 4095):
            ref = oracle.bfs_levels(arr, int(sources[i]))
            np.testing.assert_array_equal(out[i].cpu().numpy(), np.where(ref < 0, 255, ref).astype(np.uint8))
        del out
        torch.cuda.empty_cache()


@pytest.mark.parametrize("num_sources", [70, 4096])
def test_output_tile_widths_give_the_same_levels(native, oracle, num_sources):
    """The output pass's two tile widths (64 vertices on 256-thread CTAs, 128 on
    512-thread CTAs; option batch_output_tile, by graph size when 0) write the
    same bytes, also when the traversal outgrows its planes (early output
    passes merged into the final one)."""
    import bfs_simd_benchmarks_gb300 as B
    n = (1 << 14) + 37   # not a multiple of either tile width
    src, dst = B.gen_rmat(n, 16 * n, seed=1717, permute=True)
    arr = oracle.csr_arrays(n, src, dst)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        sources = B.pick_sources(g.degrees(), num_sources, seed=21)
        outs = {}
        for planes in (0, 3):
            for tile in (0, 64, 128):
                g.set_options(batch_output_tile=tile, batch_planes=planes)
                out, st = g.run_batch(sources)
                assert st["status"] == 0
                outs[(planes, tile)] = out.cpu().numpy()
        ref = outs[(0, 64)]
        for key, rows in outs.items():
            assert rows.tobytes() == ref.tobytes(), key
        for i in (0, num_sources // 2, num_sources - 1):
            want = oracle.bfs_levels(arr, int(sources[i]))
            np.testing.assert_array_equal(ref[i], np.where(want < 0, 255, want).astype(np.uint8))
        import bfs_simd_benchmarks_gb300._native as N
        with pytest.raises(N.BfsError):
            g.set_options(batch_output_tile=96)

"""Batched betweenness (bfs_bc_run_batch, bfs_bc_run_batch_device and
bfs_bc_accumulate with bc_batch = 1) through the C ABI against the oracle's
restatement of the reference's BC() (apps/betweennessCentrality_simd/
bc.cpp:1717-2097), one source at a time.

Path counts are unsigned integers and must be bit-exact for every (source,
vertex) pair; dependencies within 1e-4 * (scale + 1) of the oracle (float
sums in another order).  Repeated batched runs must give identical bits.
A batch deeper than its level planes must fall back to the single-source
kernel and still give the oracle's values.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import bc_case_names, bc_close, golden_case_names, load_bc_case, load_case

pytestmark = pytest.mark.gpu


def _check_rows(oracle, arr, sources, dep, sig, st=None):
    for i, s in enumerate(sources):
        osig, odep, ocost, oscale = oracle.bc_single(arr, int(s))
        np.testing.assert_array_equal(sig[i], osig, err_msg=f"path counts from {s} (row {i})")
        ok = bc_close(dep[i], odep, oscale)
        bad = np.flatnonzero(~ok)
        assert ok.all(), f"source {s} (row {i}): {bad[:6]} gpu {dep[i][bad[:6]]} oracle {odep[bad[:6]]}"
        reached = ocost >= 0
        assert (dep[i][~reached] == 0).all() and (sig[i][~reached] == 0).all()
        if st is not None and st["batched_sources"]:
            assert st["source_reached"][i] == int(reached.sum())


@pytest.mark.parametrize("name", bc_case_names())
def test_bc_batch_matches_oracle(native, oracle, name):
    import bfs_simd_benchmarks_gb300 as B
    c = load_bc_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    sources = np.asarray(c["sources"], np.uint32)[:64]
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        dep, sig, st = g.bc_batch(sources)
        assert st["status"] == 0 and st["num_sources"] == sources.size
        _check_rows(oracle, arr, sources, dep, sig, st)
        dep2, sig2, _ = g.bc_batch(sources)
        assert dep2.tobytes() == dep.tobytes() and sig2.tobytes() == sig.tobytes()


@pytest.mark.parametrize("name", golden_case_names())
def test_bc_batch_golden_graphs(native, oracle, name):
    """Every golden graph (duplicate edges, the 300-deep chain: a batch deeper
    than 254 levels runs one source at a time)."""
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    deg = np.bincount(c["src"], minlength=c["n"])
    cand = np.flatnonzero(deg > 0)
    sources = np.unique(np.concatenate([np.asarray(c["sources"], np.int64), cand[:: max(1, cand.size // 40)]]))[:64]
    sources = sources.astype(np.uint32)
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        dep, sig, st = g.bc_batch(sources)
        assert st["batched_sources"] + st["fallback_sources"] == sources.size
        if name.startswith("chain"):
            assert st["fallback_sources"] == sources.size
        _check_rows(oracle, arr, sources, dep, sig, st)


def test_bc_batch_rmat_64_sources_with_hubs(native, oracle):
    """An R-MAT graph whose hubs have more than 256 in- and out-edges (the
    chunked sums of both sweeps), 64 sources, duplicates and a sink among them."""
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 14
    src, dst = B.gen_rmat(n, 16 * n, seed=2024, permute=True)
    arr = oracle.csr_arrays(n, src, dst)
    outd = np.bincount(src, minlength=n)
    ind = np.bincount(dst, minlength=n)
    assert outd.max() > 256 and ind.max() > 256
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        sources = B.pick_sources(g.degrees(), 61, seed=9).astype(np.uint32)
        sink = int(np.flatnonzero(outd == 0)[0])
        sources = np.concatenate([sources, [sources[3], sink, int(np.argmax(outd))]]).astype(np.uint32)
        assert sources.size == 64
        dep, sig, st = g.bc_batch(sources)
        assert st["status"] == 0 and st["batched_sources"] == 64
        assert st["edges_matched_forward"] <= st["edges_forward"]
        assert st["edges_matched_forward"] == st["edges_matched_reverse"]
        # (edge, source) pairs summed = the shortest-path DAG edges of every source
        lev = [oracle.bfs_levels(arr, int(x)) for x in sources]
        dag = sum(int(((lv[src] >= 0) & (lv[dst] == lv[src] + 1)).sum()) for lv in lev)
        assert st["pairs_forward"] == dag and st["pairs_reverse"] == dag
        _check_rows(oracle, arr, sources, dep, sig, st)
        # the duplicate's rows equal the original's
        assert dep[61].tobytes() == dep[3].tobytes() and sig[61].tobytes() == sig[3].tobytes()
        # a batch of one, and a batch that is not a multiple of 32
        for k in (1, 37):
            d1, s1, _ = g.bc_batch(sources[:k])
            _check_rows(oracle, arr, sources[:k], d1, s1)


def test_bc_batch_several_words(native, oracle):
    """150 sources in one call: three words of the traversal (64, 64, 22
    sources), one launch each; every row against the oracle, the statistics
    summed over the launches."""
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 13
    src, dst = B.gen_rmat(n, 16 * n, seed=515, permute=True)
    arr = oracle.csr_arrays(n, src, dst)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        sources = B.pick_sources(g.degrees(), 150, seed=12).astype(np.uint32)
        dep, sig, st = g.bc_batch(sources)
        assert st["status"] == 0 and st["batched_sources"] == 150 and len(st["source_reached"]) == 150
        _check_rows(oracle, arr, sources, dep, sig, st)
        lev = [oracle.bfs_levels(arr, int(x)) for x in sources]
        dag = sum(int(((lv[src] >= 0) & (lv[dst] == lv[src] + 1)).sum()) for lv in lev)
        assert st["pairs_forward"] == dag and st["pairs_reverse"] == dag
        # the first 64 rows equal a batch of those 64 alone
        d64, s64, _ = g.bc_batch(sources[:64])
        assert d64.tobytes() == dep[:64].tobytes() and s64.tobytes() == sig[:64].tobytes()


def test_bc_batch_fallback_when_planes_run_out(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 12
    src, dst = B.gen_rmat(n, 8 * n, seed=77, permute=True)
    arr = oracle.csr_arrays(n, src, dst)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        sources = B.pick_sources(g.degrees(), 20, seed=3).astype(np.uint32)
        d_ok, s_ok, st = g.bc_batch(sources)
        assert st["batched_sources"] == 20 and st["fallback_sources"] == 0
        g.set_options(batch_planes=2)      # every traversal here is deeper than 2 planes
        dep, sig, st = g.bc_batch(sources)
        assert st["fallback_sources"] == 20 and st["batched_sources"] == 0
        _check_rows(oracle, arr, sources, dep, sig)
        assert sig.tobytes() == s_ok.tobytes()


def test_bc_batch_device_matches_host(native):
    import torch
    import bfs_simd_benchmarks_gb300 as B
    c = load_case("rmat12p_w100_s5")
    n = c["n"]
    with B.Graph.from_edges(n, c["src"], c["dst"], c["w"], c["s"]) as g:
        sources = np.asarray(c["sources"], np.uint32)[:8]
        dep, sig, _ = g.bc_batch(sources)
        d_dep = torch.empty((sources.size, n), dtype=torch.float32, device="cuda")
        d_sig = torch.empty((sources.size, n), dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        g.bc_batch_device(sources, d_dep.data_ptr(), d_sig.data_ptr(), stream)
        torch.cuda.synchronize()
        st = g.bc_stats()
        assert st["status"] == 0 and st["batched_sources"] == sources.size
        assert d_dep.cpu().numpy().tobytes() == dep.tobytes()
        assert d_sig.cpu().numpy().view(np.uint32).tobytes() == sig.tobytes()


def test_bc_batch_device_two_words_matches_host(native):
    """bfs_bc_run_batch_device with 100 sources (two words, two launches) into
    device buffers: the same bits as the host entry point."""
    import torch
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 12
    src, dst = B.gen_rmat(n, 8 * n, seed=919, permute=True)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        sources = B.pick_sources(g.degrees(), 100, seed=5).astype(np.uint32)
        dep, sig, _ = g.bc_batch(sources)
        d_dep = torch.empty((sources.size, n), dtype=torch.float32, device="cuda")
        d_sig = torch.empty((sources.size, n), dtype=torch.int32, device="cuda")
        g.bc_batch_device(sources, d_dep.data_ptr(), d_sig.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        st = g.bc_stats()
        assert st["status"] == 0 and st["batched_sources"] == 100 and len(st["source_reached"]) == 100
        assert d_dep.cpu().numpy().tobytes() == dep.tobytes()
        assert d_sig.cpu().numpy().view(np.uint32).tobytes() == sig.tobytes()


def test_bc_accumulate_batched_matches_one_by_one(native, oracle):
    """bfs_bc_accumulate over 300 sources (a batch of 256, four words, then one
    of 44) against the one-source-at-a-time accumulation and the oracle's sum."""
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 12
    src, dst = B.gen_rmat(n, 8 * n, seed=31, permute=True)
    arr = oracle.csr_arrays(n, src, dst)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        sources = B.pick_sources(g.degrees(), 300, seed=4).astype(np.uint32)
        bc1, st1 = g.betweenness(sources)
        assert st1["batched_sources"] == 300 and st1["num_sources"] == 300
        bc1b, _ = g.betweenness(sources)
        assert bc1b.tobytes() == bc1.tobytes()
        g.set_options(bc_batch=0)
        bc0, st0 = g.betweenness(sources)
        assert st0["batched_sources"] == 0 and st0["num_sources"] == 300
        assert st0["edges_reached"] == st1["edges_reached"]
        want = np.zeros(n)
        scale = np.zeros(n)
        for s in sources:
            _, d, _, sc = oracle.bc_single(arr, int(s))
            d = d.astype(np.float64)
            d[s] = 0
            sc = sc.copy()
            sc[s] = 0
            want += d
            scale += sc
        assert bc_close(bc1, want, scale).all()
        assert bc_close(bc0, want, scale).all()


def test_bc_batch_arguments(native):
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import _native as N
    c = load_case("sparse15_w16_s2")
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        with pytest.raises(N.BfsError) as e:
            g.bc_batch(np.arange(257, dtype=np.uint32))
        assert e.value.status == N.BFS_EARG
        with pytest.raises(N.BfsError) as e:
            g.bc_batch(np.array([0, c["n"]], np.uint32))
        assert e.value.status == N.BFS_EARG
        with pytest.raises(ValueError):
            g.set_options(no_such=1)
        with pytest.raises(N.BfsError):
            g.set_options(bc_batch=2)

"""Betweenness dependencies on the GPU (bfs_bc_run / bfs_bc_accumulate through
the C ABI) against the oracle's restatement of the reference's BC()
(apps/betweennessCentrality_simd/bc.cpp:1717-2097) and networkx's Brandes
values (tests/golden/bc_networkx.npz).

Path counts are unsigned integers and must be bit-exact.  Dependencies are
float sums whose order differs from the oracle's: |gpu - oracle| <=
1e-4 * (scale + 1), scale being the magnitude of the float sums behind each
value.  Repeated GPU runs must be bit-identical (fixed summation order).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import bc_case_names, bc_close, golden_case_names, load_bc_case, load_case

pytestmark = pytest.mark.gpu


def _check_source(oracle, arr, g, s):
    dep, sig, st = g.bc(int(s))
    osig, odep, ocost, oscale = oracle.bc_single(arr, int(s))
    np.testing.assert_array_equal(sig, osig, err_msg=f"path counts from {s}")
    ok = bc_close(dep, odep, oscale)
    bad = np.flatnonzero(~ok)
    assert ok.all(), f"source {s}: {bad[:6]} gpu {dep[bad[:6]]} oracle {odep[bad[:6]]}"
    assert st["status"] == 0
    reached = ocost >= 0
    assert st["reached"] == int(reached.sum())
    assert st["depth"] == int(ocost.max())
    assert st["edges_reached"] == int(arr["degrees"].astype(np.uint64)[reached].sum())
    assert (dep[~reached] == 0).all() and (sig[~reached] == 0).all()
    return dep, sig, st


@pytest.mark.parametrize("name", bc_case_names())
def test_bc_matches_oracle_and_networkx(native, oracle, name):
    import bfs_simd_benchmarks_gb300 as B
    c = load_bc_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        for i, s in enumerate(c["sources"]):
            dep, _, _ = _check_source(oracle, arr, g, s)
            _, _, cost, scale = oracle.bc_single(arr, int(s))
            want = c["delta"][i].copy()
            want[s] = float((cost >= 0).sum() - 1)
            ok = bc_close(dep, want, scale)
            assert ok.all(), f"{name} source {s} vs networkx: {np.flatnonzero(~ok)[:6]}"


@pytest.mark.parametrize("name", golden_case_names())
def test_bc_golden_graphs_deterministic(native, oracle, name):
    """Every golden graph (duplicate edges included), a repeat run bit-identical,
    and the byte-level gathers (bc_level_bytes = 1) giving the same bits as the
    8-byte ones (2)."""
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        for s in c["sources"]:
            g.set_options(bc_level_bytes=2)
            dep, sig, _ = _check_source(oracle, arr, g, s)
            dep2, sig2, _ = g.bc(int(s))
            assert dep.tobytes() == dep2.tobytes() and sig.tobytes() == sig2.tobytes()
            g.set_options(bc_level_bytes=1)
            dep3, sig3, _ = g.bc(int(s))
            assert dep.tobytes() == dep3.tobytes() and sig.tobytes() == sig3.tobytes()


def test_bc_hubs_take_the_cta_path(native, oracle):
    """In- and out-degrees above 1024 (a whole CTA reduces those vertices)."""
    import bfs_simd_benchmarks_gb300 as B
    rng = np.random.default_rng(7)
    n = 6000
    src, dst = [], []
    # 0 -> 1..3000 -> 3001 (in-degree 3000) -> 3002..5999 (out-degree 2998)
    for v in range(1, 3001):
        src += [0, v]
        dst += [v, 3001]
    for v in range(3002, n):
        src.append(3001)
        dst.append(v)
    # random cross edges one level down keep path counts uneven
    extra_u = rng.integers(1, 3001, 4000)
    extra_v = rng.integers(3002, n, 4000)
    src = np.concatenate([np.array(src, np.uint32), extra_u.astype(np.uint32)])
    dst = np.concatenate([np.array(dst, np.uint32), extra_v.astype(np.uint32)])
    arr = oracle.arrays_from_edges(n, src, dst, 256, 4)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        for s in (0, 17, 3001):
            _check_source(oracle, arr, g, s)


def test_bc_many_big_vertices_in_one_level(native, oracle):
    """A level with more than 4096 big vertices (one CTA each) followed by a
    level of 1800 big vertices (chunked over the grid)."""
    import bfs_simd_benchmarks_gb300 as B
    rng = np.random.default_rng(11)
    first, pool = 4200, 1800
    n = 1 + first + pool
    src = [np.zeros(first, np.uint32)]
    dst = [np.arange(1, first + 1, dtype=np.uint32)]
    for v in range(1, first + 1):
        t = rng.choice(pool, 1100, replace=False).astype(np.uint32) + first + 1
        src.append(np.full(1100, v, np.uint32))
        dst.append(t)
    src = np.concatenate(src)
    dst = np.concatenate(dst)
    arr = oracle.arrays_from_edges(n, src, dst, 512, 8)
    with B.Graph.from_edges(n, src, dst, 512, 8) as g:
        for mode in (1, 2):
            g.set_options(bc_level_bytes=mode)
            _, _, st = _check_source(oracle, arr, g, 0)
            assert st["level_big"][1] == first and st["level_big"][2] == pool


def test_bc_deep_chain(native, oracle):
    """5000 levels: the level sort's keys far beyond one per warp range."""
    import bfs_simd_benchmarks_gb300 as B
    n = 5000
    src = np.arange(n - 1, dtype=np.uint32)
    dst = src + 1
    # a few shortcuts that create two shortest paths around some vertices
    src = np.concatenate([src, np.array([10, 100, 2000], np.uint32)])
    dst = np.concatenate([dst, np.array([12, 102, 2002], np.uint32)])
    arr = oracle.arrays_from_edges(n, src, dst, 64, 4)
    with B.Graph.from_edges(n, src, dst, 64, 4) as g:
        g.set_options(bc_level_bytes=1)   # deeper than 254 levels: the 8-byte gathers are used anyway
        _check_source(oracle, arr, g, 0)
        _check_source(oracle, arr, g, 1500)


def test_bc_rmat18_permuted(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n, m = 1 << 18, 1 << 22
    src, dst = B.gen_rmat(n, m, 0.57, 0.19, 0.19, seed=181, dedup=True, no_self_loops=True, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, 1024, 16)
    deg = arr["degrees"]
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        for mode in (1, 2):
            g.set_options(bc_level_bytes=mode)
            for s in np.flatnonzero(deg > 0)[[3, 999]]:
                _check_source(oracle, arr, g, int(s))


def test_bc_accumulate_matches_networkx_and_oracle(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    c = load_bc_case("rmat10_w64_s3")
    n = c["n"]
    arr = oracle.arrays_from_edges(n, c["src"], c["dst"], c["w"], c["s"])
    scale = np.zeros(n)
    for s in range(n):
        _, _, _, sc = oracle.bc_single(arr, s)
        sc = sc.copy()
        sc[s] = 0
        scale += sc
    with B.Graph.from_edges(n, c["src"], c["dst"], c["w"], c["s"]) as g:
        bc, st = g.betweenness(np.arange(n))
        assert st["num_sources"] == n and st["status"] == 0
        ok = bc_close(bc, c["bc"], scale)
        assert ok.all(), np.flatnonzero(~ok)[:8]
        # a subset of sources against the oracle's sum
        subset = np.array([5, 77, 300, 1023], np.uint32)
        part, _ = g.betweenness(subset)
        want = np.zeros(n)
        sc_sum = np.zeros(n)
        for s in subset:
            _, d, _, sc = oracle.bc_single(arr, int(s))
            d = d.astype(np.float64)
            d[s] = 0
            sc = sc.copy()
            sc[s] = 0
            want += d
            sc_sum += sc
        assert bc_close(part, want, sc_sum).all()


def test_bc_device_entry_points_match_host(native):
    import torch
    import bfs_simd_benchmarks_gb300 as B
    c = load_case("rmat12p_w100_s5")
    n = c["n"]
    with B.Graph.from_edges(n, c["src"], c["dst"], c["w"], c["s"]) as g:
        s = int(c["sources"][1])
        dep, sig, _ = g.bc(s)
        d_dep = torch.empty(n, dtype=torch.float32, device="cuda")
        d_sig = torch.empty(n, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        g.bc_device(s, d_dep.data_ptr(), d_sig.data_ptr(), stream)
        torch.cuda.synchronize()
        assert g.bc_stats()["status"] == 0
        assert d_dep.cpu().numpy().tobytes() == dep.tobytes()
        assert d_sig.cpu().numpy().view(np.uint32).tobytes() == sig.tobytes()
        srcs = c["sources"]
        g.set_options(bc_batch=0)   # the device accumulation runs one source at a time
        host_bc, _ = g.betweenness(srcs)
        acc = torch.zeros(n, dtype=torch.float32, device="cuda")
        g.betweenness_device(srcs, acc.data_ptr(), stream)
        g.betweenness_device(srcs, acc.data_ptr(), stream)   # adds: twice the sum
        torch.cuda.synchronize()
        np.testing.assert_allclose(acc.cpu().numpy(), 2 * host_bc, rtol=1e-6, atol=1e-6)


def test_bc_arguments(native):
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import _native as N
    c = load_case("sparse15_w16_s2")
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        with pytest.raises(N.BfsError) as e:
            g.bc(c["n"])
        assert e.value.status == N.BFS_EARG
        with pytest.raises(N.BfsError):
            g.betweenness(np.array([0, c["n"] + 5], np.uint32))
        # a source with no out-edges reaches nothing else
        deg = np.bincount(c["src"], minlength=c["n"])
        s = int(np.flatnonzero(deg == 0)[0])
        dep, sig, st = g.bc(s)
        assert st["reached"] == 1 and sig[s] == 1 and (dep == 0).all()

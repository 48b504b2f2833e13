"""bfs_run_noalloc: the traversal for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc -- a plug-in whose host framework owns
all device memory, or a request path that cannot take cudaMalloc's device-wide
synchronisation.  bfs_run_noalloc keeps its scratch in a fixed device array
inside the library instead.  This test calls it through the C ABI twice in a
row (the second call runs on the scratch the first one left behind) and
checks its levels bit-exact against the regular entry point, bfs_run, and the
oracle; around the second call neither torch's allocator nor the device's
free memory may change.  It sits in its own file, collected last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _csr(n, src, dst):
    order = np.argsort(src, kind="stable")
    col = dst[order].astype(np.uint32)
    row = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(np.bincount(src, minlength=n), out=row[1:])
    return row.astype(np.uint32), col


def _call(native, torch, n, d_row, d_col, s, d_lev, d_st):
    stream = torch.cuda.current_stream()
    return native.bfs_run_noalloc(n, C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), int(s),
                                  C.c_void_p(d_lev.data_ptr()), C.c_void_p(d_st.data_ptr()),
                                  C.c_void_p(stream.cuda_stream))


def test_noalloc_matches_bfs_run_twice(native, oracle):
    torch = pytest.importorskip("torch")
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 15
    src, dst = B.gen_rmat(n, 16 * n, seed=4242, permute=True)
    row, col = _csr(n, src, dst)
    arr = oracle.arrays_from_edges(n, src, dst, 1024, 16)
    d_row = torch.from_numpy(row.view(np.int32)).cuda()
    d_col = torch.from_numpy(col.view(np.int32)).cuda()
    d_lev = torch.empty(n, dtype=torch.int32, device="cuda")
    d_st = torch.empty(1, dtype=torch.int32, device="cuda")
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        sources = B.pick_sources(g.degrees(), 2, seed=17)
        for k, s in enumerate(sources):   # two calls in a row on the same device scratch
            d_st.fill_(-7)                # the call must write its own status
            torch.cuda.synchronize()
            if k == 1:
                alloc0 = torch.cuda.memory_allocated()
                free0, _ = torch.cuda.mem_get_info()
            st = _call(native, torch, n, d_row, d_col, s, d_lev, d_st)
            assert st == 0
            torch.cuda.synchronize()
            if k == 1:
                assert torch.cuda.memory_allocated() == alloc0
                free1, _ = torch.cuda.mem_get_info()
                assert free1 == free0, "the allocation-free call changed the device's free memory"
            assert int(d_st.item()) == 0
            got = d_lev.cpu().numpy()
            expect, _, _ = g.run(int(s), parents=False)
            np.testing.assert_array_equal(got, expect)
            np.testing.assert_array_equal(got, oracle.bfs_levels(arr, int(s)))


def test_noalloc_reports_a_bad_column(native):
    torch = pytest.importorskip("torch")
    # 0 -> 1 -> {2, 9}: vertex id 9 does not exist in a 4-vertex graph
    row = np.array([0, 1, 3, 3, 3], np.uint32)
    col = np.array([1, 2, 9], np.uint32)
    d_row = torch.from_numpy(row.view(np.int32)).cuda()
    d_col = torch.from_numpy(col.view(np.int32)).cuda()
    d_lev = torch.empty(4, dtype=torch.int32, device="cuda")
    d_st = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    assert _call(native, torch, 4, d_row, d_col, 0, d_lev, d_st) == 0
    torch.cuda.synchronize()
    assert int(d_st.item()) == 4  # BFS_EARG: the bad edge was skipped and reported
    np.testing.assert_array_equal(d_lev.cpu().numpy(), [0, 1, 2, -1])


def test_noalloc_rejects_oversized_graph(native):
    big = (1 << 20) + 1
    st = native.bfs_run_noalloc(big, C.c_void_p(16), C.c_void_p(16), 0, C.c_void_p(16), None, None)
    assert st == 8  # BFS_EUNSUPPORTED, nothing launched

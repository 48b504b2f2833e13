"""bfs_run_noalloc: the traversal for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc -- a plug-in whose host framework owns
all device memory, or a request path that cannot take cudaMalloc's device-wide
synchronisation.  bfs_run_noalloc keeps its scratch in a fixed device array
inside the library instead.  This test calls it through the C ABI twice in a
row (the second call runs on the scratch the first one left behind) and
checks its levels bit-exact against the regular entry point, bfs_run.
It sits in its own file, collected last.
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


def test_noalloc_matches_bfs_run_twice(native):
    torch = pytest.importorskip("torch")
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 15
    src, dst = B.gen_rmat(n, 16 * n, seed=4242, permute=True)
    row, col = _csr(n, src, dst)
    d_row = torch.from_numpy(row.view(np.int32)).cuda()
    d_col = torch.from_numpy(col.view(np.int32)).cuda()
    d_lev = torch.empty(n, dtype=torch.int32, device="cuda")
    d_st = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        sources = B.pick_sources(g.degrees(), 2, seed=17)
        for s in sources:   # two calls in a row on the same device scratch
            st = native.bfs_run_noalloc(n, C.c_void_p(d_row.data_ptr()), C.c_void_p(d_col.data_ptr()), int(s),
                                        C.c_void_p(d_lev.data_ptr()), C.c_void_p(d_st.data_ptr()),
                                        C.c_void_p(stream.cuda_stream))
            assert st == 0
            torch.cuda.synchronize()
            assert int(d_st.item()) == 0
            expect, _, _ = g.run(int(s), parents=False)
            np.testing.assert_array_equal(d_lev.cpu().numpy(), expect)


def test_noalloc_rejects_oversized_graph(native):
    big = (1 << 20) + 1
    st = native.bfs_run_noalloc(big, C.c_void_p(16), C.c_void_p(16), 0, C.c_void_p(16), None, None)
    assert st == 8  # BFS_EUNSUPPORTED, nothing launched

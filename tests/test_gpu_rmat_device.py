"""The device R-MAT generator (bfs_gen_rmat_device, through the C ABI) draws
exactly the host generator's edge list (bfs_gen_rmat): same candidates, same
first-occurrence deduplication, same truncation, same relabelling; and a graph
built from the device arrays directly traverses to the oracle's levels."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,m,permute,dedup,loops", [
    (1 << 16, 1 << 20, False, True, False),
    (100_003, 1_500_000, True, True, False),
    (1 << 12, 1 << 16, True, False, True),
    (3000, 40000, False, True, True),
    (5, 20, False, True, False),
    (1 << 20, 1 << 24, True, True, False),
])
def test_device_generator_equals_host_generator(native, n, m, permute, dedup, loops):
    import bfs_simd_benchmarks_gb300 as B
    hs, hd = B.gen_rmat(n, m, seed=4321, permute=permute, dedup=dedup, no_self_loops=not loops)
    ds, dd = B.gen_rmat_device(n, m, seed=4321, permute=permute, dedup=dedup, no_self_loops=not loops)
    np.testing.assert_array_equal(ds.cpu().numpy().view(np.uint32), hs)
    np.testing.assert_array_equal(dd.cpu().numpy().view(np.uint32), hd)


def test_graph_from_device_edges(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n, m = 50_000, 800_000
    ds, dd = B.gen_rmat_device(n, m, seed=99, permute=True)
    hs, hd = ds.cpu().numpy().view(np.uint32), dd.cpu().numpy().view(np.uint32)
    arr = oracle.csr_arrays(n, hs, hd)
    with B.Graph.from_device_edges(n, ds.data_ptr(), dd.data_ptr(), m, 512, 8) as g:
        np.testing.assert_array_equal(g.degrees(), arr["degrees"])
        for s in B.pick_sources(arr["degrees"], 3, seed=4):
            lev, _, st = g.run(int(s), parents=False)
            np.testing.assert_array_equal(lev, oracle.bfs_levels(arr, int(s)))


def test_device_generator_argument_errors(native):
    import bfs_simd_benchmarks_gb300 as B
    with pytest.raises(B.BfsError):
        B.gen_rmat_device(4, 20, seed=1)  # more distinct edges than a 4-vertex graph has

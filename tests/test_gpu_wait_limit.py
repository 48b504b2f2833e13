"""Failure detection without a GPU fault: the bounded device waits.

Every grid barrier of the traversal kernels gives up after the run's wait
limit (bfs_options.wait_limit_us), records BFS_ETIMEOUT and lets the kernel
return, so that a CTA that never arrives cannot hang the GPU.  The test makes
such a wait run out on purpose: option test_hold_barrier makes CTA 0 skip
its arrival at one barrier, with a 1 ms limit.  The run must report
BFS_ETIMEOUT through the C ABI, and the next run on the same graph, with the
options back to normal, must give the oracle's levels (the kernel left its
barrier and status words clean).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BFS_ETIMEOUT = 6


def _graph(B):
    n = 1 << 14
    src, dst = B.gen_rmat(n, 16 * n, seed=606, permute=True)
    return n, src, dst


@pytest.mark.parametrize("hold", [1, 2, 3])
def test_single_source_wait_runs_out_then_recovers(native, oracle, hold):
    import bfs_simd_benchmarks_gb300 as B
    n, src, dst = _graph(B)
    arr = oracle.csr_arrays(n, src, dst)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        s = int(B.pick_sources(g.degrees(), 1, seed=5)[0])
        g.set_options(wait_limit_us=1000, test_hold_barrier=hold)
        with pytest.raises(B.BfsError) as e:
            g.run(s)
        assert e.value.status == BFS_ETIMEOUT
        g.set_options(wait_limit_us=0, test_hold_barrier=0)
        for _ in range(2):
            lev, _, st = g.run(s, parents=False)
            assert st["status"] == 0
            np.testing.assert_array_equal(lev, oracle.bfs_levels(arr, s))


@pytest.mark.parametrize("hold", [1, 3])
def test_batched_wait_runs_out_then_recovers(native, oracle, hold):
    import bfs_simd_benchmarks_gb300 as B
    n, src, dst = _graph(B)
    arr = oracle.csr_arrays(n, src, dst)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        sources = B.pick_sources(g.degrees(), 96, seed=6)  # above batch_single_max: the bit-sliced kernel
        g.set_options(wait_limit_us=1000, test_hold_barrier=hold)
        with pytest.raises(B.BfsError) as e:
            g.run_batch(sources)
        assert e.value.status == BFS_ETIMEOUT
        g.set_options(wait_limit_us=0, test_hold_barrier=0)
        out, st = g.run_batch(sources)
        assert st["status"] == 0
        rows = out.cpu().numpy()
        for i in (0, 17, 95):
            ref = oracle.bfs_levels(arr, int(sources[i]))
            np.testing.assert_array_equal(rows[i], np.where(ref < 0, 255, ref).astype(np.uint8))


@pytest.mark.parametrize("hold", [1, 2])
def test_batched_betweenness_wait_runs_out_then_recovers(native, oracle, hold):
    """The batched betweenness call (its traversal and its own launch share the
    option): the status comes back through bfs_bc_run_batch, and the next call
    gives the oracle's values."""
    import bfs_simd_benchmarks_gb300 as B
    from conftest import bc_close
    n, src, dst = _graph(B)
    arr = oracle.csr_arrays(n, src, dst)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        sources = B.pick_sources(g.degrees(), 8, seed=8).astype(np.uint32)
        g.set_options(wait_limit_us=1000, test_hold_barrier=hold)
        with pytest.raises(B.BfsError) as e:
            g.bc_batch(sources)
        assert e.value.status == BFS_ETIMEOUT
        g.set_options(wait_limit_us=0, test_hold_barrier=0)
        dep, sig, st = g.bc_batch(sources)
        assert st["status"] == 0 and st["batched_sources"] == sources.size
        for i in (0, 7):
            osig, odep, _, oscale = oracle.bc_single(arr, int(sources[i]))
            np.testing.assert_array_equal(sig[i], osig)
            assert bc_close(dep[i], odep, oscale).all()


def test_wait_limit_option_round_trips(native):
    import bfs_simd_benchmarks_gb300 as B
    n, src, dst = _graph(B)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        g.set_options(wait_limit_us=5000)
        lev, _, st = g.run(int(B.pick_sources(g.degrees(), 1, seed=5)[0]), parents=False)
        assert st["status"] == 0
        with pytest.raises(ValueError):
            g.set_options(no_such_option=1)

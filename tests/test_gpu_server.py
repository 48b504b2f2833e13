"""The serving loop (bfs_server_*, through the C ABI).

Each query's levels must be the same alone and in the mix: every result is
compared with that source's single-source traversal (bfs_run levels as
uint8, 255 = unreached) while queries on several graphs are submitted from
several threads, coalesced into batches and overlapped on the device.  Also:
admission by the memory budget, coalescing, device and discarded results,
open-loop replay statistics.
"""
from __future__ import annotations

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graphs(B, specs):
    out = []
    for scale, ef, seed, perm in specs:
        n = 1 << scale
        src, dst = B.gen_rmat(n, ef * n, seed=seed, permute=perm)
        out.append(B.Graph.from_edges(n, src, dst, 1024, 16))
    return out


def _alone(g, source):
    lev, _, _ = g.run(int(source), parents=False)
    return np.where(lev < 0, 255, lev).astype(np.uint8)


def test_results_alone_and_in_the_mix(native):
    import bfs_simd_benchmarks_gb300 as B
    graphs = _graphs(B, [(12, 16, 1201, False), (14, 8, 1401, True), (13, 16, 1301, False)])
    rng = np.random.default_rng(3)
    queries = []
    for gi, g in enumerate(graphs):
        srcs = B.pick_sources(g.degrees(), 60, seed=gi + 10)
        queries += [(gi, int(s)) for s in srcs]
    order = rng.permutation(len(queries))
    queries = [queries[i] for i in order]
    expect = {q: _alone(graphs[q[0]], q[1]) for q in set(queries)}
    with B.Server(budget_bytes=8 << 30, slot_bytes=64 << 20, max_batch=64, num_slots=3) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        assert ids == [0, 1, 2]
        outs = [np.zeros(graphs[q[0]].num_vertices, np.uint8) for q in queries]
        tickets = [None] * len(queries)

        def worker(part):
            for i in part:
                gi, s = queries[i]
                tickets[i] = srv.submit_host(gi, s, outs[i])

        threads = [threading.Thread(target=worker, args=(range(k, len(queries), 4),)) for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        results = [srv.wait(t) for t in tickets]
        for i, (q, r) in enumerate(zip(queries, results)):
            assert r["status"] == 0
            np.testing.assert_array_equal(outs[i], expect[q], err_msg=f"query {i} {q}")
        st = srv.stats()
        assert st["completed"] == len(queries) and st["graphs"] == 3
        assert st["batches"] < len(queries), "queries on one graph should have been coalesced"
        assert max(r["batch_size"] for r in results) > 1
        assert st["p99_ms"] >= st["p50_ms"] > 0
        deg = [g.degrees().astype(np.uint64) for g in graphs]
        m = sum(int(deg[q[0]][expect[q] != 255].sum()) for q in queries)
        assert st["edges_traversed"] == m
    for g in graphs:
        g.close()


def test_coalescing_cap_and_device_results(native):
    torch = pytest.importorskip("torch")
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import _native as N
    (g,) = _graphs(B, [(12, 16, 77, True)])
    n = g.num_vertices
    srcs = B.pick_sources(g.degrees(), 200, seed=4)
    dev = torch.zeros((len(srcs), n), dtype=torch.uint8, device="cuda")
    # slot of 40 results: at most 40 queries per traversal
    with B.Server(budget_bytes=4 << 30, slot_bytes=40 * n, max_batch=1024, num_slots=2) as srv:
        gid = srv.add_graph(g)
        tickets = [srv.submit(gid, int(s), dev[i].data_ptr(), N.BFS_DST_DEVICE) for i, s in enumerate(srcs)]
        res = [srv.wait(t) for t in tickets]
        assert max(r["batch_size"] for r in res) <= 40
        got = dev.cpu().numpy()
        for i, s in enumerate(srcs):
            np.testing.assert_array_equal(got[i], _alone(g, s), err_msg=f"source {s}")
        # discarded results still complete
        for s in srcs[:10]:
            srv.submit(gid, int(s))
        srv.drain()
        assert srv.stats()["completed"] == len(srcs) + 10
    g.close()


def test_admission_budget_and_errors(native):
    import bfs_simd_benchmarks_gb300 as B
    big, small = _graphs(B, [(16, 16, 161, False), (10, 8, 101, False)])
    with B.Server(budget_bytes=(64 << 20) + (8 << 20), slot_bytes=32 << 20, num_slots=2, planes=4) as srv:
        with pytest.raises(B.BfsError) as ei:
            srv.add_graph(big)                 # graph + batch state over the budget
        assert ei.value.status == 5           # BFS_EBUDGET
        gid = srv.add_graph(small)
        with pytest.raises(B.BfsError):
            srv.submit(gid, small.num_vertices)  # source out of range
        with pytest.raises(B.BfsError):
            srv.submit(gid + 1, 0)               # unknown graph
        assert srv.stats()["device_bytes"] <= (64 << 20) + (8 << 20)
    with pytest.raises(B.BfsError):
        B.Server(budget_bytes=1 << 20, slot_bytes=1 << 20, num_slots=2)  # slots alone exceed it
    big.close()
    small.close()


def test_replay_poisson_statistics(native):
    import bfs_simd_benchmarks_gb300 as B
    graphs = _graphs(B, [(12, 16, 5, False), (13, 16, 6, False)])
    rng = np.random.default_rng(1)
    count = 3000
    gids = rng.integers(0, 2, count).astype(np.uint32)
    srcs = np.array([int(B.pick_sources(graphs[i].degrees(), 1, seed=int(k))[0]) for k, i in enumerate(gids)],
                    np.uint32)
    arrivals = np.cumsum(rng.exponential(1e9 / 20000, count)).astype(np.uint64)  # 20k queries/s
    with B.Server(budget_bytes=4 << 30, slot_bytes=256 << 20, num_slots=3) as srv:
        for g in graphs:
            srv.add_graph(g)
        srv.replay(gids, srcs, arrivals)
        st = srv.stats()
        assert st["completed"] == count and st["submitted"] == count and st["refused"] == 0
        assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
        assert st["edges_traversed"] > 0 and st["batches"] <= count
    for g in graphs:
        g.close()

"""Parity of the CUDA path (through the C ABI) with the reference's levels.

Golden levels come from the reference's own bfs_simd; bigger graphs are
checked against the oracle's restatement of it.  Levels must be bit-exact;
parents must form a valid BFS tree; the direction trace must equal the
oracle's under the reference's switch rule.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import golden_case_names, load_case

pytestmark = pytest.mark.gpu
CASES = golden_case_names()


def _check_run(B, oracle, arr, g, src, expect=None, trace=True):
    lev, par, st = g.run(int(src))
    if expect is None:
        expect = oracle.bfs_levels(arr, int(src))
    np.testing.assert_array_equal(lev, expect, err_msg=f"levels differ from source {src}")
    assert oracle.check_parents(arr, int(src), lev, par) == 0, "parents are not a BFS tree"
    assert st["status"] == 0
    assert st["reached"] == int((lev >= 0).sum())
    deg = arr["degrees"].astype(np.uint64)
    assert st["edges_traversed"] == int(deg[lev >= 0].sum())
    if trace:
        _, _, otrace, _ = oracle.bfs_hybrid(arr, int(src))
        n = min(len(otrace), st["num_steps"])
        assert st["trace"][:n] == otrace[:n], "direction trace differs from the reference rule"
    return lev, st


@pytest.mark.parametrize("bottom_up", ["pull", "stream"])
@pytest.mark.parametrize("mode", ["persistent", "stepwise"])
@pytest.mark.parametrize("name", CASES)
def test_golden_levels_from_edges(native, oracle, name, mode, bottom_up):
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        g.set_options(mode=mode, bottom_up=bottom_up)
        for i, src in enumerate(c["sources"]):
            _check_run(B, oracle, arr, g, src, expect=c["levels"][i])


@pytest.mark.parametrize("name", CASES)
def test_golden_levels_from_reference_files(native, oracle, name, tmp_path):
    """bfs_graph_load on files written by the product tools (the README pipeline)."""
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    base = str(tmp_path / "out.x")
    B.write_edge_list(base, c["n"], c["src"], c["dst"])
    B.tool_csr_tiling(base)
    B.tool_coo_tiling(base, c["w"], c["w"])
    B.tool_column_major(base, c["w"], c["s"], c["s"])
    with B.Graph.load(base, c["w"], c["s"]) as g:
        for i, src in enumerate(c["sources"]):
            _check_run(B, oracle, arr, g, src, expect=c["levels"][i], trace=False)


@pytest.mark.parametrize("name", CASES)
def test_golden_levels_from_arrays(native, oracle, name):
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    with B.Graph.from_arrays(c["n"], arr["degrees"], arr["csr_dst"], arr["heads"], arr["tails"],
                             arr["tile_offsets"], c["w"], c["s"]) as g:
        for i, src in enumerate(c["sources"]):
            _check_run(B, oracle, arr, g, src, expect=c["levels"][i], trace=False)


@pytest.mark.parametrize("bottom_up", ["pull", "stream"])
@pytest.mark.parametrize("w,s", [(512, 8), (1024, 16), (2048, 32), (4096, 8), (96, 7)])
def test_tile_shapes_scale14(native, oracle, w, s, bottom_up):
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 14
    src, dst = B.gen_rmat(n, 16 * n, seed=1400 + w + s, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, w, s)
    srcs = B.pick_sources(arr["degrees"], 4, seed=w * 7 + s)
    with B.Graph.from_edges(n, src, dst, w, s) as g:
        g.set_options(bottom_up=bottom_up)
        for sv in srcs:
            _check_run(B, oracle, arr, g, sv)


def test_pull_long_scans_and_queue_overflow(native, oracle):
    """A graph where many destinations need long in-edge scans (hubs of in-edges
    reached late) exercises pass 2 and the full-queue fallback of the pull step."""
    import bfs_simd_benchmarks_gb300 as B
    rng = np.random.default_rng(5)
    n = 20000
    # a chain 0->1->...->199 feeding a fan-out, plus 600 high in-degree vertices whose
    # in-edges mostly come from vertices reached only at the end of the chain
    chain = np.arange(199)
    src = [chain, np.full(2000, 199)]
    dst = [chain + 1, rng.choice(np.arange(200, n), 2000, replace=False)]
    hubs = rng.choice(np.arange(200, n), 600, replace=False)
    for h in hubs:
        ins = rng.choice(np.arange(200, n), 60, replace=False)
        src.append(ins)
        dst.append(np.full(60, h))
    src = np.concatenate(src).astype(np.uint32)
    dst = np.concatenate(dst).astype(np.uint32)
    arr = oracle.arrays_from_edges(n, src, dst, 256, 4)
    with B.Graph.from_edges(n, src, dst, 256, 4) as g:
        g.set_options(to_dense_ratio=1000000, to_sparse_ratio=1000000)  # every later step bottom-up
        lev, par, st = g.run(0)
        np.testing.assert_array_equal(lev, oracle.bfs_levels(arr, 0))
        assert oracle.check_parents(arr, 0, lev, par) == 0
        assert st["dense_steps"] > 0


def test_direction_thresholds_do_not_change_levels(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 15
    src, dst = B.gen_rmat(n, 16 * n, seed=77)
    arr = oracle.arrays_from_edges(n, src, dst, 1024, 16)
    sv = int(B.pick_sources(arr["degrees"], 1, seed=5)[0])
    ref = oracle.bfs_levels(arr, sv)
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        seen = set()
        for td, ts, wmax, cmax in [(20, 20, 32, 4096), (1, 1, 32, 4096), (100000, 100000, 32, 4096),
                                   (5, 50, 8, 64), (200, 10, 64, 100000)]:
            g.set_options(to_dense_ratio=td, to_sparse_ratio=ts, warp_max_degree=wmax, cta_max_degree=cmax)
            lev, par, st = g.run(sv)
            np.testing.assert_array_equal(lev, ref)
            assert oracle.check_parents(arr, sv, lev, par) == 0
            seen.add(tuple(st["trace"]))
        assert len(seen) > 1, "the options should change the direction trace"


def test_unvisited_edge_switch_rule_and_grid_shape_do_not_change_levels(native, oracle):
    """Beamer's direction rule (switch_rule=1) and one CTA per SM: other step
    directions and another grid, the same levels, in both execution modes."""
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 15
    src, dst = B.gen_rmat(n, 16 * n, seed=78, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, 1024, 16)
    srcs = [int(s) for s in B.pick_sources(arr["degrees"], 3, seed=9)]
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        traces = set()
        for mode in ("persistent", "stepwise"):
            for alpha, beta, cps in [(14, 24, 0), (2, 8, 1), (64, 256, 0), (4, 64, 1)]:
                g.set_options(mode=mode, switch_rule=1, bu_alpha=alpha, td_beta=beta, ctas_per_sm=cps)
                for s in srcs:
                    lev, par, st = g.run(s)
                    np.testing.assert_array_equal(lev, oracle.bfs_levels(arr, s))
                    assert oracle.check_parents(arr, s, lev, par) == 0
                    traces.add((mode, alpha, beta, s, tuple(st["trace"])))
        # both modes decide the same directions for the same options
        per = {}
        for mode, a, b, s, tr in traces:
            per.setdefault((a, b, s), set()).add(tr)
        assert all(len(v) == 1 for v in per.values())
        assert len({tr for *_, tr in traces}) > 1


def test_edge_cases(native, oracle):
    import bfs_simd_benchmarks_gb300 as B
    # no edges at all
    with B.Graph.from_edges(10, np.zeros(0, np.uint32), np.zeros(0, np.uint32), 4, 2) as g:
        lev, par, st = g.run(3)
        exp = np.full(10, -1, np.int32)
        exp[3] = 0
        np.testing.assert_array_equal(lev, exp)
        assert par[3] == 3 and st["reached"] == 1
    # a single vertex with a self loop
    with B.Graph.from_edges(1, np.zeros(1, np.uint32), np.zeros(1, np.uint32), 1024, 16) as g:
        lev, _, _ = g.run(0)
        assert lev.tolist() == [0]
    # source without out-edges in a non-trivial graph; N not a multiple of 32
    n = 1000
    src, dst = B.gen_rmat(n, 8000, seed=3)
    arr = oracle.arrays_from_edges(n, src, dst, 64, 3)
    sink = int(np.flatnonzero(arr["degrees"] == 0)[0])
    with B.Graph.from_edges(n, src, dst, 64, 3) as g:
        lev, _, st = g.run(sink)
        assert (lev >= 0).sum() == 1 and lev[sink] == 0
        with pytest.raises(B.BfsError):
            g.run(n)  # source out of range


def test_run_device_on_torch_stream(native, oracle):
    torch = pytest.importorskip("torch")
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 14
    src, dst = B.gen_rmat(n, 16 * n, seed=9)
    arr = oracle.arrays_from_edges(n, src, dst, 1024, 16)
    sv = int(B.pick_sources(arr["degrees"], 1, seed=1)[0])
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        lev = torch.empty(n, dtype=torch.int32, device="cuda")
        par = torch.empty(n, dtype=torch.int32, device="cuda")
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            g.run_device(sv, lev.data_ptr(), par.data_ptr(), s.cuda_stream)
        st = g.last_stats()
        s.synchronize()
        np.testing.assert_array_equal(lev.cpu().numpy(), oracle.bfs_levels(arr, sv))
        assert oracle.check_parents(arr, sv, lev.cpu().numpy(), par.cpu().numpy().view(np.uint32)) == 0
        assert st["status"] == 0


def test_cli_dump_matches_reference_format(native, oracle, tmp_path):
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import build
    c = load_case("rmat10_w64_s3")
    base = str(tmp_path / "out.x")
    B.write_edge_list(base, c["n"], c["src"], c["dst"])
    B.tool_csr_tiling(base)
    B.tool_coo_tiling(base, 64, 64)
    B.tool_column_major(base, 64, 3, 3)
    (tmp_path / "path").mkdir()
    env = dict(os.environ, BFS_PATH_DUMP="1", BFS_RUNS="3")
    r = subprocess.run([build.CLI, base, "64", "3", "-x"], capture_output=True, text=True, cwd=tmp_path, env=env)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 4 and lines[-1].startswith("Average: ")
    assert all(len(l.split()) == 2 for l in lines[:3])
    ref = tmp_path / "ref"
    ref.mkdir()
    oracle.write_path_dump(str(ref), c["levels"][0])   # source 0 = the CLI default
    for t in range(64):
        assert (tmp_path / "path" / f"path{t}.txt").read_bytes() == (ref / f"path{t}.txt").read_bytes()


def test_pokec_shape_64_sources(native, oracle):
    """1,632,803 vertices / 30,622,564 edges, permuted R-MAT, W=1024 S=16, 64 sources."""
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import workloads
    wl = workloads.get("pokec")
    src, dst = wl.edges()
    arr = oracle.arrays_from_edges(wl.n, src, dst, wl.w, wl.s)
    srcs = wl.sources(arr["degrees"])
    assert len(srcs) == 64
    with B.Graph.from_edges(wl.n, src, dst, wl.w, wl.s) as g:
        for sv in srcs:
            lev, par, st = g.run(int(sv))
            ref, _, trace, _ = oracle.bfs_hybrid(arr, int(sv))
            np.testing.assert_array_equal(lev, ref, err_msg=f"source {sv}")
            k = min(len(trace), st["num_steps"])
            assert st["trace"][:k] == trace[:k]
        assert oracle.check_parents(arr, int(sv), lev, par) == 0


@pytest.mark.parametrize("shape", [(1 << 14, 16, 1024, 16, True), (20011, 7, 512, 8, False), (1 << 12, 24, 4096, 32, True)])
def test_device_build_matches_host_build(native, oracle, shape):
    """BFS_LOAD_DEVICE_BUILD: the same degrees, groups and packed size as the
    host build, and the reference's levels in both bottom-up variants and
    batched."""
    import bfs_simd_benchmarks_gb300 as B
    n, ef, w, s, perm = shape
    src, dst = B.gen_rmat(n, ef * n, seed=n + w, permute=perm)
    arr = oracle.arrays_from_edges(n, src, dst, w, s)
    srcs = B.pick_sources(arr["degrees"], 6, seed=3)
    with B.Graph.from_edges(n, src, dst, w, s) as gh, B.Graph.from_edges(n, src, dst, w, s, device_build=True) as gd:
        ih, idv = gh.info(), gd.info()
        for k in ("num_vertices", "num_edges", "num_groups", "packed_words", "max_out_degree", "side_length",
                  "num_stripes"):
            assert ih[k] == idv[k], k
        np.testing.assert_array_equal(gh.degrees(), gd.degrees())
        for bu in ("pull", "stream"):
            gd.set_options(bottom_up=bu)
            for sv in srcs:
                _check_run(B, oracle, arr, gd, sv)
        lev, st = gd.run_batch(B.pick_sources(arr["degrees"], 70, seed=4))
        exp = np.where(oracle.bfs_levels(arr, int(B.pick_sources(arr["degrees"], 70, seed=4)[0])) < 0, 255,
                       oracle.bfs_levels(arr, int(B.pick_sources(arr["degrees"], 70, seed=4)[0])))
        np.testing.assert_array_equal(lev.cpu().numpy()[0], exp.astype(np.uint8))


def test_device_build_rejects_bad_ids(native):
    import bfs_simd_benchmarks_gb300 as B
    with pytest.raises(B.BfsError) as ei:
        B.Graph.from_edges(10, np.array([1, 2], np.uint32), np.array([3, 10], np.uint32), 4, 2, device_build=True)
    assert ei.value.status == 2


def test_binary_save_load_roundtrip(native, oracle, tmp_path):
    """bfs_graph_save / bfs_graph_load_binary: the same layout and the
    reference's levels after a reload; truncated files are refused."""
    import bfs_simd_benchmarks_gb300 as B
    n = 1 << 13
    src, dst = B.gen_rmat(n, 16 * n, seed=808, permute=True)
    arr = oracle.arrays_from_edges(n, src, dst, 512, 8)
    path = str(tmp_path / "g.bin")
    with B.Graph.from_edges(n, src, dst, 512, 8, device_build=True) as g:
        g.save(path)
        info = g.info()
    with B.Graph.load_binary(path) as g2:
        i2 = g2.info()
        for k in ("num_vertices", "num_edges", "num_groups", "packed_words", "max_out_degree", "tile_width",
                  "stripe_length"):
            assert info[k] == i2[k], k
        np.testing.assert_array_equal(g2.degrees(), arr["degrees"])
        for bu in ("pull", "stream"):
            g2.set_options(bottom_up=bu)
            for sv in B.pick_sources(arr["degrees"], 4, seed=8):
                _check_run(B, oracle, arr, g2, sv)
    with B.Graph.load_binary(path, host_only=True) as g3:
        np.testing.assert_array_equal(g3.degrees(), arr["degrees"])
    data = open(path, "rb").read()
    open(path, "wb").write(data[: len(data) - 100])
    with pytest.raises(B.BfsError) as ei:
        B.Graph.load_binary(path)
    assert ei.value.status == 2


@pytest.mark.parametrize("name", ["rmat12p_w100_s5", "tiny_dups_w8_s2", "chain300_w32_s4", "sparse15_w16_s2"])
def test_bfs_order_matches_vertex_id_remap(native, oracle, name, tmp_path):
    """bfs_graph_bfs_order (GPU levels) gives tools/vertex_id_remap's map, and the
    tool with BFS_TOOL_DEVICE writes the same _reorder file as the host tool."""
    import shutil
    import bfs_simd_benchmarks_gb300 as B
    c = load_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    with B.Graph.from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"]) as g:
        np.testing.assert_array_equal(g.bfs_order(0), oracle.vertex_remap_map(arr))
    base = str(tmp_path / "out.x")
    B.write_edge_list(base, c["n"], c["src"], c["dst"])
    B.tool_csr_tiling(base)
    B.tool_vertex_remap(base)
    host = open(base + "_reorder", "rb").read()
    B.tool_vertex_remap(base, device=True)
    assert open(base + "_reorder", "rb").read() == host


def test_bfs_run_into_pinned_host_memory(native, oracle):
    """bfs_run with pinned (device-mapped) host buffers: the outputs are written
    by a copy kernel instead of a copy-engine transfer; 16-byte aligned and
    4-byte aligned destinations, with and without parents, and pageable
    buffers for comparison."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import _native as N
    n = (1 << 15) + 3
    src, dst = B.gen_rmat(n, 16 * n, seed=71, permute=True)
    arr = oracle.csr_arrays(n, src, dst)
    lib = N.load()
    with B.Graph.from_edges(n, src, dst, 1024, 16) as g:
        sources = B.pick_sources(g.degrees(), 3, seed=2)
        lev_p = torch.full((n + 4,), 7, dtype=torch.int32).pin_memory()
        par_p = torch.full((n + 4,), 7, dtype=torch.int32).pin_memory()
        for off in (0, 1, 3):
            for with_parents in (True, False):
                s = int(sources[off % 3])
                lev_p.fill_(7)
                par_p.fill_(7)
                st = N.Stats()
                lp = C.cast(lev_p.data_ptr() + 4 * off, C.POINTER(C.c_int32))
                pp = C.cast(par_p.data_ptr() + 4 * off, C.POINTER(C.c_uint32)) if with_parents else None
                N.check(lib.bfs_run(g.handle, s, lp, pp, C.byref(st)), "bfs_run")
                lev = lev_p.numpy()[off:off + n].copy()
                np.testing.assert_array_equal(lev, oracle.bfs_levels(arr, s))
                # nothing written outside the destination
                assert (lev_p.numpy()[:off] == 7).all() and (lev_p.numpy()[off + n:] == 7).all()
                if with_parents:
                    par = par_p.numpy()[off:off + n].view(np.uint32).copy()
                    assert oracle.check_parents(arr, s, lev, par) == 0
                else:
                    assert (par_p.numpy() == 7).all()
                assert st.status == 0 and st.reached == int((lev >= 0).sum())
        # pageable buffers through the same call
        lev2, par2, _ = g.run(int(sources[0]))
        np.testing.assert_array_equal(lev2, oracle.bfs_levels(arr, int(sources[0])))

#!/usr/bin/env python3
"""BFS GTEPS on one GB300: the hybrid top-down / bottom-up BFS of GraphPhi's
apps/bfs_simd, run through this repository's C ABI (libbfs_gb300.so).

Workload (default, `--workload pokec`): a seeded R-MAT stand-in for Pokec with
1,632,803 vertices and 30,622,564 directed edges (a=0.57 b=0.19 c=0.19,
permuted ids, self loops and duplicates removed), tile width 1024, stripe
length 16, and 64 seeded sources with out-degree > 0.  One step = the 64
single-source traversals; GTEPS = sum over sources of m(s) (out-degrees of the
reached vertices) / time.

  value : device time (CUDA events on the launching stream) of the traversals,
          graph resident in HBM, L2 flushed (256 MiB write) before every traversal
  e2e   : the same traversals through the public bfs_run() call, levels copied
          to pinned host memory every traversal, host wall clock
  --impl reference : the CPU restatement of the reference's algorithm (oracle/,
          OpenMP on all host cores) on a bounded sample of the same workload

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

L2_FLUSH_BYTES = 256 << 20
DEVICE_BUILD_EDGES = 1 << 26  # graphs this large build their layout on the GPU (BFS_LOAD_DEVICE_BUILD)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", default="pokec")
    ap.add_argument("--mode", choices=["persistent", "stepwise"], default="persistent")
    ap.add_argument("--bottom-up", choices=["pull", "stream"], default="pull")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="bound of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sources", type=int, default=0, help="use only the first K sources (profiling runs)")
    ap.add_argument("--batch-workload", default="rmat22", help="graph of the batched measurement ('none' skips it)")
    ap.add_argument("--batch-sources", type=int, default=4096)
    ap.add_argument("--batch-steps", type=int, default=5)
    ap.add_argument("--batch-budget-mb", type=int, default=40960, help="HBM budget of the batched level planes")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (measure with the default options)")
    ap.add_argument("--bc-sources", type=int, default=16, help="betweenness measurement: sources (0 skips it)")
    ap.add_argument("--serve", default="c4", help="serving measurement: 'c4' (8 graphs, Poisson load) or 'none'")
    ap.add_argument("--serve-rates", default="2000,10000,50000", help="query arrival rates (queries/s)")
    ap.add_argument("--serve-seconds", type=float, default=1.5, help="arrival window per rate")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(workload: str):
    """Per-launch DRAM bytes of the traversal kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    ent = d.get(workload)
    return None if ent is None else ent.get("dram_bytes_per_launch")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        for line in (getattr(self, "out", "") or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes(st: dict, n: int, sw: int, pull: bool) -> int:
    """Bytes a traversal must move at minimum, from its device counters.

    Top-down: 4 B per CSR edge read, 12 B per frontier vertex expanded (queue
    entry + two row offsets).  Bottom-up, pull: 8 B per in-edge read (its
    source id + the frontier word tested), 8 B per destination tested (two
    in-list offsets) and 2 N/8-byte bitmap reads per step (visited, has-in);
    stream: 4 B per packed tile word and S*W/8 B per frontier slice staged.
    Always: 8 B per reached vertex (level + parent), 8 B per vertex of
    initialisation, two N/8-byte bitmap passes per step.
    """
    bu = (8 * st["bu_words"] + 8 * st["bu_vertices"] + st["dense_steps"] * 2 * ((n + 7) // 8)) if pull else \
        (4 * st["bu_words"] + (sw // 8) * st["bu_slices"])
    return (4 * st["td_edges"] + 12 * st["td_vertices"] + bu
            + 8 * st["reached"] + 8 * n + st["num_steps"] * 2 * ((n + 7) // 8))


def cpu_baseline(wl, src, dst, sources, seconds: float, per_call=None):
    """The oracle (the reference's algorithm restated, OpenMP on all host cores) on a bounded sample."""
    from oracle import oracle as O
    O.build(with_reference=False)
    arr = O.arrays_from_edges(wl.n, src, dst, wl.w, wl.s)
    deg = arr["degrees"].astype(np.uint64)
    threads = O.max_threads()
    edges = 0
    secs = 0.0
    done = []
    levels = {}
    t0 = time.perf_counter()
    for s in sources:
        cost, _, _, t = O.bfs_hybrid(arr, int(s), threads=threads)
        edges += int(deg[cost >= 0].sum())
        secs += t
        done.append(int(s))
        levels[int(s)] = cost
        if time.perf_counter() - t0 > seconds:
            break
    return {"value": edges / secs / 1e9, "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"{len(done)} of {len(sources)} sources of the same graph, the reference's timed region "
                      f"(traversal only), oracle/bfs_oracle.c OpenMP build"}, levels, arr


def aggregate_replicas(torch, total_ms: float, edges: int, dev, world: int):
    """Replicas: the job's time is the slowest rank's, its work every rank's."""
    if world <= 1:
        return total_ms, float(edges)
    t = torch.tensor([total_ms, float(edges)], dtype=torch.float64, device=dev)
    tmax = t.clone()
    torch.distributed.all_reduce(tmax, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
    return float(tmax[0]), float(t[1])


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from bfs_simd_benchmarks_gb300 import workloads
    import bfs_simd_benchmarks_gb300 as B
    B.load_library(build_if_missing=True)
    wl = workloads.get(args.workload)
    src, dst = wl.edges()
    from oracle import oracle as O
    O.build(with_reference=False)
    arr = O.arrays_from_edges(wl.n, src, dst, wl.w, wl.s)
    deg = arr["degrees"].astype(np.uint64)
    sources = wl.sources(arr["degrees"])
    threads = O.max_threads()
    per_step = 4
    it = 0

    def step():
        nonlocal it
        e, t = 0, 0.0
        for _ in range(per_step):
            s = int(sources[it % len(sources)])
            it += 1
            cost, _, _, sec = O.bfs_hybrid(arr, s, threads=threads)
            e += int(deg[cost >= 0].sum())
            t += sec
        return e, t

    for _ in range(args.warmup):
        step()
    E, T = 0, 0.0
    for _ in range(args.steps):
        e, t = step()
        E += e
        T += t
    val = E / T / 1e9
    line = {"metric": "BFS GTEPS (1-src & 4096-src batched), query p50/p99 ms; vs plain GPU BFS",
            "impl": "reference", "value": val, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": T / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded R-MAT)",
            "config": dict(wl.describe(), step=f"{per_step} single-source traversals on the host cores"),
            "cpu_baseline": {"value": val, "unit": "GTEPS", "cores": threads, "kind": "port",
                             "sample": f"{per_step} sources per step, {args.steps} steps, the reference's "
                                       "timed region, oracle/bfs_oracle.c OpenMP build"},
            "e2e": {"value": val, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def bench_batched(args, torch, dev, graph=None, build_s=0.0):
    """Batched multi-source BFS (bfs_run_batch): every step traverses all the
    sources at once and writes uint8 levels [sources][N] into HBM.  Compared
    with the single-source kernel on the same graph (the plain GPU BFS).
    `graph` is the single-source workload's graph when both are the same."""
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import workloads
    wl = workloads.get(args.batch_workload)
    if graph is None:
        t0 = time.perf_counter()
        src, dst = wl.edges()
        g = B.Graph.from_edges(wl.n, src, dst, wl.w, wl.s, device_build=wl.m >= DEVICE_BUILD_EDGES)
        build_s = time.perf_counter() - t0
        del src, dst
    else:
        g = graph
    g.set_options(batch_budget_mb=args.batch_budget_mb)
    deg = g.degrees()
    sources = wl.sources(deg, args.batch_sources)
    out = torch.empty((len(sources), wl.n), dtype=torch.uint8, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    tuned = None
    if not args.no_tune:
        t_t = time.perf_counter()
        r = g.tune(sources, single=False, batch=True)
        tuned = {"batch_push_div": r["options"]["batch_push_div"], "tuned_gteps": r["batch_gteps"],
                 "default_gteps": r["default_batch_gteps"], "trials": r["num_trials"],
                 "seconds": round(time.perf_counter() - t_t, 2),
                 "note": "the bit-sliced kernel reads CSR + in-edge lists only: tile width and stripe length "
                         "do not enter it, so only its push/pull threshold is tuned"}
    runs = []
    for i in range(max(3, args.warmup) + args.batch_steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.run_batch_device(sources, out.data_ptr(), stream.cuda_stream)
            e1.record(stream)
        st = g.last_batch_stats()
        if st["status"] != 0:
            raise RuntimeError(f"batched traversal status {st['status']}")
        if i >= max(3, args.warmup):
            runs.append((e0.elapsed_time(e1), st))
    ms = [r[0] for r in runs]
    edges = runs[0][1]["edges_traversed"]
    gteps = edges * len(ms) / (sum(ms) / 1e3) / 1e9
    # the same batch as one CUDA-graph launch (sources resident on the device)
    d_src = torch.tensor(np.asarray(sources, dtype=np.int64), dtype=torch.int32, device=dev)
    gms = []
    with g.batch_graph(d_src.data_ptr(), len(sources), out.data_ptr()) as bgr:
        for i in range(max(3, args.warmup) + args.batch_steps):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xFF)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                bgr.launch(stream.cuda_stream)
                e1.record(stream)
            gst = g.last_batch_stats()
            if gst["status"] != 0 or gst["edges_traversed"] != edges:
                raise RuntimeError("CUDA-graph batch differs from the direct launch")
            if i >= max(3, args.warmup):
                gms.append(e0.elapsed_time(e1))
    cuda_graph = {"ms_per_batch_mean": statistics.mean(gms), "gteps": edges * len(gms) / (sum(gms) / 1e3) / 1e9,
                  "launch": "bfs_batch_graph_launch: memset + cooperative traversal + output pass as one graph"}
    # the single-source kernel on the same graph, a sample of the same sources
    lev = torch.empty(wl.n, dtype=torch.int32, device=dev)
    single_ms, single_edges, rows_ok = [], 0, 0
    check = list(range(0, len(sources), max(1, len(sources) // 8)))[:8]
    host = out.cpu() if len(sources) * wl.n <= (1 << 31) else None
    for j, s in enumerate(sources[:64]):
        with torch.cuda.stream(stream):
            flush.fill_(j & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.run_device(int(s), lev.data_ptr(), 0, stream.cuda_stream)
            e1.record(stream)
        st = g.last_stats()
        single_ms.append(e0.elapsed_time(e1))
        single_edges += st["edges_traversed"]
    for i in check:
        with torch.cuda.stream(stream):
            g.run_device(int(sources[i]), lev.data_ptr(), 0, stream.cuda_stream)
        g.last_stats()
        ref = lev.cpu().numpy()
        ref = np.where(ref < 0, 255, ref).astype(np.uint8)
        row = host[i].numpy() if host is not None else out[i].cpu().numpy()
        rows_ok += int(np.array_equal(row, ref))
    single_gteps = single_edges / (sum(single_ms) / 1e3) / 1e9
    st = runs[-1][1]
    # algorithmic bytes of a batch: every level writes its N x K-word plane, every
    # frontier word a pull reads is 8 B (above 512 sources the device counts one
    # word per row read, so this is a lower bound), the output is N bytes per source
    alg = st["depth"] * 8 * st["words_per_vertex"] * wl.n + 8 * st["words_gathered"] + len(sources) * wl.n
    peak, peak_kind = peaks()
    achieved = alg / (statistics.mean(ms) / 1e3) / 1e9
    res = {
        "workload": wl.describe() | {"sources": len(sources)}, "graph_build_s": round(build_s, 2),
        "gteps": gteps, "ms_per_batch_mean": statistics.mean(ms), "ms_per_batch_p50": statistics.median(ms),
        "levels_ms_mean": statistics.mean(r[1]["levels_ms"] for r in runs),
        "edges_traversed_per_batch": edges, "depth": st["depth"], "push_levels": st["push_levels"],
        "planes": st["planes"], "spills": st["spills"], "words_gathered": st["words_gathered"],
        "level_ms": st["level_ms"], "level_frontier": st["level_frontier"], "level_push": st["level_push"],
        "level_phase_ms": st["level_phase_ms"], "setup_ms": st["setup_ms"], "output_ms": st["output_ms"],
        "grid_ctas": st["grid_ctas"], "batch_state_bytes": st["device_bytes"],
        "output_bytes": len(sources) * wl.n,
        "plain_gpu_bfs": {"gteps": single_gteps, "ms_per_traversal_mean": statistics.mean(single_ms),
                          "sources": len(single_ms), "kernel": "k_bfs_persistent (single source)"},
        "speedup_vs_plain_gpu_bfs": gteps / single_gteps,
        "cuda_graph": cuda_graph,
        "autotune": tuned,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "kernels": "k_ms_bfs + k_ms_emit", "peak_kind": peak_kind, "algorithmic_bytes_per_batch": alg},
        "parity": f"batched rows equal single-source levels on {rows_ok}/{len(check)} sources checked",
        "steps": len(ms), "l2": "flushed (256 MiB write) before every batch; batch state far above L2",
    }
    if graph is None:
        g.close()
    del out
    torch.cuda.empty_cache()
    return res


def bench_bc(args, torch, dev, g, sources, flush, arr=None):
    """Betweenness dependencies (bfs_bc_run_device, apps/betweennessCentrality_simd
    /bc.cpp:1717): per source one single-source traversal and one dependency
    launch (level sort, path counts, dependency sums).  GTEPS = sum of m(s)
    (out-degrees of reached vertices) / device time, L2 flushed before each
    source; e2e through bfs_bc_run with float dependencies copied to the host."""
    n = g.num_vertices
    srcs = [int(s) for s in sources[: args.bc_sources]]
    stream = torch.cuda.Stream(device=dev)
    dep = torch.empty(n, dtype=torch.float32, device=dev)
    sig = torch.empty(n, dtype=torch.int32, device=dev)

    def one(s):
        with torch.cuda.stream(stream):
            flush.fill_(s & 0xFF)
        g.bc_device(s, dep.data_ptr(), sig.data_ptr(), stream.cuda_stream)
        st = g.bc_stats()
        if st["status"] != 0:
            raise RuntimeError(f"betweenness device status {st['status']}")
        return st

    for _ in range(max(1, args.warmup)):
        one(srcs[0])
    torch.cuda.synchronize()
    sts = []
    for _ in range(args.steps):
        for s in srcs:
            sts.append(one(s))
    dev_ms = sum(st["device_ms"] for st in sts)
    trav_ms = sum(st["traversal_ms"] for st in sts)
    edges = sum(st["edges_reached"] for st in sts)
    k_ms = dev_ms - trav_ms
    read_edges = sum(st["edges_forward"] + st["edges_reverse"] for st in sts)
    reached = sum(st["reached"] for st in sts)
    # algorithmic bytes of the dependency launch: per edge read its neighbour id
    # and the neighbour's level (8 B); per reached vertex its level, two offset
    # pairs, its order slot, path count, sum and dependency (40 B); per vertex
    # the sort's level read and the initialised outputs (12 B)
    alg = 8 * read_edges + 40 * reached + 12 * n * len(sts)
    peak, _ = peaks()
    ach = alg / (k_ms / 1e3) / 1e9 if k_ms > 0 else 0.0
    # e2e: host dependencies
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_edges = 0
    for s in srcs:
        d, _, st = g.bc(s, paths=False)
        e2e_edges += st["edges_reached"]
    e2e_s = time.perf_counter() - t0
    out = {
        "what": "betweenness dependencies of single sources (forward path counts + reverse float sums)",
        "sources": len(srcs), "steps": args.steps,
        "gteps": edges / (dev_ms / 1e3) / 1e9,
        "ms_per_source_mean": dev_ms / len(sts),
        "traversal_ms_mean": trav_ms / len(sts),
        "dependency_kernel_ms_mean": k_ms / len(sts),
        "phase_ms_mean": {k: statistics.mean(st[k] for st in sts) for k in ("sort_ms", "paths_ms", "dependencies_ms")},
        "depth_mean": statistics.mean(st["depth"] for st in sts),
        "example_levels": {k: sts[0][k] for k in ("level_vertices", "level_big", "level_medium", "level_paths_ms",
                                                  "level_dependencies_ms")},
        "roofline": {"kernel": "k_bc", "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak if peak else None, "algorithmic_bytes_per_launch": alg / len(sts)},
        "e2e": {"value": e2e_edges / e2e_s / 1e9, "unit": "GTEPS", "d2h_bytes_per_step": 4 * n * len(srcs),
                "note": "bfs_bc_run(): float dependencies to host memory"},
        "gpu_launches": 3 * len(sts),
    }
    if arr is not None:
        from oracle import oracle as O
        ok = 0
        checked = srcs[:2]
        cpu_s = 0.0
        cpu_edges = 0
        deg = arr["degrees"].astype(np.uint64)
        for s in checked:
            t1 = time.perf_counter()
            osig, odep, ocost, oscale = O.bc_single(arr, s)
            cpu_s += time.perf_counter() - t1
            cpu_edges += int(deg[ocost >= 0].sum())
            d, p, _ = g.bc(s)
            ok += int(np.array_equal(p, osig) and
                      bool((np.abs(d.astype(np.float64) - odep) <= 1e-4 * (np.abs(oscale) + 1)).all()))
        out["parity"] = (f"{ok}/{len(checked)} sources: path counts bit-exact, dependencies within "
                         "1e-4 x (scale + 1) of the oracle")
        out["cpu_baseline"] = {"value": cpu_edges / cpu_s / 1e9, "unit": "GTEPS", "cores": 1, "kind": "port",
                               "sample": f"{len(checked)} sources, oracle/bfs_oracle.c orc_bc_single (sequential, "
                                         "includes building the reverse graph)"}
    return out


def bench_serving(args, torch, dev):
    """The serving loop: 8 resident R-MAT graphs (scales 14, 16, 18-23, edge
    factor 16) under a 40 GB HBM admission budget; open-loop Poisson arrivals
    of (graph, source) queries drawn uniformly, coalesced per graph into
    batches of up to 1024 sources; levels are computed and left on the device
    (BFS_DST_NONE) so that latency measures the traversal path."""
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import workloads
    t0 = time.perf_counter()
    graphs = []
    for wl in workloads.serve_graphs():
        src, dst = wl.edges()
        graphs.append((wl, B.Graph.from_edges(wl.n, src, dst, wl.w, wl.s, device_build=wl.m >= DEVICE_BUILD_EDGES)))
        del src, dst
    build_s = time.perf_counter() - t0
    srv = B.Server(budget_bytes=40 * 10**9)
    for _, g in graphs:
        srv.add_graph(g)
    pools = [wl.sources(g.degrees(), 4096) for wl, g in graphs]
    rng = np.random.default_rng(2024)

    def trace(rate, seconds):
        count = max(1, int(rate * seconds))
        gids = rng.integers(0, len(graphs), count).astype(np.uint32)
        picks = rng.integers(0, 4096, count)
        srcs = np.array([pools[gi][k] for gi, k in zip(gids, picks)], dtype=np.uint32)
        arr = np.cumsum(rng.exponential(1e9 / rate, count)).astype(np.uint64)
        return gids, srcs, arr

    srv.replay(*trace(5000, 0.4))  # warm-up
    rates = []
    with ClockSampler(dev.index or 0) as clk:
        for rate in [float(x) for x in args.serve_rates.split(",") if x]:
            gids, srcs, arr = trace(rate, args.serve_seconds)
            srv.reset_stats()
            t1 = time.perf_counter()
            srv.replay(gids, srcs, arr)
            wall = time.perf_counter() - t1
            st = srv.stats()
            rates.append({"offered_qps": rate, "queries": int(st["completed"]), "achieved_qps": st["completed"] / wall,
                          "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
                          "max_ms": st["max_ms"], "mean_batch": st["mean_batch"], "batches": int(st["batches"]),
                          "gteps": st["edges_traversed"] / wall / 1e9, "wall_s": wall,
                          "slots_in_flight_mean": st["device_ms"] / 1e3 / wall})
    res = {"graphs": [{"workload": wl.name, "vertices": wl.n, "edges": wl.m} for wl, _ in graphs],
           "budget_bytes": 40 * 10**9, "admitted_bytes": srv.stats()["device_bytes"], "graph_build_s": round(build_s, 1),
           "max_batch": 1024, "slots": 3, "results": "left on the device (BFS_DST_NONE)",
           "latency": "submit -> traversal and output pass complete, host clock", "rates": rates,
           "clocks": clk.summary()}
    srv.close()
    for _, g in graphs:
        g.close()
    torch.cuda.empty_cache()
    return res


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import _native as N
    from bfs_simd_benchmarks_gb300 import workloads
    B.load_library(build_if_missing=True)
    wl = workloads.get(args.workload)
    t_gen = time.perf_counter()
    src, dst = wl.edges()
    g = B.Graph.from_edges(wl.n, src, dst, wl.w, wl.s, device_build=wl.m >= DEVICE_BUILD_EDGES)
    g.set_options(mode=args.mode, bottom_up=args.bottom_up)
    info = g.info()
    t_gen = time.perf_counter() - t_gen
    degrees = g.degrees()
    sources = wl.sources(degrees)
    if args.sources:
        sources = sources[: args.sources]
    n = wl.n
    sw = wl.s * wl.w
    tuned = None
    if not args.no_tune and args.mode == "persistent":
        t_t = time.perf_counter()
        r = g.tune(sources, single=True)
        tuned = {"options": {k: r["options"][k] for k in ("bottom_up", "to_dense_ratio", "to_sparse_ratio",
                                                           "warp_max_degree", "cta_max_degree")},
                 "tuned_gteps_kernel": r["single_gteps"], "default_gteps_kernel": r["default_single_gteps"],
                 "trials": r["num_trials"], "seconds": round(time.perf_counter() - t_t, 2)}
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    lev = torch.empty(n, dtype=torch.int32, device=dev)
    par = torch.empty(n, dtype=torch.int32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)

    def traverse(s: int, timed: list | None):
        with torch.cuda.stream(stream):
            flush.fill_(s & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.run_device(int(s), lev.data_ptr(), par.data_ptr(), stream.cuda_stream)
            e1.record(stream)
        st = g.last_stats()  # synchronises on the stream after the traversal
        if timed is not None:
            timed.append((e0, e1, st))
        return st

    # warm-up steps (also records m(s) of every source)
    for _ in range(args.warmup):
        for s in sources:
            traverse(int(s), None)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    timed = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            for s in sources:
                traverse(int(s), timed)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    trav_ms = [a.elapsed_time(b) for a, b, _ in timed]
    kern_ms = [st["kernel_ms"] for _, _, st in timed]
    edges = sum(st["edges_traversed"] for _, _, st in timed)
    for _, _, st in timed:
        if st["status"] != 0:
            raise RuntimeError(f"device status {st['status']}")
    total_ms = sum(trav_ms)
    total_ms_max, edges_all = aggregate_replicas(torch, total_ms, edges, dev, world)
    value = edges_all / (total_ms_max / 1e3) / 1e9

    # roofline of the traversal kernel (k_bfs_persistent), per launch
    alg = [algorithmic_bytes(st, n, sw, args.bottom_up == "pull") for _, _, st in timed]
    achieved = statistics.mean(alg) / (statistics.mean(kern_ms) / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = ncu_traffic(args.workload)

    # e2e through the public call with host buffers
    lib = N.load()
    pinned = torch.empty(n, dtype=torch.int32, pin_memory=True)
    pptr = C.cast(pinned.data_ptr(), C.POINTER(C.c_int32))
    torch.cuda.synchronize()
    e2e_edges = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s in sources:
            stc = N.Stats()
            N.check(lib.bfs_run(g.handle, int(s), pptr, None, C.byref(stc)), "bfs_run")
            e2e_edges += stc.edges_traversed
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = e2e_edges / e2e_s / 1e9

    batched = None
    if args.batch_workload != "none" and world == 1:
        same = args.batch_workload == args.workload
        batched = bench_batched(args, torch, dev, g if same else None, t_gen if same else 0.0)
    serving = None
    if args.serve != "none" and world == 1:
        serving = bench_serving(args, torch, dev)

    cpu = None
    parity = None
    cpu_arr = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, cpu_levels, cpu_arr = cpu_baseline(wl, src, dst, sources, args.cpu_seconds)
        ok = 0
        for s, ref in cpu_levels.items():
            got, _, _ = g.run(s, parents=False)
            ok += int(np.array_equal(got, ref))
        parity = f"levels bit-exact on {ok}/{len(cpu_levels)} sources checked against the oracle"
    bc = None
    if args.bc_sources > 0 and world == 1:
        bc = bench_bc(args, torch, dev, g, sources, flush, cpu_arr)
    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": "BFS GTEPS (1-src & 4096-src batched), query p50/p99 ms; vs plain GPU BFS",
            "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded R-MAT stand-in, see config)",
            "config": dict(wl.describe(), step=f"{len(sources)} single-source traversals",
                           parallelism="replicas" if world > 1 else "single GPU", mode=args.mode,
                           bottom_up=args.bottom_up,
                           l2=f"flushed (256 MiB write) before every traversal; graph {info['device_bytes'] / 1e6:.0f} MB > L2",
                           grid_ctas=timed[0][2]["grid_ctas"], column_groups=info["num_groups"],
                           autotune=tuned,
                           graph_build_s=round(t_gen, 2)),
            "single_source": {"gteps": value, "ms_per_traversal_mean": statistics.mean(trav_ms),
                              "ms_per_traversal_p50": statistics.median(trav_ms),
                              "ms_per_traversal_p99": float(np.percentile(trav_ms, 99)),
                              "edges_per_traversal_mean": edges / len(timed),
                              "dense_steps_mean": statistics.mean(st["dense_steps"] for _, _, st in timed),
                              "steps_mean": statistics.mean(st["num_steps"] for _, _, st in timed),
                              "phase_ms_mean": {k: statistics.mean(st[k] for _, _, st in timed)
                                                for k in ("dense_ms", "to_dense_ms", "sparse_ms", "to_sparse_ms")},
                              "example_steps": {"trace": timed[0][2]["trace"], "step_ms": timed[0][2]["step_ms"]},
                              "bu_cycles_per_cta_mean": [round(statistics.mean(st["bu_cycles"][i] for _, _, st in timed)
                                                               / max(1, timed[0][2]["grid_ctas"])) for i in range(6)]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_bfs_persistent", "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                         if peak_kind == "measured" else "fallback",
                         "algorithmic_bytes_per_launch": statistics.mean(alg),
                         "launch_ms_mean": statistics.mean(kern_ms)},
            "e2e": {"value": e2e_value, "unit": "GTEPS", "h2d_bytes_per_step": 4 * len(sources),
                    "d2h_bytes_per_step": 4 * n * len(sources),
                    "note": "bfs_run(): source as a launch parameter, int32 levels to pinned host memory"},
            "gpu_launches": 2 * len(timed),
            "clocks": clocks,
            "cpu_baseline": cpu,
            "parity": parity,
            "batched": batched,
            "serving": serving,
            "betweenness": bc,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    g.close()


if __name__ == "__main__":
    main()

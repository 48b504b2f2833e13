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

from bfs_simd_benchmarks_gb300 import workloads  # noqa: E402  (numpy only: loads no library)

L2_FLUSH_BYTES = 256 << 20
DEVICE_BUILD_EDGES = 1 << 26  # graphs this large build their layout on the GPU (BFS_LOAD_DEVICE_BUILD)


METRIC = "BFS GTEPS (1-src & 4096-src batched), query p50/p99 ms; vs plain GPU BFS"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", default="pokec")
    ap.add_argument("--mode", choices=["persistent", "stepwise"], default="persistent")
    ap.add_argument("--bottom-up", choices=["pull", "stream"], default=None,
                    help="bottom-up variant (default: the autotuner's choice, pull without tuning)")
    ap.add_argument("--no-shape-search", action="store_true",
                    help="keep the workload's tile width / stripe length / layout (skip bfs_autotune)")
    ap.add_argument("--tile-width", type=int, default=0, help="with --no-tune: this tile width (profiling runs)")
    ap.add_argument("--stripe-length", type=int, default=0, help="with --no-tune: this stripe length")
    ap.add_argument("--degree-order", action="store_true", help="with --no-tune: the degree-ordered layout")
    ap.add_argument("--options", default="", help="with --no-tune: traversal options as JSON (profiling runs)")
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
    ap.add_argument("--large", default="twitter", help="large single-GPU graph measured last ('none' skips it)")
    ap.add_argument("--large-sources", type=int, default=16, help="large graph: single-source traversals")
    ap.add_argument("--large-batch", type=int, default=1024, help="large graph: sources of the batched traversal")
    ap.add_argument("--large-budget-mb", type=int, default=65536, help="large graph: HBM budget of the level planes")
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


def ncu_traffic(workload: str, key: str = "dram_bytes_per_launch"):
    """DRAM bytes per launch (or per batch) from the committed ncu summaries, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    ent = d.get(workload)
    return None if ent is None else ent.get(key)


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


def host_cpu_info() -> dict:
    """The host cores the CPU legs run on: count, model and ISA."""
    import platform
    info = {"machine": platform.machine(), "nproc": os.cpu_count(),
            "cores_usable": len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()}
    model, flags, impl, part = None, "", None, None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                k, v = k.strip().lower(), v.strip()
                if k == "model name" and model is None:
                    model = v
                elif k in ("flags", "features") and not flags:
                    flags = v
                elif k == "cpu implementer" and impl is None:
                    impl = v
                elif k == "cpu part" and part is None:
                    part = v
    except OSError:
        pass
    arm_parts = {("0x41", "0xd4f"): "Arm Neoverse V2 (NVIDIA Grace)", ("0x41", "0xd40"): "Arm Neoverse V1",
                 ("0x41", "0xd0c"): "Arm Neoverse N1", ("0x41", "0xd8e"): "Arm Neoverse N3",
                 ("0x41", "0xd84"): "Arm Neoverse V3"}
    if model is None and impl is not None:
        model = arm_parts.get((impl.lower(), (part or "").lower()), f"Arm implementer {impl} part {part}")
    fl = set(flags.split())
    simd = [x for x in ("avx512f", "avx512bw", "avx2", "sve2", "sve", "asimd") if x in fl]
    info["model"] = model
    info["isa"] = info["machine"] + (" + " + ", ".join(simd) if simd else "")
    info["oracle_build"] = "plain C + OpenMP, gcc -O2 (scalar loops; no explicit SIMD)"
    if "avx512f" not in fl:
        info["note"] = "no AVX-512 on this host: the reference's bfs_simd (AVX-512 intrinsics) cannot run here"
    return info


def bench_config(wl, num_sources: int) -> dict:
    """The workload both arms (GPU and reference) measure: same keys, same values."""
    return dict(wl.describe(), sources=num_sources, step=f"{num_sources} single-source traversals",
                l2="GPU arm: flushed (256 MiB write) before every traversal; graph far above L2")


def oracle_workload(wl, limit: int = 0):
    """The workload's graph and sources built on the checker's side only
    (oracle/: generator, tool orders, CSR); no product library is loaded."""
    from oracle import oracle as O
    O.build(with_reference=False)
    src, dst = O.gen_rmat(wl.n, wl.m, wl.a, wl.b, wl.c, seed=wl.seed, permute=wl.permute)
    arr = O.arrays_from_edges(wl.n, src, dst, wl.w, wl.s)
    sources = wl.sources(arr["degrees"])
    if limit:
        sources = sources[:limit]
    return O, arr, [int(s) for s in sources]


def cpu_leg(args, wl, keep_levels: int = 8):
    """cpu_baseline: the oracle (the reference's algorithm restated, OpenMP on
    all host cores) timed on a bounded sample of the same workload.  It runs
    before torch or CUDA are touched in this process, with a warm-up, so its
    rate is the reference arm's."""
    O, arr, sources = oracle_workload(wl, args.sources)
    deg = arr["degrees"].astype(np.uint64)
    threads = O.max_threads()
    for s in sources[:4]:  # warm-up: thread pool, page faults of the per-run arrays
        O.bfs_hybrid(arr, s, threads=threads)
    edges, secs, runs, passes = 0, 0.0, 0, 0
    levels = {}
    t0 = time.perf_counter()
    while True:
        for s in sources:
            cost, _, _, t = O.bfs_hybrid(arr, s, threads=threads)
            edges += int(deg[cost >= 0].sum())
            secs += t
            runs += 1
            if passes == 0 and len(levels) < keep_levels:
                levels[s] = cost
        passes += 1
        if time.perf_counter() - t0 > args.cpu_seconds:
            break
    return {"value": edges / secs / 1e9, "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"{passes} pass(es) over all {len(sources)} sources of the same graph ({runs} traversals) "
                      "after a 4-traversal warm-up, the reference's timed region (traversal only, "
                      "apps/bfs_simd/bfs.cpp:806-913), oracle/bfs_oracle.c OpenMP build, run before any "
                      "CUDA work in this process",
            "host": host_cpu_info()}, levels


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
    """The reference arm: the reference's CPU algorithm (oracle/bfs_oracle.c,
    OpenMP on all host cores; bfs_simd itself needs AVX-512) on the same
    workload, config and metric as the GPU arm.  One step = every source once,
    like the GPU arm's step.  Only the checker's library is loaded."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    wl = workloads.get(args.workload)
    O, arr, sources = oracle_workload(wl, args.sources)
    deg = arr["degrees"].astype(np.uint64)
    threads = O.max_threads()

    def step():
        e, t = 0, 0.0
        for s in sources:
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
    line = {"metric": METRIC, "impl": "reference", "value": val, "unit": "GTEPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": T / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded R-MAT stand-in, see config)", "config": bench_config(wl, len(sources)),
            "cpu_baseline": {"value": val, "unit": "GTEPS", "cores": threads, "kind": "port",
                             "sample": f"all {len(sources)} sources per step, {args.steps} steps after "
                                       f"{args.warmup} warm-up steps, the reference's timed region "
                                       "(apps/bfs_simd/bfs.cpp:806-913), oracle/bfs_oracle.c OpenMP build",
                             "host": host_cpu_info()},
            "e2e": {"value": val, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def bench_batched(args, torch, dev, graph=None, build_s=0.0, edges=None):
    """Batched multi-source BFS (bfs_run_batch): every step traverses all the
    sources at once and writes uint8 levels [sources][N] into HBM.  Compared
    with the single-source kernel on the same graph (the plain GPU BFS);
    sampled rows are checked against the oracle.  `graph` (and its `edges`)
    is the single-source workload's graph when both are the same."""
    import bfs_simd_benchmarks_gb300 as B
    from oracle import oracle as O
    wl = workloads.get(args.batch_workload)
    if graph is None:
        t0 = time.perf_counter()
        src, dst = wl.edges()
        g = B.Graph.from_edges(wl.n, src, dst, wl.w, wl.s, device_build=wl.m >= DEVICE_BUILD_EDGES)
        build_s = time.perf_counter() - t0
    else:
        g = graph
        src, dst = edges
    oarr = O.csr_arrays(wl.n, src, dst)
    del src, dst
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
        ref = O.bfs_levels(oarr, int(sources[i]))
        ref = np.where(ref < 0, 255, ref).astype(np.uint8)
        row = host[i].numpy() if host is not None else out[i].cpu().numpy()
        rows_ok += int(np.array_equal(row, ref))
    single_gteps = single_edges / (sum(single_ms) / 1e3) / 1e9
    st = runs[-1][1]
    # algorithmic bytes of a batch: every level writes its N x K-word plane, every
    # 64-bit frontier word a pull gathers is 8 B (counted on the device), the
    # output is N bytes per source
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
                     "kernels": "k_ms_bfs + k_ms_emit", "peak_kind": peak_kind, "algorithmic_bytes_per_batch": alg,
                     "traffic": ncu_traffic(args.batch_workload, "dram_bytes_per_batch"),
                     "traffic_note": "per batch; from the R-MAT scale 18 capture scaled x16 "
                                     "(profiles/k_ms_bfs_emit_rmat18_4096src.md)"},
        "parity": f"batched rows bit-exact to the oracle's levels (oracle/bfs_oracle.c orc_bfs_levels) on "
                  f"{rows_ok}/{len(check)} sampled sources",
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


def bench_bc_batch(args, torch, dev, g, sources, flush, arr=None):
    """Batched betweenness (bfs_bc_run_batch_device): 64 sources from one
    bit-sliced traversal and one path-count / dependency launch over all of
    them.  GTEPS = sum of m(s) / device time, L2 flushed before each batch;
    e2e through bfs_bc_accumulate over the same sources (centrality to host
    memory), against the per-source loop of bench_bc."""
    n = g.num_vertices
    srcs = np.asarray(sources[:64], np.uint32)
    k = int(srcs.size)
    stream = torch.cuda.Stream(device=dev)
    dep = torch.empty((k, n), dtype=torch.float32, device=dev)

    def one(i):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
        g.bc_batch_device(srcs, dep.data_ptr(), 0, stream.cuda_stream)
        st = g.bc_stats()
        if st["status"] != 0 or st["batched_sources"] != k:
            raise RuntimeError(f"batched betweenness status {st['status']}, batched {st['batched_sources']}")
        return st

    for i in range(max(1, args.warmup)):
        one(i)
    torch.cuda.synchronize()
    sts = [one(i) for i in range(args.steps)]
    dev_ms = statistics.mean(st["device_ms"] for st in sts)
    trav_ms = statistics.mean(st["traversal_ms"] for st in sts)
    kern_ms = statistics.mean(st["paths_ms"] + st["dependencies_ms"] for st in sts)
    st0 = sts[0]
    edges = st0["edges_reached"]
    reached_pairs = sum(st0["source_reached"])
    depth = st0["depth"]
    # algorithmic bytes of k_bc_batch: per edge read its neighbour id and the
    # neighbour's level word (12 B); per (edge, source) pair summed the
    # neighbour's value (4 B); per reached (vertex, source) pair the path count
    # written, read back and the dependency sum written (12 B); every level's
    # plane read twice (16 B per vertex and level)
    alg = (12 * (st0["edges_forward"] + st0["edges_reverse"]) + 4 * (st0["pairs_forward"] + st0["pairs_reverse"]) +
           12 * reached_pairs + 16 * n * (depth + 1))
    peak, _ = peaks()
    ach = alg / (kern_ms / 1e3) / 1e9 if kern_ms > 0 else 0.0
    traffic = ncu_traffic("pokec_bc_batch", "dram_bytes_per_launch")
    # e2e: centrality over the same sources to host memory
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cent, ast = g.betweenness(srcs)
    e2e_s = time.perf_counter() - t0
    out = {
        "what": "betweenness of 64 sources at once on the bit-sliced traversal (path counts + dependency sums for "
                "every (vertex, source) pair)",
        "sources": k, "steps": args.steps,
        "gteps": edges / (dev_ms / 1e3) / 1e9,
        "ms_per_batch": dev_ms, "ms_per_source": dev_ms / k,
        "traversal_ms": trav_ms, "kernel_ms": kern_ms, "output_ms": dev_ms - trav_ms - kern_ms,
        "phase_ms_mean": {x: statistics.mean(st[x] for st in sts) for x in ("paths_ms", "dependencies_ms")},
        "depth": depth,
        "edges_read": {"forward": st0["edges_forward"], "reverse": st0["edges_reverse"]},
        "edges_serving_a_source": st0["edges_matched_forward"],
        "edge_source_pairs": st0["pairs_forward"],
        "example_levels": {x: st0[x] for x in ("level_vertices", "level_paths_ms", "level_dependencies_ms")},
        "roofline": {"kernel": "k_bc_batch", "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak if peak else None, "algorithmic_bytes_per_launch": alg,
                     "traffic": traffic},
        "e2e": {"value": ast["edges_reached"] / e2e_s / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": 4 * k,
                "d2h_bytes_per_step": 4 * n, "note": "bfs_bc_accumulate(): 64 sources, centrality to host memory"},
        "gpu_launches": 3,
    }
    if arr is not None:
        from oracle import oracle as O
        d, p, _ = g.bc_batch(srcs[:8])
        ok = 0
        for i in (0, 7):
            osig, odep, _, oscale = O.bc_single(arr, int(srcs[i]))
            ok += int(np.array_equal(p[i], osig) and
                      bool((np.abs(d[i].astype(np.float64) - odep) <= 1e-4 * (np.abs(oscale) + 1)).all()))
        out["parity"] = (f"{ok}/2 sources of a batch: path counts bit-exact, dependencies within 1e-4 x (scale + 1) "
                         "of the oracle")
    return out


def bench_serving(args, torch, dev):
    """The serving loop: 8 resident R-MAT graphs (scales 14, 16, 18-23, edge
    factor 16) under a 40 GB HBM admission budget; open-loop Poisson arrivals
    of (graph, source) queries drawn uniformly, coalesced per graph into
    batches of up to 1024 sources; levels are computed and left on the device
    (BFS_DST_NONE) so that latency measures the traversal path.  Then a burst
    of queries whose levels are delivered to host memory (BFS_DST_HOST), with
    a sample of them checked against the oracle."""
    import bfs_simd_benchmarks_gb300 as B
    t0 = time.perf_counter()
    graphs, edges = [], []
    for wl in workloads.serve_graphs():
        src, dst = wl.edges()
        graphs.append((wl, B.Graph.from_edges(wl.n, src, dst, wl.w, wl.s, device_build=wl.m >= DEVICE_BUILD_EDGES)))
        edges.append((src, dst))
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
                          # wall = the arrival window + the drain of the batches in flight at its end
                          "arrival_window_s": float(arr[-1]) / 1e9,
                          "drain_ms": max(0.0, wall - float(arr[-1]) / 1e9) * 1e3,
                          "slots_in_flight_mean": st["device_ms"] / 1e3 / wall})
    host = serve_host_check(srv, graphs, edges, pools)
    res = {"graphs": [{"workload": wl.name, "vertices": wl.n, "edges": wl.m} for wl, _ in graphs],
           "budget_bytes": 40 * 10**9, "admitted_bytes": srv.stats()["device_bytes"], "graph_build_s": round(build_s, 1),
           "max_batch": 1024, "slots": 3, "results": "rates: left on the device (BFS_DST_NONE); host_delivery: "
                                                      "uint8 levels copied to host memory (BFS_DST_HOST)",
           "latency": "submit -> traversal and output pass complete (rates) / levels in host memory (host_delivery), "
                      "host clock", "rates": rates, "host_delivery": host,
           "clocks": clk.summary()}
    srv.close()
    for _, g in graphs:
        g.close()
    torch.cuda.empty_cache()
    return res


def bench_large(args, torch, dev):
    """The large single-GPU configuration (Twitter shape: 41,652,230 vertices,
    1,468,365,182 edges, permuted ids, W=1024, S=16): the edge list drawn on
    the GPU (the host generator's list, element for element), the layout built
    on the GPU from the device arrays, then `large_sources` single-source
    traversals and one `large_batch`-source batched traversal, timed with CUDA
    events, L2 flushed before each.  Parity at full size: the BFS-level
    certificate of the oracle (oracle/bfs_oracle.c orc_check_levels: every
    edge and vertex checked against the levels) for 2 single-source results
    and 2 batched rows."""
    import bfs_simd_benchmarks_gb300 as B
    from oracle import oracle as O
    wl = workloads.get(args.large)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ds, dd = B.gen_rmat_device(wl.n, wl.m, wl.a, wl.b, wl.c, seed=wl.seed, permute=wl.permute)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    g = B.Graph.from_device_edges(wl.n, ds.data_ptr(), dd.data_ptr(), wl.m, wl.w, wl.s)
    build_s = time.perf_counter() - t0
    hs = ds.cpu().numpy().view(np.uint32)
    hd = dd.cpu().numpy().view(np.uint32)
    del ds, dd
    torch.cuda.empty_cache()
    deg = g.degrees()
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    lev = torch.empty(wl.n, dtype=torch.int32, device=dev)
    par = torch.empty(wl.n, dtype=torch.int32, device=dev)
    sources = wl.sources(deg, args.large_sources)

    def single(s):
        with torch.cuda.stream(stream):
            flush.fill_(int(s) & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.run_device(int(s), lev.data_ptr(), par.data_ptr(), stream.cuda_stream)
            e1.record(stream)
        st = g.last_stats()
        if st["status"] != 0:
            raise RuntimeError(f"large graph: traversal status {st['status']}")
        return e0.elapsed_time(e1), st

    for s in sources[:2]:
        single(s)
    runs = [single(s) for s in sources]
    s_ms = sum(r[0] for r in runs)
    s_edges = sum(r[1]["edges_traversed"] for r in runs)
    checks, ok = 0, 0
    for s in sources[:2]:
        single(s)
        checks += 1
        ok += int(O.check_levels(wl.n, hs, hd, int(s), lev.cpu().numpy()) == 0)
    # the batched traversal
    g.set_options(batch_budget_mb=args.large_budget_mb)
    bsrc = wl.sources(deg, args.large_batch)
    out = torch.empty((len(bsrc), wl.n), dtype=torch.uint8, device=dev)
    bruns = []
    for i in range(3):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.run_batch_device(bsrc, out.data_ptr(), stream.cuda_stream)
            e1.record(stream)
        st = g.last_batch_stats()
        if st["status"] != 0:
            raise RuntimeError(f"large graph: batched status {st['status']}")
        if i >= 1:
            bruns.append((e0.elapsed_time(e1), st))
    b_ms = statistics.mean(r[0] for r in bruns)
    b_edges = bruns[0][1]["edges_traversed"]
    for i in (0, len(bsrc) - 1):
        row = out[i].cpu().numpy()
        checks += 1
        ok += int(O.check_levels(wl.n, hs, hd, int(bsrc[i]), np.where(row == 255, -1, row.astype(np.int32))) == 0)
    single_gteps = s_edges / (s_ms / 1e3) / 1e9
    batch_gteps = b_edges / (b_ms / 1e3) / 1e9
    st = bruns[-1][1]
    res = {"workload": wl.describe() | {"sources": len(sources), "batch_sources": len(bsrc)},
           "generate_s": round(gen_s, 2), "generator": "bfs_gen_rmat_device (the host generator's edge list)",
           "graph_build_s": round(build_s, 2),
           "single_source": {"gteps": single_gteps, "ms_per_traversal_mean": s_ms / len(runs),
                             "edges_per_traversal_mean": s_edges / len(runs), "sources": len(runs)},
           "batched": {"gteps": batch_gteps, "ms_per_batch_mean": b_ms, "levels_ms": st["levels_ms"],
                       "output_ms": st["output_ms"], "depth": st["depth"], "planes": st["planes"],
                       "spills": st["spills"], "words_per_vertex": st["words_per_vertex"],
                       "output_bytes": len(bsrc) * wl.n, "steps": len(bruns)},
           "speedup_batched_vs_single_source": batch_gteps / single_gteps,
           "parity": f"{ok}/{checks} level vectors (2 single-source, 2 batched rows) pass the oracle's BFS-level "
                     "certificate over all edges and vertices (oracle/bfs_oracle.c orc_check_levels)",
           "l2": "flushed (256 MiB write) before every traversal and batch"}
    del out
    g.close()
    torch.cuda.empty_cache()
    return res


def serve_host_check(srv, graphs, edges, pools, count: int = 256, per_graph: int = 2):
    """A burst of `count` queries over all graphs with levels delivered to
    host memory; `per_graph` results of every graph compared with the oracle."""
    from oracle import oracle as O
    rng = np.random.default_rng(99)
    gids = rng.integers(0, len(graphs), count)
    picks = rng.integers(0, 4096, count)
    outs = [np.empty(graphs[gi][0].n, np.uint8) for gi in gids]
    srv.reset_stats()
    t0 = time.perf_counter()
    tickets = [srv.submit_host(int(gi), int(pools[gi][k]), outs[i]) for i, (gi, k) in enumerate(zip(gids, picks))]
    lat = [srv.wait(t)["latency_ms"] for t in tickets]
    wall = time.perf_counter() - t0
    st = srv.stats()
    ok = checked = 0
    for gi, (wl, _) in enumerate(graphs):
        idx = [i for i in range(count) if gids[i] == gi][:per_graph]
        if not idx:
            continue
        oarr = O.csr_arrays(wl.n, *edges[gi])
        for i in idx:
            ref = O.bfs_levels(oarr, int(pools[gi][picks[i]]))
            ok += int(np.array_equal(outs[i], np.where(ref < 0, 255, ref).astype(np.uint8)))
            checked += 1
        del oarr
    return {"queries": count, "submitted": "as one burst from the host thread", "wall_s": wall,
            "achieved_qps": count / wall, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_batch": st["mean_batch"],
            "d2h_bytes": int(sum(o.nbytes for o in outs)),
            "parity": f"{ok}/{checked} sampled results bit-exact to the oracle's levels "
                      f"(oracle/bfs_oracle.c orc_bfs_levels), {per_graph} per graph"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    wl = workloads.get(args.workload)
    cpu, cpu_levels = None, {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, cpu_levels = cpu_leg(args, wl)  # before torch and CUDA are touched
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import bfs_simd_benchmarks_gb300 as B
    from bfs_simd_benchmarks_gb300 import _native as N
    B.load_library(build_if_missing=True)
    t_gen = time.perf_counter()
    src, dst = wl.edges()
    t_gen = time.perf_counter() - t_gen
    degrees = np.bincount(src, minlength=wl.n).astype(np.uint32)  # out-degrees, as Graph.degrees()
    sources = wl.sources(degrees)
    if args.sources:
        sources = sources[: args.sources]
    n = wl.n
    # layout search (bfs_autotune): tile width over the tile-size computer's
    # range x stripe length {8, 16, 32} x {caller ids, degree order}, each
    # layout built on the GPU and its options tuned on 16 of the sources
    W, S, degree_order, shape_tune = args.tile_width or wl.w, args.stripe_length or wl.s, args.degree_order, None
    shape_opts = json.loads(args.options) if args.options else None
    if not args.no_tune and not args.no_shape_search and args.mode == "persistent":
        t_t = time.perf_counter()
        r = B.autotune(wl.n, src, dst, sources[:16], tile_widths=None, stripe_lengths=(8, 16, 32),
                       device_build=True, layouts=True)
        W, S = r["tile_width"], r["stripe_length"]
        degree_order = r["load_flags"] == N.BFS_LOAD_DEGREE_ORDER
        shape_opts = {k: v for k, v in r["options"].items() if k not in ("wait_limit_us", "test_hold_barrier")}
        best = {}
        for t in r["trials"]:
            key = (t["tile_width"], t["stripe_length"], "degree order" if t["load_flags"] else "caller ids")
            best[key] = max(best.get(key, 0.0), t["gteps"])
        shape_tune = {"tile_width": W, "stripe_length": S,
                      "layout": "degree order" if degree_order else "caller ids",
                      "threads_per_cta": 512,  # the kernels' compile-time block size
                      "ctas_per_sm": shape_opts["ctas_per_sm"] or "max (2)",
                      "gteps_kernel_16_sources": r["single_gteps"],
                      "layouts_tried": [{"tile_width": k[0], "stripe_length": k[1], "layout": k[2], "best_gteps": v}
                                        for k, v in sorted(best.items())],
                      "seconds": round(time.perf_counter() - t_t, 2)}
    t_b = time.perf_counter()
    g = B.Graph.from_edges(wl.n, src, dst, W, S, device_build=True, degree_order=degree_order)
    if shape_opts:
        g.set_options(**shape_opts)
    g.set_options(mode=args.mode, **({"bottom_up": args.bottom_up} if args.bottom_up else {}))
    info = g.info()
    t_gen += time.perf_counter() - t_b
    sw = S * W
    tuned = None
    if not args.no_tune and args.mode == "persistent":
        t_t = time.perf_counter()
        r = g.tune(sources, single=True)
        tuned = {"options": {k: r["options"][k] for k in ("bottom_up", "to_dense_ratio", "to_sparse_ratio",
                                                           "warp_max_degree", "cta_max_degree", "switch_rule",
                                                           "bu_alpha", "td_beta", "ctas_per_sm")},
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
    pull = g.get_options()["bottom_up"] == N.BFS_BU_PULL
    alg = [algorithmic_bytes(st, n, sw, pull) for _, _, st in timed]
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

    # both bottom-up variants on the same graph and options: one pass over the sources each
    # (the streamed one is the reference's dense step: packed tiles through bulk copies)
    variants = {}
    base_bu = g.get_options()["bottom_up"]
    for name, bu in (("pull", N.BFS_BU_PULL), ("stream", N.BFS_BU_STREAM)):
        try:
            g.set_options(bottom_up=bu)
            for s in sources[:4]:
                traverse(int(s), None)
            tv = []
            for s in sources:
                traverse(int(s), tv)
        except N.BfsError as e:
            variants[name] = {"error": str(e)}
            continue
        vms = sum(a.elapsed_time(b) for a, b, _ in tv)
        variants[name] = {"gteps": sum(st["edges_traversed"] for _, _, st in tv) / (vms / 1e3) / 1e9,
                          "ms_per_traversal": vms / len(tv),
                          "dense_steps_mean": statistics.mean(st["dense_steps"] for _, _, st in tv),
                          "dense_ms_mean": statistics.mean(st["dense_ms"] for _, _, st in tv)}
    g.set_options(bottom_up=base_bu)

    batched = None
    if args.batch_workload != "none" and world == 1:
        same = args.batch_workload == args.workload
        batched = bench_batched(args, torch, dev, g if same else None, t_gen if same else 0.0,
                                (src, dst) if same else None)
    serving = None
    if args.serve != "none" and world == 1:
        serving = bench_serving(args, torch, dev)

    parity = None
    if cpu_levels:
        ok = 0
        for s, ref in cpu_levels.items():
            got, _, _ = g.run(s, parents=False)
            ok += int(np.array_equal(got, ref))
        parity = f"levels bit-exact on {ok}/{len(cpu_levels)} sources checked against the oracle"
    large = None
    bc = None
    if args.bc_sources > 0 and world == 1:
        bc_arr = None
        if not args.no_cpu_baseline:
            from oracle import oracle as O
            bc_arr = O.csr_arrays(wl.n, src, dst)
        # betweenness runs on the caller's ids (a degree-ordered layout refuses it)
        bc_g = B.Graph.from_edges(wl.n, src, dst, W, S, device_build=True) if degree_order else g
        bc = bench_bc(args, torch, dev, bc_g, sources, flush, bc_arr)
        bc["batched"] = bench_bc_batch(args, torch, dev, bc_g, sources, flush, bc_arr)
        if bc_g is not g:
            bc_g.close()
    if args.large != "none" and world == 1:
        large = bench_large(args, torch, dev)
    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": METRIC,
            "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded R-MAT stand-in, see config)",
            "config": bench_config(wl, len(sources)),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "gpu_config": {"mode": args.mode, "bottom_up": "pull" if pull else "stream",
                           "tile_width": W, "stripe_length": S, "layout": "degree order" if degree_order else "caller ids",
                           "layout_search": shape_tune,
                           "graph_device_bytes": info["device_bytes"], "grid_ctas": timed[0][2]["grid_ctas"],
                           "column_groups": info["num_groups"], "autotune": tuned,
                           "bottom_up_variants": variants,
                           "graph_build_s": round(t_gen, 2)},
            "single_source": {"gteps": value, "ms_per_traversal_mean": statistics.mean(trav_ms),
                              "ms_per_traversal_p50": statistics.median(trav_ms),
                              "ms_per_traversal_p99": float(np.percentile(trav_ms, 99)),
                              "edges_per_traversal_mean": edges / len(timed),
                              "dense_steps_mean": statistics.mean(st["dense_steps"] for _, _, st in timed),
                              "steps_mean": statistics.mean(st["num_steps"] for _, _, st in timed),
                              "phase_ms_mean": {k: statistics.mean(st[k] for _, _, st in timed)
                                                for k in ("dense_ms", "to_dense_ms", "sparse_ms", "to_sparse_ms")},
                              "example_steps": {k: timed[0][2][k] for k in ("trace", "step_ms", "step_work_min_ms",
                                                                               "step_work_max_ms")},
                              "init_ms_mean": statistics.mean(st["device_ms"] - st["kernel_ms"] for _, _, st in timed),
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
            # per timed traversal: k_bfs_persistent, and k_unrelabel on a degree-ordered layout
            # (the L2 flush before it is torch's fill kernel, not counted)
            "gpu_launches": (2 if degree_order else 1) * len(timed),
            "clocks": clocks,
            "cpu_baseline": cpu,
            "parity": parity,
            "batched": batched,
            "serving": serving,
            "betweenness": bc,
            "large": large,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    g.close()


if __name__ == "__main__":
    main()

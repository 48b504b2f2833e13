"""The N > 1 path of bench.py on CPU: replicas only (no data-path
collective), aggregated as max time over ranks and the sum of traversed
edges; the reference arm runs on rank 0 alone.  world_size 2, gloo."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, edges = bench.aggregate_replicas(torch, 10.0 * (rank + 1), 1000 + rank, torch.device("cpu"), world)
        q.put((rank, ms, edges))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for _, ms, edges in got:
        assert ms == 20.0 and edges == 2001.0


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


@pytest.mark.timeout(600)
def test_reference_arm_line_on_rank0():
    """The reference arm on the CPU-runnable scale-16 workload prints one JSON line."""
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "rmat16", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["host"]["isa"] and line["cpu_baseline"]["host"]["nproc"] >= 1
    # the same config object as the GPU arm's line
    sys.path.insert(0, ROOT)
    import bench
    from bfs_simd_benchmarks_gb300 import workloads
    assert line["config"] == bench.bench_config(workloads.get("rmat16"), 1)


@pytest.mark.timeout(600)
def test_reference_arm_loads_no_product_library():
    """The reference arm maps the checker's library only, never libbfs_gb300.so."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'rmat16', "
            "'--steps', '1', '--warmup', '0']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPS', int('libbfs_gb300' in maps), int('liboracle.so' in maps))")
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().splitlines()[-1] == "MAPS 0 1"

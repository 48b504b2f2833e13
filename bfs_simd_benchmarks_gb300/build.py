"""Build recipe of libbfs_gb300.so and the `bfs` CLI (in-tree, sm_103a only).

Every translation unit goes through nvcc with one -gencode
(arch=compute_103a,code=sm_103a); they compile in parallel and link into
bfs_simd_benchmarks_gb300/_lib/.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIB_DIR, "libbfs_gb300.so")
CLI = os.path.join(LIB_DIR, "bfs")

SOURCES = ["api.cu", "bfs_kernels.cu", "bfs_noalloc.cu", "msbfs.cu", "bc.cu", "bc_batch.cu", "build_device.cu", "rmat_device.cu", "server.cpp", "autotune.cpp", "host_io.cpp", "layout.cpp", "rmat.cpp"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libbfs_gb300.so")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles the library and the CLI if any source is newer; returns the .so path."""
    nvcc = _nvcc()
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "bfs_gb300.h"))
    objs = []
    jobs = []
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3", "-Xcompiler", "-pthread"]
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(LIB_DIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            jobs.append([nvcc] + GENCODE + common + ["-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if force or _stale(LIB, objs):
        _run([nvcc] + GENCODE + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-pthread"])
    cli_src = os.path.join(CSRC, "cli_bfs.cpp")
    if force or _stale(CLI, [cli_src, LIB]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", cli_src, "-o", CLI, "-L" + LIB_DIR, "-lbfs_gb300",
              "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)

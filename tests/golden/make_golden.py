"""Generates the golden fixtures in tests/golden/ by running the REFERENCE itself.

Runs only where the reference sources are present (they are compiled in place
into oracle/_ref by `make -C oracle ref`).  For every case it

  1. writes the edge list (1-indexed "N M" format, README.md:19-24) with the
     labels of vertex 0 and the chosen source swapped, because the reference
     always starts from vertex 0 (apps/bfs_simd/bfs.cpp:1159);
  2. runs the reference's tools/csr_tiling, tools/coo_tiling and
     tools/column_major_tile on it under the "<g>_reorder" name that
     apps/bfs_simd reads (bfs.cpp:983);
  3. runs apps/bfs_simd built with -DONEDEBUG, which writes path/path<t>.txt
     (bfs.cpp:927-954), and un-swaps the levels;
  4. records sha256 digests of every tool output file, and of the
     tools/vertex_id_remap output for the unswapped graph.

The fixtures keep the edge lists of small cases and, for the scale-16 case,
only the generator parameters plus a digest of the edge list.

    BFS_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
import bfs_simd_benchmarks_gb300 as B  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("BFS_REFERENCE_DIR", "")  # the reference checkout; no default path


def sha_files(paths: list[str]) -> str:
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def family(prefix: str) -> list[str]:
    return [f"{prefix}-{t}" for t in range(64)]


def edges_digest(src, dst) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(src, dtype="<u4").tobytes())
    h.update(np.ascontiguousarray(dst, dtype="<u4").tobytes())
    return h.hexdigest()


def run(cmd, cwd=None):
    subprocess.run(cmd, cwd=cwd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def reference_levels(work: str, n: int, src, dst, w: int, s: int, source: int, weighted_csr: bool = False):
    """Levels from the reference's own pipeline and bfs_simd, source relabelled to 0."""
    perm = np.arange(n, dtype=np.uint32)
    perm[0], perm[source] = source, 0
    ps, pd = perm[src], perm[dst]
    g = os.path.join(work, "g")
    reo = g + "_reorder"
    O.write_edge_list(reo, n, ps, pd)
    run([O.reference_binary("csr_tiling"), reo])
    run([O.reference_binary("coo_tiling"), reo, str(w), str(w)])
    run([O.reference_binary("column_major_tile"), reo, str(w), str(s), str(s)])
    digests = {
        "untiled": sha_files(family(reo + "_untiled") + [reo + "_untiled-nneibor"]),
        "coo": sha_files(family(f"{reo}_coo-tiled-{w}") + [f"{reo}_coo-tiled-{w}-offsets", f"{reo}_coo-tiled-{w}-nneibor"]),
        "col": sha_files(family(f"{reo}_col-{s}-coo-tiled-{w}") + [f"{reo}_col-{s}-coo-tiled-{w}-offsets",
                                                                     f"{reo}_col-{s}-coo-tiled-{w}-nneibor"]),
    }
    pathdir = os.path.join(work, "path")
    os.makedirs(pathdir, exist_ok=True)
    run([O.reference_binary("bfs_simd_debug"), g, str(w), str(s)], cwd=work)
    lev_relabelled = O.read_path_dump(pathdir, n)
    levels = lev_relabelled[perm]  # level of old vertex v = level of its new label perm[v]
    shutil.rmtree(pathdir)
    for f in os.listdir(work):
        os.remove(os.path.join(work, f))
    return levels.astype(np.int32), digests


def case_files(work: str, n: int, src, dst, w: int, s: int) -> dict:
    """Reference tool digests for the unswapped graph (and vertex_id_remap)."""
    g = os.path.join(work, "h")
    O.write_edge_list(g, n, src, dst)
    run([O.reference_binary("csr_tiling"), g])
    run([O.reference_binary("coo_tiling"), g, str(w), str(w)])
    run([O.reference_binary("column_major_tile"), g, str(w), str(s), str(s)])
    run([O.reference_binary("vertex_id_remap"), g], cwd=work)
    d = {
        "untiled": sha_files(family(g + "_untiled") + [g + "_untiled-nneibor"]),
        "coo": sha_files(family(f"{g}_coo-tiled-{w}") + [f"{g}_coo-tiled-{w}-offsets", f"{g}_coo-tiled-{w}-nneibor"]),
        "col": sha_files(family(f"{g}_col-{s}-coo-tiled-{w}") + [f"{g}_col-{s}-coo-tiled-{w}-offsets",
                                                               f"{g}_col-{s}-coo-tiled-{w}-nneibor"]),
        "reorder": sha_files([g + "_reorder"]),
    }
    for f in os.listdir(work):
        p = os.path.join(work, f)
        if os.path.isfile(p):
            os.remove(p)
    return d


def weighted_digest(work: str, n: int, src, dst, wts) -> str:
    g = os.path.join(work, "wg")
    O.write_edge_list(g, n, src, dst, wts)
    run([O.reference_binary("csr_tiling_weighted"), g])
    d = sha_files(family(g + "_untiled") + [g + "_untiled-nneibor"])
    for f in os.listdir(work):
        os.remove(os.path.join(work, f))
    return d


def cases():
    rng = np.random.default_rng(20261203)
    out = []
    # 1: scale-10 R-MAT, tail stripe (SIDE 16, S 3)
    s, d = B.gen_rmat(1024, 16384, seed=101)
    out.append(dict(name="rmat10_w64_s3", n=1024, src=s, dst=d, w=64, s=3, store_edges=True))
    # 2: scale-12 R-MAT with permuted ids, W not a power of two and N % W != 0
    s, d = B.gen_rmat(4096, 32768, seed=202, permute=True)
    out.append(dict(name="rmat12p_w100_s5", n=4096, src=s, dst=d, w=100, s=5, store_edges=True))
    # 3: tiny graph with duplicate edges and self loops (the tools keep both)
    n = 37
    src = rng.integers(0, n, 150).astype(np.uint32)
    dst = rng.integers(0, n, 150).astype(np.uint32)
    src = np.concatenate([src, [3, 3, 5, 5, 5]]).astype(np.uint32)
    dst = np.concatenate([dst, [3, 9, 5, 7, 7]]).astype(np.uint32)
    out.append(dict(name="tiny_dups_w8_s2", n=n, src=src, dst=dst, w=8, s=2, store_edges=True))
    # 4: long chain plus shortcuts (many top-down steps)
    n = 300
    src = np.concatenate([np.arange(n - 1), rng.integers(0, n, 40)]).astype(np.uint32)
    dst = np.concatenate([np.arange(1, n), rng.integers(0, n, 40)]).astype(np.uint32)
    out.append(dict(name="chain300_w32_s4", n=n, src=src, dst=dst, w=32, s=4, store_edges=True))
    # 5: fewer than 64 edges and fewer than 20 (threshold E/20 == 0)
    n = 50
    src = rng.integers(0, n, 15).astype(np.uint32)
    dst = rng.integers(0, n, 15).astype(np.uint32)
    out.append(dict(name="sparse15_w16_s2", n=n, src=src, dst=dst, w=16, s=2, store_edges=True))
    # 6: the scale-16, edge factor 16 R-MAT at W=1024, S=16 (only parameters + digest stored)
    s, d = B.gen_rmat(65536, 1048576, seed=16)
    out.append(dict(name="rmat16_w1024_s16", n=65536, src=s, dst=d, w=1024, s=16, store_edges=False,
                    gen=dict(num_vertices=65536, num_edges=1048576, a=0.57, b=0.19, c=0.19, seed=16,
                             dedup=True, no_self_loops=True, permute=False)))
    return out


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "apps", "bfs_simd")):
        sys.exit("set BFS_REFERENCE_DIR to the reference checkout: the golden fixtures can only be regenerated "
                 "where its sources are")
    O.build(with_reference=True)
    summary = {}
    with tempfile.TemporaryDirectory() as work:
        for c in cases():
            n, src, dst, w, s = c["n"], c["src"], c["dst"], c["w"], c["s"]
            deg = np.bincount(src, minlength=n)
            rng = np.random.default_rng(zlib.crc32(c["name"].encode()))
            cand = np.flatnonzero(deg > 0)
            sources = [0] + sorted(set(int(x) for x in rng.choice(cand, size=min(3, cand.size), replace=False)))
            levels, swapped_digests = [], []
            for sv in sources:
                lv, dg = reference_levels(work, n, src, dst, w, s, sv)
                levels.append(lv)
                swapped_digests.append(dg)
            files = case_files(work, n, src, dst, w, s)
            rec = dict(n=n, w=w, s=s, m=int(len(src)), sources=np.array(sources, dtype=np.uint32),
                       levels=np.stack(levels).astype(np.int32),
                       edges_sha256=edges_digest(src, dst))
            if c["store_edges"]:
                rec["src"] = np.asarray(src, dtype=np.uint32)
                rec["dst"] = np.asarray(dst, dtype=np.uint32)
            np.savez_compressed(os.path.join(OUT, c["name"] + ".npz"), **rec)
            summary[c["name"]] = dict(n=n, m=int(len(src)), w=w, s=s, sources=sources, files=files,
                                      swapped_files=swapped_digests, edges_sha256=rec["edges_sha256"],
                                      gen=c.get("gen"), level_histograms=[
                                          {int(k): int(v) for k, v in zip(*np.unique(l, return_counts=True))}
                                          for l in levels])
            print(c["name"], "sources", sources, "max level", [int(l.max()) for l in levels])
        # weighted csr_tiling digest (3-column files)
        rng = np.random.default_rng(7)
        n = 200
        src = rng.integers(0, n, 900).astype(np.uint32)
        dst = rng.integers(0, n, 900).astype(np.uint32)
        wts = rng.integers(1, 100, 900).astype(np.uint32)
        summary["weighted_csr"] = dict(n=n, digest=weighted_digest(work, n, src, dst, wts))
        np.savez_compressed(os.path.join(OUT, "weighted_csr.npz"), n=n, src=src, dst=dst, wts=wts)
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(summary, f, indent=1, sort_keys=True)
    print("wrote", OUT)


if __name__ == "__main__":
    main()

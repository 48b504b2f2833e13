"""Shared test setup: the `gpu` marker, library builds and golden fixtures."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def native():
    """libbfs_gb300.so, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    from bfs_simd_benchmarks_gb300 import _native, build
    build.build()
    return _native.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build(with_reference=False)
    O.lib()
    return O


@pytest.fixture(scope="session")
def golden_summary():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def golden_case_names():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return sorted(k for k in json.load(f) if k != "weighted_csr")


def load_case(name: str) -> dict:
    """A golden case with its edge list (regenerated and digest-checked when not stored)."""
    import hashlib
    z = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)[name]
    if "src" not in z:
        from bfs_simd_benchmarks_gb300 import gen_rmat
        g = meta["gen"]
        z["src"], z["dst"] = gen_rmat(g["num_vertices"], g["num_edges"], g["a"], g["b"], g["c"], seed=g["seed"],
                                      dedup=g["dedup"], no_self_loops=g["no_self_loops"], permute=g["permute"])
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(z["src"], dtype="<u4").tobytes())
    h.update(np.ascontiguousarray(z["dst"], dtype="<u4").tobytes())
    assert h.hexdigest() == meta["edges_sha256"], f"edge list of {name} differs from the fixture"
    z["meta"] = meta
    z["n"] = int(z["n"])
    z["w"] = int(z["w"])
    z["s"] = int(z["s"])
    return z


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


BC_RTOL = 1e-4  # float dependencies vs a double or differently ordered float evaluation


def bc_case_names():
    z = np.load(os.path.join(GOLDEN, "bc_networkx.npz"))
    return [str(x) for x in z["names"]]


def load_bc_case(name: str) -> dict:
    """A graph of the networkx betweenness fixtures with its edge list."""
    z = np.load(os.path.join(GOLDEN, "bc_networkx.npz"))
    out = {"n": int(z[name + "__n"]), "sources": z[name + "__sources"], "delta": z[name + "__delta"],
           "bc": z[name + "__bc"] if name + "__bc" in z.files else None}
    if name.startswith("hand_"):
        out["src"], out["dst"] = z[name + "__src"], z[name + "__dst"]
        out["w"], out["s"] = 4, 2
    else:
        c = load_case(name)
        out["src"], out["dst"], out["w"], out["s"] = c["src"], c["dst"], c["w"], c["s"]
    return out


def bc_close(got, want, scale, rtol: float = BC_RTOL) -> np.ndarray:
    """Mask of dependencies within rtol of the error scale of their float sums."""
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return np.abs(got - want) <= rtol * (np.abs(scale) + 1.0)

"""Golden outputs of the reference's tools/tile-size-computer for a set of
(N, E) pairs, from its own binary compiled from source (oracle/Makefile,
target `ref`).  Writes tests/golden/tile_size.json; run where the reference
sources are present:  python tests/golden/make_tile_size_golden.py
"""
import json
import os
import re
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

PAIRS = [(1 << 16, 1 << 20), (1_632_803, 30_622_564), (1 << 22, 1 << 26), (41_652_230, 1_468_365_182),
         (1 << 14, 1 << 18), (1 << 20, 1 << 24), (1 << 23, 1 << 27), (1000, 8000), (100_000, 1_000_000),
         (3_000_000, 117_000_000), (65_536, 655_360), (12_345, 98_765)]


def main():
    from oracle import oracle as O
    O.build(with_reference=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "tile-size-computer")
    out = []
    for n, m in PAIRS:
        r = subprocess.run([exe, str(n), str(m)], capture_output=True, text=True, check=True)
        lo, hi = map(int, re.match(r"min_tile_size: (\d+), max_tile_size: (\d+)", r.stdout).groups())
        out.append({"vertices": n, "edges": m, "min_tile_size": lo, "max_tile_size": hi, "stdout": r.stdout})
    with open(os.path.join(ROOT, "tests", "golden", "tile_size.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()

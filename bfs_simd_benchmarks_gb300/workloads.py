"""The synthetic workloads that stand in for the reference's datasets.

The reference downloads KONECT graphs (README.md:15-24); none are available
here, so seeded R-MAT graphs with the same vertex and edge counts and a
power-law degree skew stand in for them.  Edge counts are exact: candidates
are drawn until exactly E edges survive self-loop and duplicate removal.

  rmat16  : scale 16, 1,048,576 edges, W=1024, S=16 (the reference's CPU case)
  pokec   : 1,632,803 vertices, 30,622,564 edges, permuted ids, W=1024, S=16,
            64 seeded sources (the Pokec shape, tools/galois_data/rmat24.sh:7)
  rmat18  : scale 18, 4,194,304 edges, 4096 sources (batched; profiling size)
  rmat22  : scale 22, 67,108,864 edges, 4096 sources (batched)
  twitter : 41,652,230 vertices, 1,468,365,182 edges, permuted ids, W=1024, S=16
            (the Twitter shape, tools/galois_data/rmat24.sh:19)
  serve   : eight R-MAT graphs of scales 14,16,18,19,20,21,22,23, edge factor 16
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Workload:
    name: str
    n: int
    m: int
    w: int
    s: int
    num_sources: int
    permute: bool
    graph_id: int
    a: float = 0.57
    b: float = 0.19
    c: float = 0.19

    @property
    def seed(self) -> int:
        return self.graph_id * 1000 + 1

    def edges(self):
        from .graph import gen_rmat
        return gen_rmat(self.n, self.m, self.a, self.b, self.c, seed=self.seed, permute=self.permute)

    def sources(self, degrees, count: int | None = None) -> np.ndarray:
        from .graph import pick_sources
        return pick_sources(degrees, count or self.num_sources, seed=self.graph_id * 1000 + 7)

    def describe(self) -> dict:
        return {"workload": self.name, "vertices": self.n, "edges": self.m, "tile_width": self.w,
                "stripe_length": self.s, "sources": self.num_sources, "rmat": [self.a, self.b, self.c],
                "permuted_ids": self.permute, "seed": self.seed}


_WORKLOADS = {
    "rmat16": Workload("rmat16", 1 << 16, 1 << 20, 1024, 16, 1, False, 16),
    "pokec": Workload("pokec", 1_632_803, 30_622_564, 1024, 16, 64, True, 2),
    "rmat18": Workload("rmat18", 1 << 18, 1 << 22, 1024, 16, 4096, False, 18),
    "rmat22": Workload("rmat22", 1 << 22, 1 << 26, 1024, 16, 4096, False, 22),
    "twitter": Workload("twitter", 41_652_230, 1_468_365_182, 1024, 16, 16, True, 5),
}

SERVE_SCALES = (14, 16, 18, 19, 20, 21, 22, 23)


def get(name: str) -> Workload:
    return _WORKLOADS[name]


def serve_graphs() -> list[Workload]:
    return [Workload(f"serve_s{sc}", 1 << sc, 16 << sc, 1024, 16, 1, False, 100 + sc) for sc in SERVE_SCALES]

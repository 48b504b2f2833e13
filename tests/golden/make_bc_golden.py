"""Generates tests/golden/bc_networkx.npz: betweenness dependencies computed by
networkx (Brandes' algorithm, a published third-party implementation) on the
golden graphs.

The reference's BC program (apps/betweennessCentrality_simd/bc.cpp) prints
only timings and keeps its dependency array internal, so its values cannot be
captured by running it; these fixtures pin the oracle's restatement of its
algorithm to an independent implementation instead.

For every graph without duplicate edges (networkx collapses them) and for
each of the case's sources s it stores delta_s(v) =
sum_t sigma_st(v) / sigma_st over targets t (betweenness_centrality_subset
with sources [s], all targets, unnormalised; v = s is left out), and for
graphs of at most 1024 vertices the full unnormalised betweenness over all
sources.  Also stores two hand-made graphs (unreachable parts, a self-loop,
parallel shortest paths).

    python tests/golden/make_bc_golden.py        (needs networkx; runs here only)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from conftest import golden_case_names, load_case  # noqa: E402

CASES = ["chain300_w32_s4", "rmat10_w64_s3", "rmat12p_w100_s5", "sparse15_w16_s2"]


def handmade():
    # diamond 0->{1,2}->3->4, a second diamond behind it, vertices 8..9 unreachable
    # from 0 (9 -> 0 only), a self-loop on 3, a dead end 7
    src = [0, 0, 1, 2, 3, 3, 4, 4, 5, 6, 3, 9, 8, 2, 1]
    dst = [1, 2, 3, 3, 4, 3, 5, 6, 7, 7, 7, 0, 9, 4, 4]
    yield "hand_diamond", 10, np.array(src, np.uint32), np.array(dst, np.uint32), np.array([0, 3, 9, 8], np.uint32)
    # a 6 x 6 grid with right/down edges: binomial path counts
    s, d = [], []
    for r in range(6):
        for c in range(6):
            v = r * 6 + c
            if c < 5:
                s.append(v); d.append(v + 1)
            if r < 5:
                s.append(v); d.append(v + 6)
    yield "hand_grid6", 36, np.array(s, np.uint32), np.array(d, np.uint32), np.array([0, 7, 14, 35], np.uint32)


def main() -> None:
    import networkx as nx
    from networkx.algorithms.centrality import betweenness_centrality_subset

    out = {}
    graphs = []
    for name in CASES:
        c = load_case(name)
        graphs.append((name, c["n"], np.asarray(c["src"], np.uint32), np.asarray(c["dst"], np.uint32),
                       np.asarray(c["sources"], np.uint32)))
    graphs.extend(handmade())
    names = []
    for name, n, src, dst, sources in graphs:
        pairs = set(zip(src.tolist(), dst.tolist()))
        assert len(pairs) == len(src), f"{name} has duplicate edges"
        G = nx.DiGraph()
        G.add_nodes_from(range(n))
        G.add_edges_from(pairs)
        delta = np.zeros((len(sources), n), np.float64)
        for i, s in enumerate(sources.tolist()):
            b = betweenness_centrality_subset(G, [s], list(range(n)), normalized=False)
            delta[i] = [b[v] for v in range(n)]
        out[name + "__delta"] = delta
        out[name + "__sources"] = sources
        out[name + "__n"] = np.int64(n)
        if name.startswith("hand_"):
            out[name + "__src"] = src
            out[name + "__dst"] = dst
        if n <= 1024:
            b = nx.betweenness_centrality(G, normalized=False)
            out[name + "__bc"] = np.array([b[v] for v in range(n)], np.float64)
        names.append(name)
    out["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "bc_networkx.npz"), **out)
    print("wrote", len(names), "graphs")


if __name__ == "__main__":
    main()

"""The oracle's betweenness restatement (orc_bc_single, following
apps/betweennessCentrality_simd/bc.cpp:1717-2097) pinned against networkx's
Brandes implementation (tests/golden/bc_networkx.npz, made by
tests/golden/make_bc_golden.py).  The reference's BC program prints no
values, so an independent implementation is the pin.

Tolerance: |oracle - networkx| <= 1e-4 * (scale + 1), where scale is the
magnitude of the float sums behind each dependency (the oracle's own bound).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import bc_case_names, bc_close, load_bc_case

BC_CASES = bc_case_names()


@pytest.mark.parametrize("name", BC_CASES)
def test_oracle_bc_dependencies_match_networkx(oracle, name):
    c = load_bc_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    for i, s in enumerate(c["sources"]):
        sigma, dep, cost, scale = oracle.bc_single(arr, int(s))
        np.testing.assert_array_equal(cost, oracle.bfs_levels(arr, int(s)))
        want = c["delta"][i].copy()
        # the reference's dependency of the source itself counts the other reached vertices
        want[s] = float((cost >= 0).sum() - 1)
        ok = bc_close(dep, want, scale)
        assert ok.all(), f"{name} source {s}: {np.flatnonzero(~ok)[:8]}"
        assert (dep[cost < 0] == 0).all() and (sigma[cost < 0] == 0).all()
        assert sigma[s] == 1


@pytest.mark.parametrize("name", [n for n in BC_CASES if load_bc_case(n)["bc"] is not None])
def test_oracle_bc_sum_over_sources_matches_networkx(oracle, name):
    c = load_bc_case(name)
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    n = c["n"]
    total = np.zeros(n, np.float64)
    scale = np.zeros(n, np.float64)
    for s in range(n):
        _, dep, _, sc = oracle.bc_single(arr, s)
        dep = dep.astype(np.float64)
        dep[s] = 0.0
        sc = sc.copy()
        sc[s] = 0.0
        total += dep
        scale += sc
    ok = bc_close(total, c["bc"], scale)
    assert ok.all(), f"{name}: {np.flatnonzero(~ok)[:8]}"


def test_oracle_bc_grid_path_counts_are_binomial(oracle):
    from math import comb
    c = load_bc_case("hand_grid6")
    arr = oracle.arrays_from_edges(c["n"], c["src"], c["dst"], c["w"], c["s"])
    sigma, _, cost, _ = oracle.bc_single(arr, 0)
    for r in range(6):
        for q in range(6):
            assert sigma[r * 6 + q] == comb(r + q, r)
            assert cost[r * 6 + q] == r + q

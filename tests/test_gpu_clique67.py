"""6- and 7-clique plans (GLUMIN P23 / P24) against the oracle and closed forms.

The reference's CPU clique app stops at k = 5; the oracle's generic DAG recursion
(orc_clique_k) reproduces the reference binaries' k = 3..5 counts (checked here) and
carries the same recursion to k = 6, 7."""
from __future__ import annotations

from math import comb

import numpy as np
import pytest

from conftest import golden_samples

pytestmark = pytest.mark.gpu


def multipartite(parts, size):
    """Complete `parts`-partite graph with equal parts: k-cliques = C(parts, k) * size^k."""
    n = parts * size
    part = np.arange(n) // size
    adj = part[:, None] != part[None, :]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    rowptr[1:] = np.cumsum(adj.sum(1))
    col = np.nonzero(adj)[1].astype(np.int32)
    return rowptr, col


def test_clique67_oracle(xgm, ctx, orc, golden):
    for case in golden:
        if case["name"] == "rmat_s14_ef16":
            continue  # the oracle needs ~30 s there; the GPU case below covers skew
        nv, s, d = golden_samples(xgm, case)
        rowptr, col = orc.build_csr(nv, s, d)
        drow, dcol = orc.orient(rowptr, col)
        g = ctx.graph_from_csr(rowptr, col)
        for k in (3, 4, 5):  # the generic recursion reproduces the pinned counts
            kind = {3: "tc", 4: "clique4", 5: "clique5"}[k]
            assert int(orc.lib().orc_clique_k(k, nv, drow.ctypes.data, dcol.ctypes.data,
                                               int(np.diff(drow).max()), 0, nv, 1)) == \
                case["counts"][kind]
        for k in (6, 7):
            want = orc.count(f"clique{k}", drow, dcol)
            assert xgm.CliqueSolver(g, k) == want, (case["name"], k)
            assert ctx.count(g, f"{k}-clique") == want, (case["name"], k)
        g.close()


def test_clique67_every_variant(xgm, ctx, orc):
    nv, s, d = xgm.gen_rmat(12, 16, seed=7)
    rowptr, col = orc.build_csr(nv, s, d)
    drow, dcol = orc.orient(rowptr, col)
    g = ctx.graph_from_csr(rowptr, col)
    for k in (6, 7):
        want = orc.count(f"clique{k}", drow, dcol)
        for var in xgm.ALL_VARIANTS:
            assert ctx.count(g, f"{k}-clique", policy=xgm.SCHED_FIXED, variant=var) == want, \
                (k, var)
    g.close()


def test_clique67_closed_forms(xgm, ctx):
    for parts, size in [(8, 20), (12, 10), (7, 40)]:  # out-degrees span all tiers
        g = ctx.graph_from_csr(*multipartite(parts, size))
        for k in (6, 7):
            assert xgm.CliqueSolver(g, k) == comb(parts, k) * size ** k, (parts, size, k)
        g.close()
    n = 40
    rowptr = np.arange(0, n * n, n - 1, dtype=np.int64)[: n + 1]
    col = np.array([j for i in range(n) for j in range(n) if j != i], dtype=np.int32)
    g = ctx.graph_from_csr(rowptr, col)
    assert xgm.CliqueSolver(g, 6) == comb(n, 6)
    assert xgm.CliqueSolver(g, 7) == comb(n, 7)
    g.close()


def test_clique67_names(xgm, ctx):
    nv, s, d = xgm.gen_ba(2000, 10, seed=3)
    g = ctx.graph_from_edges(nv, s, d)
    c6, c7 = xgm.CliqueSolver(g, 6), xgm.CliqueSolver(g, 7)
    assert ctx.count(g, xgm.plan("P23")) == c6
    assert ctx.count(g, xgm.plan("P24")) == c7
    spec = "pattern:\n  edges: [" + ", ".join(
        a + b for i, a in enumerate("ABCDEF") for b in "ABCDEF"[i + 1:]) + "]\n"
    assert ctx.count(g, xgm.plan_from_spec(spec)) == c6
    with pytest.raises(xgm.XgmError):
        xgm.CliqueSolver(g, 8)
    g.close()

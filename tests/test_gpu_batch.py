"""Batched multi-graph counting and the autotuner against per-graph oracle counts."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import oracle_counts

pytestmark = pytest.mark.gpu

PATTERNS = ["triangle", "4-clique", "diamond", "tailedtriangle", "5-clique", "rectangle"]
KIND = {"triangle": "tc", "4-clique": "clique4", "diamond": "diamond",
        "tailedtriangle": "tailed", "5-clique": "clique5", "rectangle": "cycle4"}


def per_graph_oracle(orc, vo, eo, s, d):
    out = []
    for g in range(len(vo) - 1):
        lo = vo[g]
        n = int(vo[g + 1] - lo)
        rowptr, col = orc.build_csr(n, s[eo[g]:eo[g + 1]] - lo, d[eo[g]:eo[g + 1]] - lo)
        out.append(oracle_counts(orc, rowptr, col))
    return out


@pytest.fixture(scope="module")
def ba_batch(xgm):
    return xgm.gen_ba_batch(48, 100, 1500, 3, 8, seed=5)


def test_batched_counts_match_oracle(xgm, ctx, orc, ba_batch):
    vo, eo, s, d = ba_batch
    b = ctx.batch_from_edges(vo, s, d)
    want = per_graph_oracle(orc, vo, eo, s, d)
    got = ctx.count_batched(b, PATTERNS)
    for g in range(len(vo) - 1):
        for p, name in enumerate(PATTERNS):
            assert int(got[g, p]) == want[g][KIND[name]], (g, name)
    # replay of the captured CUDA graph, direct launches and a subset of plans agree
    assert np.array_equal(ctx.count_batched(b, PATTERNS), got)
    assert np.array_equal(ctx.count_batched(b, PATTERNS, use_graph=False), got)
    assert np.array_equal(ctx.count_batched(b, PATTERNS, hash_only=True), got)
    sub = ctx.count_batched(b, ["diamond", "triangle"])
    assert np.array_equal(sub[:, 0], got[:, 2]) and np.array_equal(sub[:, 1], got[:, 0])


def test_batch_from_csr_and_packed_graph(xgm, ctx, orc, ba_batch):
    vo, eo, s, d = ba_batch
    b1 = ctx.batch_from_edges(vo, s, d)
    rowptr, col = b1.download()
    r0, c0 = orc.build_csr(int(vo[-1]), s, d)
    assert np.array_equal(rowptr, r0) and np.array_equal(col, c0)
    b2 = ctx.batch_from_csr(vo, rowptr, col)
    assert np.array_equal(ctx.count_batched(b1, ["triangle", "4-clique"]),
                          ctx.count_batched(b2, ["triangle", "4-clique"]))


def test_batch_rejects_cross_graph_edges(xgm, ctx):
    vo = np.array([0, 10, 20], np.int64)
    with pytest.raises(xgm.XgmError) as e:
        ctx.batch_from_edges(vo, np.array([1, 5], np.int32), np.array([2, 15], np.int32))
    assert e.value.status == xgm.ERR_GRAPH


def test_autotuned_table_keeps_counts(xgm, ctx, ba_batch):
    vo, eo, s, d = ba_batch
    b = ctx.batch_from_edges(vo, s, d)
    base = ctx.count_batched(b, ["triangle", "4-clique", "diamond"])
    res = ctx.autotune(b, ["triangle", "4-clique", "diamond"], reps=2)
    assert res["trials"] > 1 and res["best_ms"] > 0
    tuned = ctx.count_batched(b, ["triangle", "4-clique", "diamond"], policy=xgm.SCHED_TUNED,
                              table=res["table"])
    assert np.array_equal(tuned, base)


def test_autotune_single_graph(xgm, ctx):
    nv, s, d = xgm.gen_rmat(13, 16, seed=31)
    g = ctx.graph_from_edges(nv, s, d)
    base = ctx.count(g, "4-clique")
    res = ctx.autotune(g, "4-clique", reps=2)
    assert ctx.count(g, "4-clique", policy=xgm.SCHED_TUNED, table=res["table"]) == base


def test_full_batch_config_matches_oracle(xgm, ctx, orc):
    # the batched configuration at its full size: 4096 BA graphs, n in [100, 5000],
    # m in {3..8}, seed 5; triangle + 4-clique + diamond per graph
    vo, eo, s, d = xgm.gen_ba_batch(4096, 100, 5000, 3, 8, seed=5)
    b = ctx.batch_from_edges(vo, s, d)
    got = ctx.count_batched(b, ["triangle", "4-clique", "diamond"])
    assert got.shape == (4096, 3)
    for g in range(4096):
        lo = int(vo[g])
        rowptr, col = orc.build_csr(int(vo[g + 1]) - lo, s[eo[g]:eo[g + 1]] - lo,
                                    d[eo[g]:eo[g + 1]] - lo)
        drow, dcol = orc.orient(rowptr, col)
        want = (orc.count("tc", drow, dcol), orc.count("clique4", drow, dcol),
                orc.count("diamond", rowptr, col))
        assert tuple(int(x) for x in got[g]) == want, g

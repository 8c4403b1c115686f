"""The hub kernel: hub vertices whose out-degree is just above the main CTA's capacity
(1024 < s <= 1536) run whole in one 1024-thread CTA (bitmap of the DAG induced on N+(v0)
in shared memory, the list staged by a bulk copy) instead of one sub-task per out-edge.

Counts must equal closed forms, the oracle, and the same count with every hub split
(hub_max = -1), under the plain and the learned schedule.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _complete(n):
    iu = np.triu_indices(n, 1)
    return iu[0].astype(np.int32), iu[1].astype(np.int32)


def test_hub_kernel_complete_graph(xgm, ctx):
    n = 1300  # out-degrees 0 .. 1299: 275 hubs between 1024 and 1536
    s, d = _complete(n)
    g = ctx.graph_from_edges(n, s, d)
    try:
        assert g.info()["max_out_degree"] == n - 1
        for k, pat in ((3, "triangle"), (4, "4-clique"), (5, "5-clique")):
            # 5-cliques use the hub kernel only when asked (split by default)
            got, st = ctx.count(g, pat, with_stats=True, hub_max=1536)
            assert got == math.comb(n, k), pat
            assert st["launches"] == 2, "the hub kernel ran"
            # the same with the Bloom filter + hash membership test in every CTA task
            assert ctx.count(g, pat, hub_max=1536, hash_only=True) == math.comb(n, k), pat
        # split hubs: a triangle sub-task only counts its intersection ...
        assert ctx.count(g, "triangle", hub_max=-1) == math.comb(n, 3)
        assert ctx.count(g, "triangle", hub_max=1200) == math.comb(n, 3)
        # ... deeper ones store it, and here it holds up to 1298 > 1024 members
        with pytest.raises(xgm.XgmError) as e:
            ctx.count(g, "4-clique", hub_max=-1)
        assert e.value.status == xgm.ERR_DEVICE
    finally:
        g.close()


def test_hub_kernel_complete_multipartite(xgm, ctx):
    # K_{8 x 180}: every vertex has degree 1260, so ranks follow ids and the first
    # vertices have out-degrees up to 1260; k-cliques = C(8, k) * 180^k
    r, p = 8, 180
    n = r * p
    iu = np.triu_indices(n, 1)
    keep = (iu[0] // p) != (iu[1] // p)
    g = ctx.graph_from_edges(n, iu[0][keep].astype(np.int32), iu[1][keep].astype(np.int32))
    try:
        assert 1024 < g.info()["max_out_degree"] <= 1536
        learned = xgm.trained_schedule(ctx)
        for k, pat in ((3, "triangle"), (4, "4-clique"), (5, "5-clique")):
            want = math.comb(r, k) * p ** k
            assert ctx.count(g, pat, hub_max=1536) == want, pat
            if learned:
                assert ctx.count(g, pat, **dict(learned, hub_max=1536)) == want, pat
        # split hub sub-tasks hold intersections of up to 1080 members: triangles only
        assert ctx.count(g, "triangle", hub_max=-1) == math.comb(r, 3) * p ** 3
    finally:
        g.close()


def test_hub_kernel_matches_split_on_random_graph(xgm, ctx):
    # G(20000, ~0.06): 2518 hubs with out-degrees 1025 .. 1124 (2.7 M split sub-tasks)
    nv, s, d = xgm.gen_er(20000, 12_400_000, seed=17)
    g = ctx.graph_from_edges(nv, s, d)
    try:
        assert 1024 < g.info()["max_out_degree"] <= 1536
        learned = xgm.trained_schedule(ctx)
        for pat in ("triangle", "4-clique", "5-clique"):
            whole, st = ctx.count(g, pat, with_stats=True, hub_max=1536)
            assert st["launches"] == 2
            assert ctx.count(g, pat, hub_max=-1) == whole, pat
            assert ctx.count(g, pat) == whole, pat  # default: hub kernel up to 4-cliques
            if learned:
                assert ctx.count(g, pat, **learned) == whole, pat
        # 6-cliques never use the hub kernel: every hub is split
        _, st = ctx.count(g, "6-clique", with_stats=True)
        assert st["launches"] == 1
    finally:
        g.close()

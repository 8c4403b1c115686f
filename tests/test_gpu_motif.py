"""Vertex-induced motif census and the wedge / 3-star / 4-path / vertex-induced plans.

The census replaces the reference's MotifSolver (codes/GraphMiner/src/motif/
omp_formula.cc); its golden values come from the reference's own motif_omp_formula
binary (tests/golden/make_golden.py).  Edge-induced wedge / 3-star / 4-path counts
follow from the census through the containment identities (each induced 4-vertex
subgraph holds a fixed number of edge-induced copies of each motif)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_samples

pytestmark = pytest.mark.gpu


def edge_from_census(m3, m4):
    wedge_v, tri = m3
    star, path, tail, c4, dia, k4 = m4
    return {"wedge": wedge_v + 3 * tri, "star": star + tail + 2 * dia + 4 * k4,
            "path": path + 2 * tail + 4 * c4 + 6 * dia + 12 * k4}


def test_census_golden(xgm, ctx, golden):
    for case in golden:
        nv, s, d = golden_samples(xgm, case)
        g = ctx.graph_from_edges(nv, s, d)
        assert ctx.motif_count(g, 3) == case["counts"]["motif3"], case["name"]
        assert ctx.motif_count(g, 4) == case["counts"]["motif4"], case["name"]
        assert xgm.MotifSolver(g, 4) == case["counts"]["motif4"], case["name"]
        g.close()


def test_plans_golden(xgm, ctx, golden):
    star_spec = "pattern:\n  name: star\n  edges: [AB, AC, AD]\n  order: ABCD\n"
    for case in golden:
        nv, s, d = golden_samples(xgm, case)
        g = ctx.graph_from_edges(nv, s, d)
        c = case["counts"]
        m3, m4 = c["motif3"], c["motif4"]
        e = edge_from_census(m3, m4)
        assert ctx.count(g, xgm.plan("wedge")) == e["wedge"], case["name"]
        assert ctx.count(g, xgm.plan("3-star")) == e["star"], case["name"]
        assert ctx.count(g, xgm.plan("4-path")) == e["path"], case["name"]
        assert ctx.count(g, xgm.plan("wedge", induced=True)) == m3[0], case["name"]
        for name, i in [("3-star", 0), ("4-path", 1), ("tailedtriangle", 2), ("rectangle", 3),
                        ("diamond", 4)]:
            assert ctx.count(g, xgm.plan(name, induced=True)) == m4[i], (case["name"], name)
        # GLUMIN pattern ids (vertex-induced; P2 reports each diamond twice)
        assert ctx.count(g, xgm.plan("P1")) == m4[0], case["name"]
        assert ctx.count(g, xgm.plan("P2")) == 2 * m4[4], case["name"]
        assert ctx.count(g, xgm.plan("P3")) == m4[2], case["name"]
        assert ctx.count(g, xgm.plan("P4")) == c["clique4"], case["name"]
        assert ctx.count(g, xgm.plan("P5")) == c["clique5"], case["name"]
        assert ctx.count(g, xgm.plan_from_spec(star_spec)) == m4[0], case["name"]
        g.close()


def test_census_schedules_agree(xgm, ctx, golden):
    case = next(c for c in golden if c["name"] == "rmat_s14_ef16")
    nv, s, d = golden_samples(xgm, case)
    g = ctx.graph_from_edges(nv, s, d)
    for var in xgm.ALL_VARIANTS:
        assert ctx.motif_count(g, 4, policy=xgm.SCHED_FIXED, variant=var) == \
            case["counts"]["motif4"], var
    g.close()


def test_census_oracle_larger(xgm, ctx, orc):
    for nv, s, d in [xgm.gen_rmat(15, 16, seed=21), xgm.gen_ba(20000, 12, seed=22),
                     xgm.gen_chung_lu(30000, 2.1, 2000.0, 20.0, seed=23)]:
        rowptr, col = orc.build_csr(nv, s, d)
        g = ctx.graph_from_csr(rowptr, col)
        assert ctx.motif_count(g, 3) == orc.motif(3, rowptr, col)
        assert ctx.motif_count(g, 4) == orc.motif(4, rowptr, col)
        g.close()


def _csr(nv, edges):
    adj = [set() for _ in range(nv)]
    for a, b in edges:
        adj[a].add(b)
        adj[b].add(a)
    rowptr = np.zeros(nv + 1, dtype=np.int64)
    rowptr[1:] = np.cumsum([len(a) for a in adj])
    col = np.array([v for a in adj for v in sorted(a)], dtype=np.int32)
    return rowptr, col


def test_census_small_shapes(xgm, ctx):
    from math import comb

    n = 50
    shapes = {
        "no edges": (_csr(7, []), [0, 0], [0] * 6),
        "star": (_csr(n + 1, [(0, i) for i in range(1, n + 1)]), [comb(n, 2), 0],
                 [comb(n, 3), 0, 0, 0, 0, 0]),
        "path": (_csr(10, [(i, i + 1) for i in range(9)]), [8, 0], [0, 7, 0, 0, 0, 0]),
        "cycle": (_csr(4, [(0, 1), (1, 2), (2, 3), (3, 0)]), [4, 0], [0, 0, 0, 1, 0, 0]),
        "complete": (_csr(40, [(i, j) for i in range(40) for j in range(i)]),
                     [0, comb(40, 3)], [0, 0, 0, 0, 0, comb(40, 4)]),
    }
    for name, ((rowptr, col), m3, m4) in shapes.items():
        g = ctx.graph_from_csr(rowptr, col)
        assert ctx.motif_count(g, 3) == m3, name
        assert ctx.motif_count(g, 4) == m4, name
        g.close()


def test_census_rejects_bad_arguments(xgm, ctx):
    nv, s, d = xgm.gen_rmat(8, 8, seed=1)
    g = ctx.graph_from_edges(nv, s, d)
    with pytest.raises(xgm.XgmError) as e:
        ctx.motif_count(g, 5)
    assert e.value.status == xgm.ERR_UNSUPPORTED
    # vertex-induced plans are not part of the batched call
    vo = np.array([0, nv], dtype=np.int64)
    b = ctx.batch_from_edges(vo, s, d)
    with pytest.raises(xgm.XgmError) as e:
        ctx.count_batched(b, [xgm.plan("P1")])
    assert e.value.status == xgm.ERR_UNSUPPORTED
    b.close()
    g.close()

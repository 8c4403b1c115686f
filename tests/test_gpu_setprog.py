"""GPU parity of the set-operation program interpreter (setprog.cu).

GLUMIN's P6..P22 against the golden counts (five of them pinned to the reference's own
CPU plans) and against the oracle's restatement; compiled programs for every connected
pattern of 3 to 5 vertices against brute force and, for 3 and 4 vertices, against the
engine's builtin kernels; the split path for long v2 candidate lists; edge cases.
"""
from __future__ import annotations

import itertools

import numpy as np
import pytest

from conftest import csr_digest, golden_samples
from test_setprog import _adj, _connected_patterns, _random_graph

pytestmark = pytest.mark.gpu


def _hub_graph(n, p, seed):
    # vertex 0 adjacent to every other vertex, sparse ER among the rest: the hub's
    # tasks have v2 candidate lists far above the split threshold
    rng = np.random.default_rng(seed)
    m = np.triu(rng.random((n, n)) < p, 1)
    m[0, 1:] = True
    m = m | m.T
    rowptr = np.concatenate([[0], np.cumsum(m.sum(1))]).astype(np.int64)
    col = np.concatenate([np.nonzero(m[i])[0] for i in range(n)]).astype(np.int32)
    return rowptr, col


def test_glumin5_golden(xgm, ctx, golden):
    seen = 0
    for case in golden:
        g5 = case["counts"].get("glumin5")
        if not g5:
            continue
        nv, s, d = golden_samples(xgm, case)
        g = ctx.graph_from_edges(nv, s, d)
        assert csr_digest(*g.download()) == case["csr_sha256"], case["name"]
        for name, want in g5.items():
            assert ctx.count(g, name) == want, (case["name"], name)
        g.close()
        seen += 1
    assert seen >= 4


def test_glumin5_vs_oracle_and_split(xgm, ctx, orc):
    split = 0
    for rowptr, col in (_hub_graph(400, 0.02, 5), _random_graph(300, 0.05, 6),
                        _random_graph(120, 0.2, 7)):
        g = ctx.graph_from_csr(rowptr, col)
        for pid in range(6, 23):
            got, st = ctx.count(g, f"P{pid}", with_stats=True)
            assert got == orc.glumin5(pid, rowptr, col), pid
            # bitmap launches (small-degree v0; a second for long N(v1) streams) where the
            # plan allows them, task launch, split launch
            assert st["launches"] in (2, 3, 4) and st["tasks"] == len(col)
            assert ctx.count_kernels(g, f"P{pid}") == st["launches"]
            split += st["variant_tasks"][xgm.VAR_SPLIT]
        g.close()
    assert split > 0  # the hub graph's long candidate lists went through split records


def test_compiled_programs_vs_brute_force(xgm, ctx, orc):
    pats = [a for k in (3, 4, 5) for a in _connected_patterns(k)]
    for n, p, seed in ((40, 0.3, 1), (60, 0.15, 2)):
        rowptr, col = _random_graph(n, p, seed)
        g = ctx.graph_from_csr(rowptr, col)
        for a in pats:
            for induced in (True, False):
                plan = ctx.plan(a, induced=induced, program=True)
                want = orc.occurrences(a, induced, rowptr, col)
                assert ctx.count(g, plan) == want, (a.tolist(), induced)
        g.close()
    # the 5-vertex hub graph once more, through the split path
    rowptr, col = _hub_graph(300, 0.03, 8)
    g = ctx.graph_from_csr(rowptr, col)
    for a in _connected_patterns(5)[:12]:
        for induced in (True, False):
            w = ctx.plan(a, induced=induced, program=True)
            assert ctx.count(g, w) == orc.program(w.program, rowptr, col), a.tolist()
    g.close()


def test_compiled_programs_vs_builtins(xgm, ctx):
    # 3- and 4-vertex programs against the builtin kernels on an R-MAT graph (scale 12)
    nv, s, d = xgm.gen_rmat(12, 8, seed=3)
    g = ctx.graph_from_edges(nv, s, d)
    m3, m4 = ctx.motif_count(g, 3), ctx.motif_count(g, 4)
    shapes = {"wedge": [(0, 1), (1, 2)], "triangle": [(0, 1), (1, 2), (0, 2)],
              "3-star": [(0, 1), (0, 2), (0, 3)], "4-path": [(0, 1), (1, 2), (2, 3)],
              "tailed-triangle": [(0, 1), (1, 2), (0, 2), (2, 3)],
              "4-cycle": [(0, 1), (1, 2), (2, 3), (0, 3)],
              "diamond": [(0, 1), (1, 2), (0, 2), (2, 3), (1, 3)],
              "4-clique": list(itertools.combinations(range(4), 2))}
    builtin_edge = {"triangle": "triangle", "4-cycle": "rectangle", "diamond": "diamond",
                    "tailed-triangle": "tailedtriangle", "4-clique": "4-clique",
                    "wedge": "wedge", "3-star": "3-star", "4-path": "4-path"}
    for name, edges in shapes.items():
        k = 1 + max(max(e) for e in edges)
        a = _adj(edges, k)
        ind = m3[xgm.MOTIF3_NAMES.index(name)] if k == 3 else m4[xgm.MOTIF4_NAMES.index(name)]
        assert ctx.count(g, ctx.plan(a, induced=True, program=True)) == ind, name
        assert ctx.count(g, ctx.plan(a, induced=False, program=True)) == \
            ctx.count(g, builtin_edge[name]), name
    g.close()


def test_program_edge_cases(xgm, ctx):
    bull = _adj([(0, 1), (0, 2), (0, 4), (1, 2), (1, 3)])
    # one edge, and a graph whose vertices have no edges at all
    g = ctx.graph_from_edges(2, np.array([0], np.int32), np.array([1], np.int32))
    assert ctx.count(g, "P10") == 0 and ctx.count(g, ctx.plan(bull, True)) == 0
    g.close()
    g = ctx.graph_from_csr(np.zeros(6, np.int64), np.zeros(0, np.int32))
    assert ctx.count(g, "P6") == 0 and ctx.count(g, ctx.plan(bull, False)) == 0
    g.close()
    # complete graph K8: no induced non-clique pattern; P22 = 24 * C(8, 4); 12 5-cycles
    # in every K5
    n = 8
    iu = np.triu_indices(n, 1)
    g = ctx.graph_from_edges(n, iu[0].astype(np.int32), iu[1].astype(np.int32))
    assert ctx.count(g, ctx.plan(bull, True)) == 0
    assert ctx.count(g, "P22") == 24 * 70
    assert ctx.count(g, "5-cycle") == 56 * 12
    assert ctx.count(g, "5-star") == 8 * 35  # centre, then any 4 of the other 7
    g.close()


def test_glumin5_identities_rmat_s12(xgm, ctx):
    # at a size the oracle would take minutes on: each GLUMIN plan whose count is a
    # multiple of one vertex-induced pattern equals that multiple of the compiled
    # program's count (a different program, symmetry breaking and code path), and
    # P22 = 24 x 4-cliques (clique kernel) + 12 x induced (K5 minus an edge)
    from test_setprog import GLUMIN5_PATTERNS

    nv, s, d = xgm.gen_rmat(12, 8, seed=3)
    g = ctx.graph_from_edges(nv, s, d)
    for pid, (edges, factor) in GLUMIN5_PATTERNS.items():
        compiled = ctx.count(g, ctx.plan(_adj(edges), induced=True))
        assert ctx.count(g, f"P{pid}") == factor * compiled, pid
    k5e = ctx.plan(_adj([e for e in itertools.combinations(range(5), 2) if e != (3, 4)]),
                   induced=True)
    assert ctx.count(g, "P22") == 24 * ctx.count(g, "4-clique") + 12 * ctx.count(g, k5e)
    g.close()


def test_glumin5_hub_above_bitmap_range(xgm, ctx, orc):
    # a hub of degree 1,499 (above the bitmap forms' 1,024): its tasks run in the list
    # form while the other vertices' tasks take the bitmap forms, within one count; the
    # plans here are the ones the oracle finishes quickly on such a hub (P12 a stream plan)
    rowptr, col = _hub_graph(1500, 0.01, 9)
    assert int(np.diff(rowptr).max()) > 1024
    g = ctx.graph_from_csr(rowptr, col)
    for pid in (9, 12, 13, 14, 17, 19, 20, 22):
        assert ctx.count(g, f"P{pid}") == orc.glumin5(pid, rowptr, col), pid
    g.close()


def test_record_overflow_paths(xgm, ctx, orc, monkeypatch):
    # with the record capacities lowered (test hook), the tasks that cannot queue their
    # split / stream records run them themselves; counts are unchanged
    rowptr, col = _hub_graph(400, 0.02, 5)
    g = ctx.graph_from_csr(rowptr, col)
    want = {pid: orc.glumin5(pid, rowptr, col) for pid in (6, 7, 10, 15)}
    for cap in ("0", "7"):
        monkeypatch.setenv("XGM_PROG_RECORD_CAP", cap)
        for pid, w in want.items():
            assert ctx.count(g, f"P{pid}") == w, (cap, pid)
    monkeypatch.delenv("XGM_PROG_RECORD_CAP")
    g.close()


def test_compiled_six_vertex_programs_gpu(xgm, ctx, orc):
    # every connected 6-vertex pattern, vertex- and edge-induced, against brute force on a
    # small random graph; then a hub graph (split records) against the oracle's
    # interpreter of the same program words
    pats = _connected_patterns(6)
    rowptr, col = _random_graph(22, 0.35, 4)
    g = ctx.graph_from_csr(rowptr, col)
    for a in pats:
        for induced in (True, False):
            plan = ctx.plan(a, induced=induced, program=True)
            assert ctx.count(g, plan) == orc.occurrences(a, induced, rowptr, col), \
                (a.tolist(), induced)
    g.close()
    rowptr, col = _hub_graph(120, 0.04, 11)
    g = ctx.graph_from_csr(rowptr, col)
    for edges, induced in (([(0, i) for i in range(1, 6)], True),
                           ([(i, i + 1) for i in range(5)], False),
                           ([(i, (i + 1) % 6) for i in range(6)], True)):
        plan = ctx.plan(_adj(edges, 6), induced=induced, program=True)
        assert ctx.count(g, plan) == orc.program(plan.program, rowptr, col), edges
    g.close()

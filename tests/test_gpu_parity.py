"""GPU engine vs the reference (golden counts from its binaries) and the oracle.

Every count is compared bit-exactly.  Sizes are small enough for the oracle to finish
in seconds (R-MAT up to scale 19); the full 4096-graph batch is in test_gpu_batch.py.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import (DAG_KINDS, KIND_TO_PATTERN, csr_digest, golden_samples, oracle_counts,
                      relabel_by_degree)

pytestmark = pytest.mark.gpu


def gpu_counts(ctx, g, **kw):
    return {k: ctx.count(g, p, **kw) for k, p in KIND_TO_PATTERN.items()}


def test_golden_counts_from_reference_binaries(xgm, ctx, golden):
    for case in golden:
        nv, src, dst = golden_samples(xgm, case)
        g = ctx.graph_from_edges(nv, src, dst)
        rowptr, col = g.download()
        assert csr_digest(rowptr, col) == case["csr_sha256"], case["name"]
        assert g.info()["E_dag"] == case["E_dag"]
        got = gpu_counts(ctx, g)
        assert got == {k: case["counts"][k] for k in got}, case["name"]
        g.close()


def test_csr_and_orientation_match_oracle(xgm, ctx, orc):
    nv, src, dst = xgm.gen_rmat(13, 16, seed=21)
    g = ctx.graph_from_edges(nv, src, dst)
    r0, c0 = orc.build_csr(nv, src, dst)
    r1, c1 = g.download(xgm.VIEW_UNDIRECTED)
    assert np.array_equal(r0, r1) and np.array_equal(c0, c1)
    d0, e0 = orc.orient(r0, c0)
    d1, e1 = g.download(xgm.VIEW_DAG)
    assert np.array_equal(d0, d1) and np.array_equal(e0, e1)
    info = g.info()
    assert info["max_out_degree"] == int(np.max(np.diff(d0)))
    assert info["max_degree"] == int(np.max(np.diff(r0)))


@pytest.mark.parametrize("gen", ["chung_lu", "rmat_dense", "er", "ba"])
def test_oracle_parity(xgm, ctx, orc, gen):
    if gen == "chung_lu":
        nv, s, d = xgm.gen_chung_lu(1 << 13, 2.1, 1500.0, 24.0, seed=4)
    elif gen == "rmat_dense":
        nv, s, d = xgm.gen_rmat(11, 64, seed=5)
    elif gen == "er":
        nv, s, d = xgm.gen_er(1 << 14, 1 << 18, seed=6)
    else:
        nv, s, d = xgm.gen_ba(20000, 7, seed=7)
    g = ctx.graph_from_edges(nv, s, d)
    rowptr, col = orc.build_csr(nv, s, d)
    assert gpu_counts(ctx, g) == oracle_counts(orc, rowptr, col)


def test_schedules_never_change_counts(xgm, ctx):
    nv, s, d = xgm.gen_rmat(13, 32, seed=9)
    g = ctx.graph_from_edges(nv, s, d)
    for pat in ("triangle", "4-clique", "5-clique", "diamond", "tailedtriangle"):
        base = ctx.count(g, pat)
        for var in xgm.ALL_VARIANTS:
            assert ctx.count(g, pat, policy=xgm.SCHED_FIXED, variant=var) == base, (pat, var)
        for smax, wmax, dmax, cmax in ((0, 8, 0, 64), (8, 32, 64, 128), (32, 1, -1, 1),
                                       (4, 16, 100, 2048)):
            assert ctx.count(g, pat, search_max=smax, warp_max=wmax, wide_max=dmax,
                             cta_max=cmax) == base, (pat, smax, wmax, dmax, cmax)
        for bmax, smax in ((32, 0), (8, 32), (1, 4)):  # bucket-filtered search tiers
            assert ctx.count(g, pat, bucket_max=bmax, search_max=smax) == base, (pat, bmax)
        for gmax, bmax in ((8, 0), (3, 16), (5, 32)):  # eight-lane group tasks
            assert ctx.count(g, pat, group_max=gmax, bucket_max=bmax) == base, (pat, gmax)


@pytest.mark.parametrize("gen", ["chung_lu", "rmat_dense", "ba"])
def test_membership_paths_agree(xgm, ctx, orc, gen):
    """CTA tasks test membership of a streamed element with a bitmap over the local
    set's id span when it fits, else with a Bloom filter and a hash; XGM_SCHED_HASH_ONLY
    forces the second path.  Every vertex task runs as a CTA task (SCHED_FIXED CTA), so
    both paths see every task; counts equal the oracle's either way."""
    if gen == "chung_lu":
        nv, s, d = xgm.gen_chung_lu(1 << 13, 2.1, 1500.0, 24.0, seed=4)
    elif gen == "rmat_dense":
        nv, s, d = xgm.gen_rmat(11, 64, seed=5)
    else:
        nv, s, d = xgm.gen_ba(20000, 7, seed=7)
    g = ctx.graph_from_edges(nv, s, d)
    rowptr, col = orc.build_csr(nv, s, d)
    want = oracle_counts(orc, rowptr, col)
    for hash_only in (False, True):
        got = {k: ctx.count(g, p, policy=xgm.SCHED_FIXED, variant=xgm.VAR_CTA,
                            hash_only=hash_only) for k, p in KIND_TO_PATTERN.items()}
        assert got == want, (gen, hash_only)
        assert {k: ctx.count(g, p, hash_only=hash_only)
                for k, p in KIND_TO_PATTERN.items()} == want, (gen, hash_only)


def test_upload_paths_agree(xgm, ctx, orc):
    nv, s, d = xgm.gen_ba(5000, 6, seed=13)
    rowptr, col = orc.build_csr(nv, s, d)
    g1 = ctx.graph_from_csr(rowptr, col, flags=xgm.BUILD_VALIDATE)
    g2 = ctx.graph_from_edges(nv, s, d)
    # a CSR with duplicates and self-loops is cleaned by the CLEAN flags
    dirty_r = rowptr.copy()
    dirty_c = col.copy()
    g3 = ctx.graph_from_csr(dirty_r, dirty_c, flags=xgm.BUILD_CLEAN)
    for pat in ("triangle", "4-clique", "diamond", "rectangle"):
        assert ctx.count(g1, pat) == ctx.count(g2, pat) == ctx.count(g3, pat)


def test_reference_file_format_roundtrip(xgm, ctx, orc, tmp_path):
    nv, s, d = xgm.gen_rmat(10, 8, seed=3)
    rowptr, col = orc.build_csr(nv, s, d)
    prefix = str(tmp_path / "graph")
    orc.write_graph(prefix, rowptr, col)
    g = ctx.load_graph(prefix)
    r1, c1 = g.download()
    assert np.array_equal(r1, rowptr) and np.array_equal(c1, col)
    drow, dcol = orc.orient(rowptr, col)
    assert xgm.TCSolver(g) == orc.count("tc", drow, dcol)
    assert xgm.CliqueSolver(g, 4) == orc.count("clique4", drow, dcol)
    assert xgm.CliqueSolver(g, 5) == orc.count("clique5", drow, dcol)
    assert xgm.ScSolver(g, "diamond") == orc.count("diamond", rowptr, col)
    assert xgm.ScSolver(g, "rectangle") == orc.count("cycle4", rowptr, col)
    assert xgm.ScSolver(g, "tailedtriangle") == orc.count("tailed", rowptr, col)


def _closed_form(n):
    from math import comb
    return {"tc": comb(n, 3), "clique4": comb(n, 4), "clique5": comb(n, 5),
            "diamond": comb(n, 4) * 6, "cycle4": comb(n, 4) * 3,
            "tailed": n * comb(n - 1, 2) * (n - 3)}


@pytest.mark.parametrize("n", [4, 5, 33, 70])
def test_complete_graphs(xgm, ctx, n):
    iu = np.triu_indices(n, 1)
    g = ctx.graph_from_edges(n, iu[0].astype(np.int32), iu[1].astype(np.int32))
    assert gpu_counts(ctx, g) == _closed_form(n)


def test_dense_hub_split_tasks(xgm, ctx):
    # K_1100: the lowest-ranked vertices have out-degree > 1024, so their tasks are split
    # into edge sub-tasks whose intersections exceed the shared-memory capacity; plans
    # that only need the intersection size or participation must still be exact
    n = 1100
    iu = np.triu_indices(n, 1)
    g = ctx.graph_from_edges(n, iu[0].astype(np.int32), iu[1].astype(np.int32))
    want = _closed_form(n)
    assert ctx.count(g, "triangle") == want["tc"]
    assert ctx.count(g, "diamond") == want["diamond"]
    assert ctx.count(g, "tailedtriangle") == want["tailed"]
    assert ctx.count(g, "rectangle") == want["cycle4"]


def test_cycle4_grouped_dense_tasks(xgm, ctx, orc):
    # R-MAT scale 19: hub tasks with many wedges relative to their id range run in
    # L2-resident counter groups (more than one group here); the rest in the persistent
    # kernel.  Both paths add to the same exact count.
    nv, s, d = xgm.gen_rmat(19, 16, seed=2)
    rowptr, col = orc.build_csr(nv, s, d)
    g = ctx.graph_from_csr(rowptr, col)
    assert ctx.count(g, "rectangle") == orc.count("cycle4", rowptr, col)
    g.close()


def test_edge_cases(xgm, ctx, orc):
    # no edges at all
    g = ctx.graph_from_edges(10, np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert all(v == 0 for v in gpu_counts(ctx, g).values())
    # only self-loops and duplicates
    g = ctx.graph_from_edges(4, np.array([1, 1, 2, 2], np.int32), np.array([1, 1, 2, 3], np.int32))
    assert g.info()["E"] == 2
    # star: no triangles, C(d,2)*(0) tailed, no cycles
    n = 3000
    s = np.zeros(n - 1, np.int32)
    d = np.arange(1, n, dtype=np.int32)
    g = ctx.graph_from_edges(n, s, d)
    assert gpu_counts(ctx, g) == {k: 0 for k in KIND_TO_PATTERN}
    # wheel: hub joined to a cycle (hub out-degree stays small, cycle vertices)
    m = 2000
    cyc = np.arange(m, dtype=np.int32)
    s = np.concatenate([cyc, np.full(m, m, np.int32)])
    d = np.concatenate([(cyc + 1) % m, cyc])
    g = ctx.graph_from_edges(m + 1, s, d)
    rowptr, col = orc.build_csr(m + 1, s, d)
    assert gpu_counts(ctx, g) == oracle_counts(orc, rowptr, col)


def test_invalid_inputs_raise(xgm, ctx):
    with pytest.raises(xgm.XgmError) as e:
        ctx.graph_from_edges(5, np.array([0, 7], np.int32), np.array([1, 2], np.int32))
    assert e.value.status == xgm.ERR_GRAPH
    # unsorted row rejected by VALIDATE
    rowptr = np.array([0, 2, 3, 4], np.int64)
    col = np.array([2, 1, 0, 0], np.int32)
    with pytest.raises(xgm.XgmError) as e:
        ctx.graph_from_csr(rowptr, col, flags=xgm.BUILD_VALIDATE)
    assert e.value.status == xgm.ERR_GRAPH
    with pytest.raises(xgm.XgmError):
        ctx.plan("house")  # not a supported pattern
    with pytest.raises(xgm.XgmError) as e:
        ctx.count(ctx.graph_from_edges(3, np.array([0], np.int32), np.array([1], np.int32)),
                  "4-clique", policy=xgm.SCHED_LEARNED)
    assert e.value.status == xgm.ERR_INVALID


def test_plan_from_adjacency(xgm, ctx):
    tri = np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]])
    diamond = np.ones((4, 4), int) - np.eye(4, dtype=int)
    diamond[0, 3] = diamond[3, 0] = 0
    c4 = np.array([[0, 1, 0, 1], [1, 0, 1, 0], [0, 1, 0, 1], [1, 0, 1, 0]])
    tt = np.array([[0, 1, 1, 1], [1, 0, 1, 0], [1, 1, 0, 0], [1, 0, 0, 0]])
    assert ctx.plan(tri).pattern == xgm.TRIANGLE
    assert ctx.plan(diamond).pattern == xgm.DIAMOND
    assert ctx.plan(c4).pattern == xgm.CYCLE4
    assert ctx.plan(tt).pattern == xgm.TAILED_TRIANGLE
    assert ctx.plan(np.ones((5, 5), int) - np.eye(5, dtype=int)).pattern == xgm.CLIQUE5


def test_algo_bytes_match_oracle(xgm, ctx, orc):
    # scale 14: out-degrees above the clipping threshold exist, weights must be unclipped
    nv, s, d = xgm.gen_rmat(14, 16, seed=17)
    g = ctx.graph_from_edges(nv, s, d)
    rowptr, col = orc.build_csr(nv, s, d)
    drow, dcol = orc.orient(rowptr, col)
    assert g.info()["max_out_degree"] > 96
    for kind, pat in (("tc", "triangle"), ("clique4", "4-clique"), ("clique5", "5-clique")):
        assert ctx.algo_bytes(g, pat) == orc.algo_bytes(kind, drow, dcol), kind
    for kind, pat in (("diamond", "diamond"), ("tailed", "tailedtriangle")):
        assert ctx.algo_bytes(g, pat) == orc.algo_bytes(kind, rowptr, col), kind
    # the 4-cycle wedge walk depends on the vertex order: the engine walks rank order
    rr, rc = relabel_by_degree(rowptr, col)
    assert ctx.algo_bytes(g, "rectangle") == orc.algo_bytes("cycle4", rr, rc)
    assert orc.count("cycle4", rr, rc) == orc.count("cycle4", rowptr, col)


@pytest.mark.parametrize("n", [3, 5, 8, 9, 10, 12, 33, 40])
def test_complete_graphs_every_variant(xgm, ctx, n):
    # K_n: out-degrees 0..n-1, so every task-size boundary of the variants (GROUP <= 8,
    # WARP / SEARCH / BUCKET <= 32, WIDE <= 128) is crossed; counts have closed forms
    from math import comb
    iu = np.triu_indices(n, 1)
    g = ctx.graph_from_edges(n, iu[0].astype(np.int32), iu[1].astype(np.int32))
    for var in xgm.ALL_VARIANTS:
        for k, pat in ((3, "triangle"), (4, "4-clique"), (5, "5-clique"), (6, "6-clique")):
            assert ctx.count(g, pat, policy=xgm.SCHED_FIXED, variant=var) == comb(n, k), (n, var, k)
        assert ctx.count(g, "diamond", policy=xgm.SCHED_FIXED, variant=var) == 6 * comb(n, 4)
    g.close()

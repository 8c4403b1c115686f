"""The CPU oracle against the reference's known answers and its own binaries."""
from __future__ import annotations

import os
import tempfile

import numpy as np
import pytest

from conftest import REFERENCE_GRAPHS, REFERENCE_ROOT, csr_digest, golden_samples, oracle_counts

CITESEER = os.path.join(REFERENCE_GRAPHS, "citeseer", "graph")


@pytest.mark.skipif(not os.path.exists(CITESEER + ".meta.txt"), reason="reference tree absent")
def test_citeseer_known_answers(orc):
    # triangle/README.md:53 (1,166), motif/README.md:57 (255 4-cliques),
    # count/README.md:41 (3,730 diamonds, 6,059 4-cycles)
    rowptr, col = orc.read_graph(CITESEER)
    c = oracle_counts(orc, rowptr, col)
    assert c["tc"] == 1166
    assert c["clique4"] == 255
    assert c["diamond"] == 3730
    assert c["cycle4"] == 6059
    # identities with the vertex-induced rows of motif/README.md:50-57
    # (4-cycles 3,094, diamonds 2,200, tailed triangles 22,900, 4-cliques 255)
    assert c["diamond"] == 2200 + 6 * 255
    assert c["cycle4"] == 3094 + 2200 + 3 * 255
    assert c["tailed"] == 22900 + 4 * 2200 + 12 * 255
    # the oracle's restatement of the formula motif counter, motif/README.md:52-60
    # (wedges 23,380, triangles 1,166; 4-paths 111,153, 3-stars 222,630)
    assert orc.motif(3, rowptr, col) == [23380, 1166]
    assert orc.motif(4, rowptr, col) == [222630, 111153, 22900, 3094, 2200, 255]


def test_golden_fixtures(xgm, orc, golden):
    for case in golden:
        nv, src, dst = golden_samples(xgm, case)
        rowptr, col = orc.build_csr(nv, src, dst)
        assert csr_digest(rowptr, col) == case["csr_sha256"], case["name"]
        c = oracle_counts(orc, rowptr, col)
        assert c == {k: case["counts"][k] for k in c}, case["name"]
        # vertex-induced census, fixtures from the reference's motif_omp_formula
        assert orc.motif(3, rowptr, col) == case["counts"]["motif3"], case["name"]
        assert orc.motif(4, rowptr, col) == case["counts"]["motif4"], case["name"]


def _edge_list(path):
    with open(path) as f:
        nv, _ = map(int, f.readline().split())
        e = np.array([list(map(int, l.split()[:2])) for l in f if l.strip()], dtype=np.int32)
    return nv, e[:, 0], e[:, 1]


@pytest.mark.parametrize("name", ["test_gr1.txt", "test_gr2.txt", "test_gr3.txt", "test_gr4.txt"])
def test_reference_tiny_graphs(orc, name):
    path = os.path.join(REFERENCE_ROOT, "scripts", name)
    if not os.path.exists(path) or not orc.ref_available("count_omp_base"):
        pytest.skip("reference tree / reference binaries absent")
    nv, s, d = _edge_list(path)
    rowptr, col = orc.build_csr(nv, s, d)
    prefix = os.path.join(tempfile.mkdtemp(), "graph")
    orc.write_graph(prefix, rowptr, col)
    mine = oracle_counts(orc, rowptr, col)
    for k, v in mine.items():
        if nv < 4 and k != "tc":
            continue
        assert orc.run_ref(k, prefix)[0] == v, k
    if orc.ref_available("motif_omp_formula"):
        for k in (3, 4):
            assert orc.run_ref_motif(k, prefix) == orc.motif(k, rowptr, col), k


def test_csr_build_cleans(orc):
    rng = np.random.default_rng(0)
    nv = 300
    s = rng.integers(0, nv, 5000).astype(np.int32)
    d = rng.integers(0, nv, 5000).astype(np.int32)
    s[:50] = d[:50]  # self-loops
    s = np.concatenate([s, s[:100]])  # duplicates
    d = np.concatenate([d, d[:100]])
    rowptr, col = orc.build_csr(nv, s, d)
    pairs = {(int(a), int(b)) for a, b in zip(s, d) if a != b}
    pairs |= {(b, a) for a, b in pairs}
    want = sorted(pairs)
    got = [(u, int(col[e])) for u in range(nv) for e in range(rowptr[u], rowptr[u + 1])]
    assert got == want


def test_orientation_rule(orc):
    rng = np.random.default_rng(1)
    nv = 200
    rowptr, col = orc.build_csr(nv, rng.integers(0, nv, 3000), rng.integers(0, nv, 3000))
    deg = np.diff(rowptr)
    drow, dcol = orc.orient(rowptr, col)
    for u in range(nv):
        nb = col[rowptr[u]:rowptr[u + 1]]
        keep = [v for v in nb if deg[v] > deg[u] or (deg[v] == deg[u] and v > u)]
        assert list(dcol[drow[u]:drow[u + 1]]) == keep
    assert len(dcol) * 2 == len(col)


def test_algo_bytes_tc_formula(orc):
    rng = np.random.default_rng(2)
    nv = 500
    rowptr, col = orc.build_csr(nv, rng.integers(0, nv, 8000), rng.integers(0, nv, 8000))
    drow, dcol = orc.orient(rowptr, col)
    dp = np.diff(drow)
    want = 0
    for u in range(nv):
        for v in dcol[drow[u]:drow[u + 1]]:
            want += 8 + 4 * (int(dp[u]) + int(dp[v]))
    assert orc.algo_bytes("tc", drow, dcol) == want


def test_sampled_counts_partition(orc):
    rng = np.random.default_rng(3)
    nv = 400
    rowptr, col = orc.build_csr(nv, rng.integers(0, nv, 6000), rng.integers(0, nv, 6000))
    drow, dcol = orc.orient(rowptr, col)
    full = orc.count("clique4", drow, dcol)
    parts = sum(orc.count("clique4", drow, dcol, lo=o, hi=nv, stride=4) for o in range(4))
    assert parts == full

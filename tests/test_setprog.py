"""Set-operation programs on the CPU (no GPU).

GLUMIN's 5-vertex plans P6..P22 as the oracle restates them, pinned to the reference's
own CPU plans and to brute-force pattern counts; the engine's program tables and its
pattern compiler, read through the C-ABI (xgm_plan_program) and run by the oracle's
program interpreter, against the same.
"""
from __future__ import annotations

import itertools
import os

import numpy as np
import pytest

from conftest import REFERENCE_GRAPHS

CITESEER = os.path.join(REFERENCE_GRAPHS, "citeseer", "graph")


def _adj(edges, k=5):
    a = np.zeros((k, k), dtype=np.uint8)
    for u, v in edges:
        a[u, v] = a[v, u] = 1
    return a


def _random_graph(n, p, seed):
    rng = np.random.default_rng(seed)
    m = np.triu(rng.random((n, n)) < p, 1)
    m = m | m.T
    rowptr = np.concatenate([[0], np.cumsum(m.sum(1))]).astype(np.int64)
    col = np.concatenate([np.nonzero(m[i])[0] for i in range(n)]).astype(np.int32)
    return rowptr, col


GRAPHS = [(40, 0.3, 1), (60, 0.15, 2), (30, 0.5, 3)]

# GLUMIN P id -> (vertex-induced pattern, embeddings counted per occurrence), read from
# the generated kernels (GM_kernels/P<id>-GM.yml.cuh) and confirmed here by brute force
GLUMIN5_PATTERNS = {
    6: ([(0, 1), (0, 2), (0, 3), (0, 4), (1, 4), (2, 3)], 1),          # bowtie
    7: ([(0, 1), (0, 2), (0, 4), (1, 2), (1, 3)], 2),                  # bull
    8: ([(0, 1), (0, 3), (0, 4), (1, 2), (1, 4), (2, 3)], 2),          # house
    9: ([(0, 1), (0, 2), (0, 3), (0, 4), (1, 2), (1, 3), (1, 4), (2, 3)], 2),  # K5 - 2 adj. edges
    10: ([(0, 1), (0, 2), (0, 3), (0, 4)], 1),                         # 4-star
    11: ([(0, 2), (0, 3), (0, 4), (1, 2), (1, 3)], 1),                 # tailed 4-cycle
    14: ([(0, 1), (0, 2), (0, 3), (0, 4), (1, 2), (1, 3), (2, 3)], 3),  # tailed 4-clique
    15: ([(0, 1), (0, 3), (0, 4), (1, 2)], 1),                         # chair
    16: ([(0, 1), (0, 2), (0, 4), (1, 2), (1, 3), (2, 3)], 1),         # diamond, tail at a tip
    17: ([(0, 1), (0, 2), (0, 3), (0, 4), (1, 2), (1, 4), (2, 3)], 2),  # gem
    18: ([(0, 1), (0, 2), (0, 3), (0, 4), (1, 2)], 1),                 # cricket
    20: ([(0, 1), (0, 2), (0, 3), (0, 4), (1, 2), (1, 3)], 1),         # diamond, tail at a hub
    21: ([(0, 1), (0, 4), (1, 2), (1, 3), (2, 3)], 1),                 # triangle + 2-path
}


@pytest.mark.skipif(not os.path.exists(CITESEER + ".meta.txt"), reason="reference tree absent")
def test_glumin5_against_reference_cpu_plans(orc):
    # GLUMIN's own CPU plans (src/pattern/cpu_serials.cc) restate the generated GPU plans
    # of P7, P10, P13, P15 and P20 (P13 with its repeated-vertex embeddings)
    if not orc.ref_available("glumin_pattern_cpu"):
        orc.build_ref()
    if not orc.ref_available("glumin_pattern_cpu"):
        pytest.skip("reference CPU plans did not build")
    rowptr = np.fromfile(CITESEER + ".vertex.bin", dtype=np.int64)
    col = np.fromfile(CITESEER + ".edge.bin", dtype=np.int32)
    for pid in orc.GLUMIN5_CPU:
        mine = orc.glumin5(pid, rowptr, col)
        for lut in (False, True):
            assert orc.run_ref_glumin5(pid, CITESEER, lut)[0] == mine, (pid, lut)


def test_glumin5_counts_patterns(orc):
    for n, p, seed in GRAPHS:
        rowptr, col = _random_graph(n, p, seed)
        for pid, (edges, factor) in GLUMIN5_PATTERNS.items():
            want = factor * orc.occurrences(_adj(edges), True, rowptr, col)
            assert orc.glumin5(pid, rowptr, col) == want, (pid, n, p)
        # P22 also counts the degenerate v4 = v3: 24 ordered 4-cliques per 4-clique, plus
        # 12 embeddings of every induced K5 minus one edge
        k4 = orc.occurrences(np.ones((4, 4), np.uint8) - np.eye(4, dtype=np.uint8), True,
                             rowptr, col)
        k5e = orc.occurrences(_adj([e for e in itertools.combinations(range(5), 2)
                                    if e != (3, 4)]), True, rowptr, col)
        assert orc.glumin5(22, rowptr, col) == 24 * k4 + 12 * k5e


def test_glumin5_golden_pins(orc, xgm, golden):
    from conftest import golden_samples, csr_digest
    for case in golden:
        g5 = case["counts"].get("glumin5")
        if not g5 or case["V"] > 1024:
            continue
        nv, s, d = golden_samples(xgm, case)
        rowptr, col = orc.build_csr(nv, s, d)
        assert csr_digest(rowptr, col) == case["csr_sha256"]
        for name in ("P6", "P13", "P19", "P22"):
            assert orc.glumin5(int(name[1:]), rowptr, col) == g5[name], (case["name"], name)


def test_engine_glumin_tables(xgm, orc):
    # the engine's P6..P22 programs (read through the C-ABI) and the oracle's loops
    for n, p, seed in GRAPHS:
        rowptr, col = _random_graph(n, p, seed)
        for pid in range(6, 23):
            w = xgm.plan(f"P{pid}").program
            assert orc.program(w, rowptr, col) == orc.glumin5(pid, rowptr, col), (pid, n)


def _connected_patterns(k):
    """One adjacency matrix per isomorphism class of connected k-vertex graphs.  The
    canonical form of every edge set (a bitmask over the vertex pairs) is the smallest
    mask over all vertex permutations, computed for all edge sets at once."""
    pairs = list(itertools.combinations(range(k), 2))
    index = {pq: i for i, pq in enumerate(pairs)}
    masks = np.arange(1 << len(pairs), dtype=np.int64)
    canon = masks.copy()
    for perm in itertools.permutations(range(k)):
        mapped = np.zeros_like(masks)
        for i, (u, v) in enumerate(pairs):
            pu, pv = perm[u], perm[v]
            j = index[(pu, pv) if pu < pv else (pv, pu)]
            mapped |= ((masks >> i) & 1) << j
        np.minimum(canon, mapped, out=canon)
    out = []
    for m in np.unique(canon):
        es = [pairs[i] for i in range(len(pairs)) if (int(m) >> i) & 1]
        a = _adj(es, k)
        reach, stack = {0}, [0]
        while stack:
            x = stack.pop()
            for y in np.nonzero(a[x])[0]:
                if int(y) not in reach:
                    reach.add(int(y))
                    stack.append(int(y))
        if len(reach) == k:
            out.append(a)
    return out


def test_compiled_programs_count_occurrences(xgm, orc):
    # every connected pattern of 3 to 5 vertices, vertex- and edge-induced: the compiled
    # program (symmetry breaking, explicit exclusion of matched vertices) counts each
    # occurrence once
    pats = [a for k in (3, 4, 5) for a in _connected_patterns(k)]
    assert len(pats) == 2 + 6 + 21
    for n, p, seed in GRAPHS[:2]:
        rowptr, col = _random_graph(n, p, seed)
        for a in pats:
            for induced in (True, False):
                w = xgm.plan(a, induced=induced, program=True).program
                assert w is not None and w[1] == a.shape[0]
                want = orc.occurrences(a, induced, rowptr, col)
                assert orc.program(w, rowptr, col) == want, (a.tolist(), induced, n)


def test_compiled_six_vertex_programs(xgm, orc):
    # every connected 6-vertex pattern (112), vertex- and edge-induced, on a small random
    # graph: the compiled program run by the oracle's interpreter equals brute force
    pats = _connected_patterns(6)
    assert len(pats) == 112
    rowptr, col = _random_graph(22, 0.35, 4)
    for a in pats:
        for induced in (True, False):
            w = xgm.plan(a, induced=induced, program=True).program
            assert w is not None and w[1] == 6
            assert orc.program(w, rowptr, col) == orc.occurrences(a, induced, rowptr, col), \
                (a.tolist(), induced)


def test_program_slots_fit_bitmap_forms(xgm):
    # the bitmap kernels hold 8 slots per task (kLutSlots); a 4- or 5-vertex program
    # above that would run in the list form only.  Every GLUMIN plan and every compiled
    # 4- and 5-vertex program stays within it; 6-vertex programs fit the 16 of the format
    for pid in range(6, 23):
        assert xgm.plan(f"P{pid}").program[2] <= 8, pid
    for k, cap in ((4, 8), (5, 8), (6, 16)):
        for a in _connected_patterns(k):
            for induced in (True, False):
                assert xgm.plan(a, induced=induced, program=True).program[2] <= cap, \
                    (a.tolist(), induced)


def test_program_plan_api(xgm):
    # 5-vertex non-clique patterns compile without asking; the 5-clique stays a builtin
    bull = _adj([(0, 1), (0, 2), (0, 4), (1, 2), (1, 3)])
    p = xgm.plan(bull, induced=True)
    assert p.pattern == xgm.PROGRAM and p.induced
    assert xgm.plan(np.ones((5, 5), np.uint8) - np.eye(5, dtype=np.uint8)).pattern == xgm.CLIQUE5
    # a program's words: version, k, slots within bounds, operand codes well formed
    w = p.program
    assert w[0] == 2 and w[1] == 5 and 0 < w[2] <= 16 and w[4] in (0, 1)
    with pytest.raises(xgm.XgmError) as e:  # disconnected
        xgm.plan(_adj([(0, 1), (2, 3), (3, 4)]), induced=True)
    assert e.value.status == xgm.ERR_UNSUPPORTED
    with pytest.raises(xgm.XgmError) as e:  # seven vertices, no clique
        xgm.plan(_adj([(i, i + 1) for i in range(6)], 7), induced=True)
    assert e.value.status == xgm.ERR_UNSUPPORTED
    assert xgm.plan(_adj([(i, i + 1) for i in range(5)], 6), induced=True).program[1] == 6

"""GPU counts at the benchmark configurations against the reference's own binaries.

tests/golden/config_counts.json holds, per configuration graph, the sha256 of its CSR
and the counts of the reference's OpenMP binaries (tc_omp_base, clique_omp_base,
count_omp_base; made by tests/golden/make_config_golden.py):

  - triangle (and the other patterns) on R-MAT scale 16, edge factor 16, seed 1;
  - triangle / 4-clique / diamond / 5-clique on R-MAT scale 22, edge factor 16, seed 2;
  - edge-induced diamond / 4-cycle / tailed triangle / 4-clique (and triangle) on
    Erdos-Renyi G(2^21, avg degree 32), seed 3, and Chung-Lu (2^21 vertices,
    exponent 2.1, maximum weight 50,000, avg degree 32), seed 4;
  - triangle / 4-clique / diamond / 5-clique on the held-out R-MAT scale 23, edge
    factor 16, seed 99.

Each test regenerates the graph with the engine's generator, builds it on the GPU,
checks the digest of the downloaded CSR (the same graph the reference counted) and
compares every count bit for bit, under the plain heuristic schedule and the trained
learned schedule.  The oracle cannot run at these sizes in a test; these fixtures are
the pin.
"""
from __future__ import annotations

import json
import os

import pytest

from conftest import KIND_TO_PATTERN, ROOT, csr_digest

pytestmark = pytest.mark.gpu

CONFIG_PATH = os.path.join(ROOT, "tests", "golden", "config_counts.json")
CONFIGS = json.load(open(CONFIG_PATH)) if os.path.exists(CONFIG_PATH) else {}


def _samples(xgm, rec):
    gen, a, seed = rec["gen"], rec["args"], rec["seed"]
    if gen == "rmat":
        return xgm.gen_rmat(a[0], a[1], seed=seed)
    if gen == "er":
        return xgm.gen_er(a[0], a[1], seed=seed)
    if gen == "chung_lu":
        return xgm.gen_chung_lu(a[0], a[1], a[2], a[3], seed=seed)
    raise ValueError(gen)


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_config_counts_match_reference(xgm, ctx, name):
    rec = CONFIGS[name]
    nv, src, dst = _samples(xgm, rec)
    g = ctx.graph_from_edges(nv, src, dst)
    del src, dst
    try:
        rowptr, col = g.download()
        assert csr_digest(rowptr, col) == rec["csr_sha256"], "not the graph the reference counted"
        del rowptr, col
        info = g.info()
        assert (info["V"], info["E"], info["E_dag"]) == (rec["V"], rec["E"], rec["E_dag"])
        learned = xgm.trained_schedule(ctx)
        for kind, want in sorted(rec["counts"].items()):
            pattern = KIND_TO_PATTERN[kind]
            assert ctx.count(g, pattern) == want, f"{name} {kind} (heuristic)"
            if learned:
                assert ctx.count(g, pattern, **learned) == want, f"{name} {kind} (learned)"
    finally:
        g.close()

"""Generates tests/golden/batch_counts.json: per-graph counts of the 4096-graph batch.

The batch of the batched-counting workload: 4096 Barabasi-Albert graphs, n drawn
log-uniformly in [100, 5000], m uniform in {3..8}, seed 5 (oracle/gen.c, the same samples
as the engine's generator).  Per graph, the oracle (oracle/oracle.c, pinned to the
reference's own binaries on Barabasi-Albert graphs in golden_counts.json) counts
triangles and 4-cliques on the degree-oriented DAG and edge-induced diamonds on the
undirected graph.  The file holds the per-pattern totals and the sha256 of the
[graphs x 3] little-endian uint64 count array (triangle, 4-clique, diamond per graph),
which bench.py compares with the batched launch's output.

    python tests/golden/make_batch_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "batch_counts.json")
PATTERNS = ["triangle", "4-clique", "diamond"]


def main() -> None:
    graphs = 4096
    vo, eo, src, dst = oracle.gen_ba_batch(graphs, 100, 5000, 3, 8, seed=5)
    out = np.zeros((graphs, 3), dtype=np.uint64)
    for gi in range(graphs):
        lo, hi = int(vo[gi]), int(vo[gi + 1])
        s = src[eo[gi]:eo[gi + 1]] - lo
        d = dst[eo[gi]:eo[gi + 1]] - lo
        rowptr, col = oracle.build_csr(hi - lo, s, d)
        drow, dcol = oracle.orient(rowptr, col)
        out[gi] = [oracle.count("tc", drow, dcol), oracle.count("clique4", drow, dcol),
                   oracle.count("diamond", rowptr, col)]
    rec = {"graphs": graphs, "generator": "Barabasi-Albert batch, n in [100, 5000] "
                                          "log-uniform, m in {3..8}, seed 5",
           "patterns": PATTERNS,
           "totals": {p: int(out[:, i].sum()) for i, p in enumerate(PATTERNS)},
           "per_graph_sha256": hashlib.sha256(out.astype("<u8").tobytes()).hexdigest(),
           "source": "oracle (oracle/oracle.c), per graph"}
    with open(OUT, "w") as f:
        json.dump(rec, f, indent=1)
    print(rec)


if __name__ == "__main__":
    main()

"""Command-line counter, the engine's counterpart of the reference's solver binaries.

    python x-gminer_gb300/xgm_count.py --graph <prefix> --pattern 4-clique
    python x-gminer_gb300/xgm_count.py --rmat 21 --pattern 5-clique [--policy heuristic]

Mirrors `clique_omp_base <graph> <k>` / `count_omp_base <graph> <pattern>`
(codes/GraphMiner/src/{clique,count}/main.cc) and xgminer's `--graph --patternID`
(xgminer/include/cmd_option.h:30-159): loads a graph in the reference's binary CSR
layout (or generates a seeded R-MAT), counts one pattern on the GPU and prints the
count with the call's device timings as one JSON line.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
xgm = importlib.import_module("x-gminer_gb300")

# xgminer patternIDs (xgminer/include/common.h:185-208): 1-3 the count-app shapes, the
# GraphPi shapes by their names in xgminer/src/pattern_graphpi.cpp:60-146 (edge-induced,
# as GraphPi counts them; 6-vertex ones as adjacency matrices), and GLUMIN's P1-P24
# (glumin.h:34-39 maps patternID - 16 to the P-number)
PATTERN_IDS = {1: "triangle", 2: "rectangle", 3: "diamond", 10: "diamond", 11: "5-cycle",
               13: "5-house"}
PATTERN_IDS.update({i: f"P{i - 16}" for i in range(17, 41)})
GRAPHPI_6 = {14: [(0, 1), (0, 2), (0, 4), (1, 2), (1, 5), (2, 3), (3, 4), (3, 5), (4, 5)],
             15: [(0, 1), (0, 2), (1, 2), (1, 3), (1, 4), (2, 3), (2, 5), (0, 4), (0, 5)]}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    src = ap.add_mutually_exclusive_group(required=True)
    src.add_argument("--graph", help="prefix of <prefix>.meta.txt / .vertex.bin / .edge.bin")
    src.add_argument("--rmat", type=int, metavar="SCALE", help="seeded R-MAT, edge factor 16")
    src.add_argument("--er", type=int, nargs=2, metavar=("N", "M"),
                     help="seeded Erdos-Renyi G(N, M) edge samples")
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--pattern", default="4-clique")
    ap.add_argument("--patternID", type=int,
                    help="xgminer pattern id: 1-3, 10, 11, 13-15 (GraphPi shapes), "
                         "17-40 = GLUMIN P1-P24")
    ap.add_argument("--policy", choices=["heuristic", "learned"], default="heuristic")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--hub-max", type=int, default=0,
                    help="hub kernel bound (xgm_sched.hub_max; -1: split every hub)")
    args = ap.parse_args()
    if args.patternID and args.patternID not in PATTERN_IDS and args.patternID not in GRAPHPI_6:
        raise SystemExit(f"patternID {args.patternID} is not a supported plan "
                         f"(supported: {sorted(list(PATTERN_IDS) + list(GRAPHPI_6))})")
    if args.patternID in GRAPHPI_6:
        import numpy as np

        pattern = np.zeros((6, 6), dtype=np.uint8)
        for u, v in GRAPHPI_6[args.patternID]:
            pattern[u, v] = pattern[v, u] = 1
    else:
        pattern = PATTERN_IDS[args.patternID] if args.patternID else args.pattern
    ctx = xgm.Context(0)
    if args.graph:
        g = ctx.load_graph(args.graph)
    elif args.er:
        nv, s, d = xgm.gen_er(args.er[0], args.er[1], seed=args.seed)
        g = ctx.graph_from_edges(nv, s, d)
    else:
        nv, s, d = xgm.gen_rmat(args.rmat, 16, seed=args.seed)
        g = ctx.graph_from_edges(nv, s, d)
    kw = {}
    if args.policy == "learned":
        kw = xgm.trained_schedule(ctx)
        if not kw:
            raise SystemExit("costmodel.json is absent or was trained for another feature "
                             "layout; retrain it with x-gminer_gb300/train_costmodel.py")
    kw["hub_max"] = args.hub_max
    for _ in range(args.repeat):
        count, st = ctx.count(g, xgm.plan(pattern), with_stats=True, **kw)
        name = pattern if isinstance(pattern, str) else f"patternID {args.patternID}"
        print(json.dumps({"pattern": name, "count": count, "graph": g.info(), **st}))
    ctx.close()


if __name__ == "__main__":
    main()

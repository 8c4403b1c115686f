"""Generates tests/golden/golden_counts.json.

For each seeded synthetic graph below, the edge samples come from the engine's host
generators (integer-only, identical on x86-64 and aarch64), the CSR from the oracle's
CSR build, and every count from the reference's OWN OpenMP binaries (oracle/_ref,
built from the reference sources by oracle/build_ref.sh) run on the graph files:
tc/clique/count omp_base for the six plans, motif_omp_formula for the k = 3 and k = 4
vertex-induced motif census ("motif3", "motif4", in the reference's output order).  The
oracle restatement is cross-checked on the way.  On the graphs listed in GLUMIN5_CASES,
"glumin5" holds GLUMIN's 5-vertex plans P6..P22: P7, P10, P13, P15 and P20 from the
reference's own CPU plans (glumin_pattern_cpu, list and LUT forms, which must agree
with the oracle), the others from the oracle's restatement of the generated kernels.  A sha256 of the CSR bytes lets the
GPU tests confirm they regenerated the same graph.

Run from the repository root (needs the reference tree for oracle/_ref):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import importlib
import json
import os
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

xgm = importlib.import_module("x-gminer_gb300")

CASES = [
    {"name": "rmat_s10_ef16", "gen": "rmat", "args": [10, 16], "seed": 1},
    {"name": "rmat_s12_ef8", "gen": "rmat", "args": [12, 8], "seed": 3},
    {"name": "rmat_s14_ef16", "gen": "rmat", "args": [14, 16], "seed": 2},
    {"name": "er_n4096_m40000", "gen": "er", "args": [4096, 40000], "seed": 3},
    {"name": "ba_n3000_m5", "gen": "ba", "args": [3000, 5], "seed": 4},
    {"name": "ba_n200_m8", "gen": "ba", "args": [200, 8], "seed": 9},
]
KINDS = ["tc", "clique4", "clique5", "diamond", "cycle4", "tailed"]
GLUMIN5_CASES = {"rmat_s10_ef16", "er_n4096_m40000", "ba_n3000_m5", "ba_n200_m8"}


def samples(case):
    g, a, seed = case["gen"], case["args"], case["seed"]
    if g == "rmat":
        return xgm.gen_rmat(a[0], a[1], seed=seed)
    if g == "er":
        return xgm.gen_er(a[0], a[1], seed=seed)
    if g == "ba":
        return xgm.gen_ba(a[0], a[1], seed=seed)
    raise ValueError(g)


def csr_digest(rowptr, col) -> str:
    h = hashlib.sha256()
    h.update(rowptr.astype("<i8").tobytes())
    h.update(col.astype("<i4").tobytes())
    return h.hexdigest()


def main() -> None:
    if not oracle.build_ref():
        raise SystemExit("reference binaries unavailable (needs the reference tree)")
    out = []
    tmp = tempfile.mkdtemp()
    for case in CASES:
        nv, src, dst = samples(case)
        rowptr, col = oracle.build_csr(nv, src, dst)
        drow, dcol = oracle.orient(rowptr, col)
        prefix = os.path.join(tmp, case["name"])
        oracle.write_graph(prefix, rowptr, col)
        counts = {}
        for k in KINDS:
            ref, _ = oracle.run_ref(k, prefix)
            mine = oracle.count(k, drow, dcol) if k in ("tc", "clique4", "clique5") else \
                oracle.count(k, rowptr, col)
            if ref != mine:
                raise SystemExit(f"{case['name']} {k}: reference {ref} != oracle {mine}")
            counts[k] = ref
        for k in (3, 4):  # vertex-induced motif census, motif_omp_formula
            ref = oracle.run_ref_motif(k, prefix)
            mine = oracle.motif(k, rowptr, col)
            if ref != mine:
                raise SystemExit(f"{case['name']} motif{k}: reference {ref} != oracle {mine}")
            counts[f"motif{k}"] = ref
        if case["name"] in GLUMIN5_CASES:
            g5 = {}
            for pid in range(6, 23):
                mine = oracle.glumin5(pid, rowptr, col)
                if pid in oracle.GLUMIN5_CPU:
                    for lut in (False, True):
                        try:
                            ref, _ = oracle.run_ref_glumin5(pid, prefix, lut)
                        except RuntimeError:
                            # the LUT form of P20 (LUT_5anti_tailed_diamond) aborts with
                            # heap corruption on rmat_s10_ef16; the list form is the pin
                            if not lut:
                                raise
                            print(f"  {case['name']} P{pid}: reference LUT form failed")
                            continue
                        if ref != mine:
                            raise SystemExit(f"{case['name']} P{pid}: reference {ref} != "
                                             f"oracle {mine}")
                g5[f"P{pid}"] = mine
            counts["glumin5"] = g5
        rec = dict(case)
        rec.update({"V": int(nv), "E": int(len(col)), "E_dag": int(len(dcol)),
                    "csr_sha256": csr_digest(rowptr, col), "counts": counts,
                    "source": "oracle/_ref reference OpenMP binaries"})
        out.append(rec)
        print(case["name"], counts)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_counts.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()

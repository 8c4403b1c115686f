"""Generates tests/golden/config_counts.json: counts at the benchmark configurations.

Each configuration graph is generated by the oracle's seeded generators (oracle/gen.c,
the same samples as the engine's), built into the reference's binary CSR format by the
oracle's CSR build, and counted by the reference's OWN OpenMP binaries (oracle/_ref,
built from the reference sources by oracle/build_ref.sh):

  triangle       tc_omp_base      codes/GraphMiner/src/triangle/omp_base.cc:5-26
  4/5-clique     clique_omp_base  codes/GraphMiner/src/clique/omp_base.cc:20-36
                                  (automine_4clique / automine_5clique,
                                  src/clique/cpu_kernels/clique_base.h:53-68, 95-)
  diamond / 4-cycle / tailed triangle (edge-induced)
                 count_omp_base   codes/GraphMiner/src/count/omp_base.cc:5-58

The reference binaries orient the graph themselves (src/common/graph.cc:233-275).  A
sha256 of the CSR bytes lets the GPU tests confirm that they regenerated the same
graph.  Each (config, pattern) pair is one job; results are merged into the JSON file
as they finish, so long jobs (5-cliques at R-MAT scale 22) can run separately:

    python tests/golden/make_config_golden.py                # every job not yet done
    python tests/golden/make_config_golden.py --job rmat_s22_ef16_seed2:clique5
    python tests/golden/make_config_golden.py --list

Needs the reference tree (for oracle/_ref) and an x86-64 host with AVX2 for
count_omp_base.
"""
from __future__ import annotations

import argparse
import fcntl
import hashlib
import json
import os
import platform
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "config_counts.json")

# name -> (generator, args, seed, kinds).  Sizes and seeds are the benchmark
# configurations: triangle on R-MAT s16; 4/5-clique on R-MAT s22; edge-induced motifs
# on Erdos-Renyi and Chung-Lu with 2^21 vertices; the held-out R-MAT s23 graph of the
# learned scheduler.
CONFIGS = {
    "rmat_s16_ef16_seed1": ("rmat", [16, 16], 1,
                            ["tc", "clique4", "clique5", "diamond", "cycle4", "tailed"]),
    "rmat_s22_ef16_seed2": ("rmat", [22, 16], 2, ["tc", "clique4", "diamond", "clique5"]),
    "er_n2097152_deg32_seed3": ("er", [1 << 21, 1 << 25], 3,
                                ["tc", "diamond", "cycle4", "tailed", "clique4"]),
    "chung_lu_n2097152_g2.1_w50000_deg32_seed4": ("chung_lu", [1 << 21, 2.1, 50000.0, 32.0], 4,
                                                  ["tc", "diamond", "cycle4", "tailed",
                                                   "clique4"]),
    "rmat_s23_ef16_seed99": ("rmat", [23, 16], 99, ["tc", "clique4", "diamond", "clique5"]),
}
DAG_KINDS = ("tc", "clique4", "clique5")


def samples(gen, args, seed):
    if gen == "rmat":
        return oracle.gen_rmat(args[0], args[1], seed=seed)
    if gen == "er":
        return oracle.gen_er(args[0], args[1], seed=seed)
    if gen == "chung_lu":
        return oracle.gen_chung_lu(*args, seed=seed)
    raise ValueError(gen)


def csr_digest(rowptr, col) -> str:
    h = hashlib.sha256()
    h.update(rowptr.astype("<i8").tobytes())
    h.update(col.astype("<i4").tobytes())
    return h.hexdigest()


def update(name: str, fn) -> None:
    """Read-modify-write of one config's record under a file lock."""
    lock = open(os.path.join(tempfile.gettempdir(), "xgm_config_counts.lock"), "w")
    fcntl.flock(lock, fcntl.LOCK_EX)
    try:
        data = json.load(open(OUT)) if os.path.exists(OUT) else {}
        fn(data.setdefault(name, {}))
        with open(OUT + ".tmp", "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(OUT + ".tmp", OUT)
    finally:
        fcntl.flock(lock, fcntl.LOCK_UN)
        lock.close()


def run_config(name: str, kinds) -> None:
    gen, args, seed, _ = CONFIGS[name]
    t0 = time.time()
    nv, src, dst = samples(gen, args, seed)
    rowptr, col = oracle.build_csr(nv, src, dst)
    del src, dst
    deg = rowptr[1:] - rowptr[:-1]
    info = {"gen": gen, "args": args, "seed": seed, "V": int(nv), "E": int(len(col)),
            "E_dag": int(len(col) // 2), "max_degree": int(deg.max()),
            "csr_sha256": csr_digest(rowptr, col)}
    print(f"{name}: V={nv} E={len(col)} maxdeg={int(deg.max())} built in "
          f"{time.time() - t0:.1f} s", flush=True)
    with tempfile.TemporaryDirectory() as tmp:
        prefix = os.path.join(tmp, name)
        oracle.write_graph(prefix, rowptr, col)
        del rowptr, col
        for k in kinds:
            t1 = time.time()
            cnt, secs = oracle.run_ref(k, prefix)
            wall = time.time() - t1
            print(f"  {k}: {cnt} (reference {secs:.2f} s, wall {wall:.1f} s)", flush=True)

            def put(rec, k=k, cnt=cnt, secs=secs):
                rec.update(info)
                rec.setdefault("counts", {})[k] = cnt
                rec.setdefault("reference_seconds", {})[k] = round(secs, 3)
                rec["source"] = ("oracle/_ref reference OpenMP binaries "
                                 f"({os.cpu_count()} threads, {platform.machine()})")
            update(name, put)


def main() -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--job", action="append", default=[],
                   help="config:kind (default: every job not yet in the file)")
    p.add_argument("--list", action="store_true")
    p.add_argument("--skip", action="append", default=[], help="kinds to leave out")
    a = p.parse_args()
    done = json.load(open(OUT)) if os.path.exists(OUT) else {}
    jobs = []
    if a.job:
        for j in a.job:
            c, k = j.split(":")
            jobs.append((c, k))
    else:
        for c, (_, _, _, kinds) in CONFIGS.items():
            for k in kinds:
                if k not in a.skip and k not in done.get(c, {}).get("counts", {}):
                    jobs.append((c, k))
    if a.list:
        for j in jobs:
            print(":".join(j))
        return
    if not oracle.build_ref():
        raise SystemExit("reference binaries unavailable (needs the reference tree)")
    by_cfg = {}
    for c, k in jobs:
        by_cfg.setdefault(c, []).append(k)
    for c, kinds in by_cfg.items():
        run_config(c, kinds)


if __name__ == "__main__":
    main()

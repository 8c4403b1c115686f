#!/usr/bin/env python3
"""Benchmark: exact k-clique counting on one GB300, matches/s and GTEPS.

Workload (the k-clique configuration): R-MAT scale 22 (4,194,304 vertices), edge factor
16 (67,108,864 samples), (a,b,c,d) = (0.57,0.19,0.19,0.05), seed 2; symmetrised,
deduplicated, self-loops removed, degree-oriented DAG (ties by id), int32 CSR.  Seeded
synthetic data stands in for the reference's real-world graphs.

A step is one exact count of the pattern (default 4-clique) over the whole graph through
the engine: task generation (schedule) + the persistent counting launch, graph resident
in HBM.  `value` is matches/s from CUDA-event device time; `e2e` is the same metric
through the C ABI from host CSR buffers (pinned), host->device copy, GPU orientation,
count and the 8-byte result read inside the timed region.

  python bench.py [--gpus N --steps K --warmup W] [--impl engine|reference]
                  [--pattern 4-clique|5-clique] [--policy learned|heuristic]

--impl reference times the reference's CPU counting algorithm (oracle port of the
G2Miner OpenMP path, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {"graph": "rmat", "scale": 22, "edge_factor": 16, "abcd": [0.57, 0.19, 0.19, 0.05],
            "seed": 2}
PATTERN_KIND = {"4-clique": "clique4", "5-clique": "clique5", "triangle": "tc"}
COSTMODEL = os.path.join(ROOT, "x-gminer_gb300", "costmodel.json")
L2_BYTES = 129 * 1024 * 1024


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="engine", choices=["engine", "reference"])
    p.add_argument("--pattern", default="4-clique", choices=list(PATTERN_KIND))
    p.add_argument("--policy", default="learned", choices=["learned", "heuristic"])
    p.add_argument("--scale", type=int, default=WORKLOAD["scale"])
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--workload", default="clique",
                   choices=["clique", "batch", "motifs", "patterns5"],
                   help="clique: k-clique counting on R-MAT s22; batch: 4096 BA graphs; "
                        "motifs: edge-induced 4-vertex motifs on ER and Chung-Lu 2^21; "
                        "patterns5: GLUMIN's 5-vertex plans P6-P22 on R-MAT s12 and ER 2^16")
    p.add_argument("--graphs", type=int, default=4096)
    return p.parse_args()


# ------------------------------------------------------------------ distributed
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            backend = "nccl" if _cuda_ok() else "gloo"
            td.init_process_group(backend)
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, x: float, op: str) -> float:
        if not self.pg:
            return x
        import torch

        dev = f"cuda:{self.local}" if _cuda_ok() else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def _cuda_ok() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def _sync():
    if _cuda_ok():
        import torch

        torch.cuda.synchronize()


# ----------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------- helpers
def load_engine():
    return importlib.import_module("x-gminer_gb300")


def load_model(xgm, ctx):
    """The trained cost model (x-gminer_gb300/costmodel.json) and its schedule settings
    (queue order, margin) as count() keyword arguments."""
    if not os.path.exists(COSTMODEL):
        return None, {}
    with open(COSTMODEL) as f:
        spec = json.load(f)
    if (spec.get("features") != xgm.MODEL_FEATURES or spec.get("variants") != xgm.NUM_VARIANTS
            or len(spec["params"]) != xgm.MODEL_PARAMS):
        return None, {}  # trained for another feature layout: fall back to the heuristic
    import numpy as np

    m = xgm.Model(ctx)
    m.set_params(np.asarray(spec["params"], dtype=np.float32))
    return m, {"order_by_cost": int(spec.get("order_by_cost", 1)),
               "margin": float(spec.get("margin", 0.0))}


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic(pattern: str):
    """dram bytes per launch of the counting kernel from the committed ncu summary."""
    name = {"4-clique": "k_clique4", "5-clique": "k_clique5", "triangle": "k_clique3"}[pattern]
    path = os.path.join(ROOT, "profiles", f"{name}_rmat_s22.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return int(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def cpu_sample(orc, kind: str, drow, dcol, budget_s: float):
    """Times the oracle port on every `stride`-th top-level vertex (all host threads),
    with the stride picked from a short calibration so the sample takes ~budget_s."""
    nv = len(drow) - 1
    cores = orc.threads()
    # halve a power-of-two stride (nested samples: every 2^k-th vertex) until the sample
    # takes at least half the budget; that sample is the measurement
    stride = 1 << 20
    while True:
        t0 = time.perf_counter()
        c = orc.count(kind, drow, dcol, 0, nv, stride)
        dt = time.perf_counter() - t0
        if dt >= budget_s / 2 or stride == 1:
            return c, dt, stride, cores
        stride //= 2


def gen_graph(xgm, scale):
    a, b, c, _ = WORKLOAD["abcd"]
    return xgm.gen_rmat(scale, WORKLOAD["edge_factor"], a, b, c, seed=WORKLOAD["seed"])


# ------------------------------------------------------------------- engine arm
def engine_arm(args, dist: Dist) -> None:
    import numpy as np
    import torch

    xgm = load_engine()
    torch.cuda.set_device(dist.local)
    ctx = xgm.Context(dist.local)
    nv, src, dst = gen_graph(xgm, args.scale)
    g = ctx.graph_from_edges(nv, src, dst)
    del src, dst
    info = g.info()
    model, mkw = load_model(xgm, ctx) if args.policy == "learned" else (None, {})
    policy = xgm.SCHED_LEARNED if model is not None else xgm.SCHED_HEURISTIC
    kw = {"policy": policy, "model": model, **mkw}

    def run(n, **k):
        prep, kern, cnt = [], [], None
        for _ in range(n):
            cnt, st = ctx.count(g, args.pattern, with_stats=True, **k)
            prep.append(st["prep_ms"])
            kern.append(st["kernel_ms"])
        return cnt, prep, kern

    run(args.warmup, **kw)
    dist.barrier()
    _sync()
    clocks = ClockSampler(dist.local)
    clocks.start()
    t0 = time.perf_counter()
    count, prep, kern = run(args.steps, **kw)
    _sync()
    wall = time.perf_counter() - t0
    dist.barrier()
    clk = clocks.stop()
    step_ms = [p + k for p, k in zip(prep, kern)]
    ms_per_step = dist.reduce(sum(step_ms) / args.steps, "max")
    total_matches = dist.reduce(float(count), "sum")
    value = total_matches / (ms_per_step / 1e3)
    kern_ms = statistics.mean(kern)

    # plain heuristic schedule on the same graph and steps (the baseline of the learned schedule)
    plain = None
    if policy == xgm.SCHED_LEARNED:
        run(1, policy=xgm.SCHED_HEURISTIC)
        c2, p2, k2 = run(args.steps, policy=xgm.SCHED_HEURISTIC)
        assert c2 == count, "schedules disagree on the count"
        pms = dist.reduce(sum(p + k for p, k in zip(p2, k2)) / args.steps, "max")
        plain = {"matches_per_s": total_matches / (pms / 1e3), "ms_per_step": pms,
                 "kernel_ms": statistics.mean(k2)}

    launches = ctx.count_kernels(g, args.pattern, **kw)
    peaks = measured_peaks()
    algo = ctx.algo_bytes(g, args.pattern)
    achieved = algo / (kern_ms / 1e3) / 1e9
    traffic = profile_traffic(args.pattern)
    line = {
        "metric": "matches_per_sec",
        "value": value,
        "unit": "matches/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32 ids / uint64 counts",
        "data": "synthetic (seeded R-MAT, engine host generator)",
        "config": {"workload": f"{args.pattern} counting, R-MAT scale {args.scale} edge factor 16",
                   "pattern": args.pattern, "graph": dict(WORKLOAD, scale=args.scale),
                   "V": info["V"], "E_undirected_entries": info["E"], "E_dag": info["E_dag"],
                   "max_degree": info["max_degree"], "max_out_degree": info["max_out_degree"],
                   "schedule": "learned" if policy == xgm.SCHED_LEARNED else "heuristic",
                   "parallelism": f"replicas x{dist.world}",
                   "l2": "inputs larger than L2 (adjacency %.0f MB > 129 MB)" % (info["E"] * 4 / 2**20)},
        "count": count,
        "gteps": info["E_dag"] / (ms_per_step / 1e3) / 1e9,
        "kernel_ms": kern_ms,
        "prep_ms": statistics.mean(prep),
        "wall_ms_per_step": wall * 1e3 / args.steps,
        "plain_heuristic": plain,
        "gpu_launches": launches * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                     "traffic": traffic, "algo_bytes_per_launch": algo,
                     # the measured DRAM traffic of the launch over its time: what the
                     # kernel actually moves (it reads each list once per task)
                     "dram_gbs": (traffic / (kern_ms / 1e3) / 1e9) if traffic else None,
                     "dram_frac": (traffic / (kern_ms / 1e3) / 1e9 / peaks["hbm_gbs"])
                     if traffic else None,
                     "peak_source": peaks["source"]},
        "clocks": clk,
    }

    # end to end through the C ABI from pinned host buffers
    if not args.no_e2e:
        rowptr, col = g.download()
        rp = torch.empty(len(rowptr), dtype=torch.int64, pin_memory=True)
        cp = torch.empty(len(col), dtype=torch.int32, pin_memory=True)
        rp.numpy()[:] = rowptr
        cp.numpy()[:] = col
        del rowptr, col
        g.close()
        e2e_t = []
        for i in range(args.warmup + args.steps):
            _sync()
            t0 = time.perf_counter()
            ge = ctx.graph_from_csr(rp.numpy(), cp.numpy())
            c3 = ctx.count(ge, args.pattern, **kw)
            ge.close()
            _sync()
            if i >= args.warmup:
                e2e_t.append(time.perf_counter() - t0)
            assert c3 == count
        e2e_s = dist.reduce(sum(e2e_t) / len(e2e_t), "max")
        line["e2e"] = {"value": total_matches / e2e_s, "unit": "matches/s",
                       "h2d_bytes_per_step": int(rp.numel() * 8 + cp.numel() * 4),
                       "d2h_bytes_per_step": 8, "ms_per_step": e2e_s * 1e3}
        g = None

    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        import oracle

        if g is None:
            rowptr, col = rp.numpy(), cp.numpy()
        else:
            rowptr, col = g.download()
        drow, dcol = oracle.orient(rowptr, col)
        c, dt, stride, cores = cpu_sample(oracle, PATTERN_KIND[args.pattern], drow, dcol,
                                          args.cpu_seconds)
        line["cpu_baseline"] = {"value": c / dt, "unit": "matches/s", "cores": cores,
                                "kind": "port",
                                "sample": f"every {stride}-th top-level vertex of the same DAG "
                                          f"({c} matches in {dt:.2f} s, OpenMP oracle port)"}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


# ------------------------------------------------------------------- batch arm
BATCH_PATTERNS = ["triangle", "4-clique", "diamond"]


def batch_arm(args, dist: Dist) -> None:
    """Batched multi-graph counting: Barabasi-Albert graphs, n log-uniform in
    [100, 5000], m uniform in {3..8}, seed 5; triangle + 4-clique + diamond per graph in
    one persistent launch replayed as a CUDA graph.  Compared with the same counts made
    by one xgm_count call per (graph, pattern)."""
    import numpy as np
    import torch

    xgm = load_engine()
    torch.cuda.set_device(dist.local)
    ctx = xgm.Context(dist.local)
    vo, eo, src, dst = xgm.gen_ba_batch(args.graphs, 100, 5000, 3, 8, seed=5)
    b = ctx.batch_from_edges(vo, src, dst)
    model, mkw = load_model(xgm, ctx)
    tune = ctx.autotune(b, BATCH_PATTERNS, reps=3)
    runs = {"heuristic": {}, "tuned": {"policy": xgm.SCHED_TUNED, "table": tune["table"]}}
    if model is not None:
        runs["learned"] = {"policy": xgm.SCHED_LEARNED, "model": model, **mkw}
    res, ref, kernels = {}, None, {}
    clocks = ClockSampler(dist.local)
    clocks.start()
    for name, kw in runs.items():
        for _ in range(args.warmup):
            ctx.count_batched(b, BATCH_PATTERNS, **kw)
        _sync()
        ms = []
        for _ in range(args.steps):
            out, st = ctx.count_batched(b, BATCH_PATTERNS, with_stats=True, **kw)
            ms.append(st["kernel_ms"])
            kernels[name] = st["launches"]  # kernel nodes of the replayed CUDA graph
        if ref is None:
            ref = out
        assert np.array_equal(out, ref), f"{name} schedule changed a count"
        res[name] = statistics.mean(ms)
    clk = clocks.stop()
    total = float(ref.astype(np.float64).sum())
    best = min(res, key=res.get)
    # per-graph calls on a sample of graphs, scaled to the whole batch
    sample = list(range(0, args.graphs, max(1, args.graphs // 256)))
    loop_s, loop_matches, loop_graphs = 0.0, 0, 0
    for gi in sample:
        lo, hi = int(vo[gi]), int(vo[gi + 1])
        g = ctx.graph_from_edges(hi - lo, src[eo[gi]:eo[gi + 1]] - lo, dst[eo[gi]:eo[gi + 1]] - lo)
        _sync()
        t0 = time.perf_counter()
        for p, pat in enumerate(BATCH_PATTERNS):
            c = ctx.count(g, pat)
            assert c == int(ref[gi, p])
            loop_matches += c
        loop_s += time.perf_counter() - t0
        loop_graphs += 1
        g.close()
    loop_ms_full = loop_s * 1e3 * args.graphs / loop_graphs
    line = {"metric": "matches_per_sec", "value": total / (res[best] / 1e3), "unit": "matches/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": res[best],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 ids / uint64 counts", "data": "synthetic (seeded Barabasi-Albert)",
            "config": {"workload": f"batched counting, {args.graphs} BA graphs, "
                                   "triangle + 4-clique + diamond per graph",
                       "graphs": args.graphs, "vertices": int(vo[-1]), "samples": int(len(src)),
                       "schedule": best},
            "schedules_ms": res, "tuned_variants": tune["variants"],
            "per_graph_calls_ms_estimate": loop_ms_full,
            "speedup_vs_per_graph_calls": loop_ms_full / res[best],
            "count_total": int(total), "gpu_launches": kernels[best] * args.steps,
            "clocks": clk}
    print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------- reference arm
def reference_arm(args, dist: Dist) -> None:
    if dist.rank != 0:
        return
    import oracle

    xgm = load_engine()  # host generator only (no GPU use)
    nv, src, dst = gen_graph(xgm, args.scale)
    rowptr, col = oracle.build_csr(nv, src, dst)
    del src, dst
    drow, dcol = oracle.orient(rowptr, col)
    kind = PATTERN_KIND[args.pattern]
    per_step = max(2.0, min(args.cpu_seconds, 150.0 / max(1, args.steps + args.warmup)))
    c, dt, stride, cores = cpu_sample(oracle, kind, drow, dcol, per_step)
    times, counts = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        ci = oracle.count(kind, drow, dcol, 0, nv, stride)
        t = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(t)
            counts.append(ci)
    ms = statistics.mean(times) * 1e3
    value = counts[-1] / (ms / 1e3)
    sample = (f"every {stride}-th top-level vertex of the R-MAT s{args.scale} DAG "
              f"({counts[-1]} matches per step); oracle port of the OpenMP path")
    line = {"metric": "matches_per_sec", "value": value, "unit": "matches/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 ids / uint64 counts", "data": "synthetic (seeded R-MAT)",
            "config": {"workload": f"{args.pattern} counting, R-MAT scale {args.scale} edge factor 16",
                       "pattern": args.pattern, "graph": dict(WORKLOAD, scale=args.scale)},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "matches/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "matches/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


MOTIF_PATTERNS = ["diamond", "rectangle", "tailedtriangle", "4-clique"]


def motifs_arm(args, dist: Dist) -> None:
    """Edge-induced diamond / 4-cycle / tailed triangle / 4-clique on an Erdos-Renyi
    G(n = 2^21, average degree 32) and a Chung-Lu power-law graph (n = 2^21, exponent
    2.1, maximum expected degree 50,000), seeded.  One step counts all four patterns on
    both graphs; matches/s = total count / total device time."""
    import torch

    xgm = load_engine()
    torch.cuda.set_device(dist.local)
    ctx = xgm.Context(dist.local)
    n = 1 << 21
    graphs = {"er": xgm.gen_er(n, n * 16, seed=31),
              "chung_lu": xgm.gen_chung_lu(n, 2.1, 50000.0, 32.0, seed=32)}
    model, mkw = load_model(xgm, ctx) if args.policy == "learned" else (None, {})
    kw = {"policy": xgm.SCHED_LEARNED, "model": model, **mkw} if model is not None else {}
    per, total_ms, total_matches, info, launches = {}, 0.0, 0, {}, 0
    clocks = ClockSampler(dist.local)
    clocks.start()
    for gname, (nv, src, dst) in graphs.items():
        g = ctx.graph_from_edges(nv, src, dst)
        info[gname] = g.info()
        for pat in MOTIF_PATTERNS:
            for _ in range(args.warmup):
                ctx.count(g, pat, **kw)
            _sync()
            ms, cnt = [], 0
            for _ in range(args.steps):
                cnt, st = ctx.count(g, pat, with_stats=True, **kw)
                ms.append(st["kernel_ms"] + st["prep_ms"])
                launches += st["launches"]
            per[f"{gname}/{pat}"] = {"count": cnt, "ms": statistics.mean(ms)}
            total_ms += statistics.mean(ms)
            total_matches += cnt
        g.close()
    clk = clocks.stop()
    line = {"metric": "matches_per_sec", "value": total_matches / (total_ms / 1e3),
            "unit": "matches/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32 ids / uint64 counts",
            "data": "synthetic (seeded Erdos-Renyi and Chung-Lu)",
            "config": {"workload": "edge-induced 4-vertex motifs, ER 2^21 deg 32 and "
                                   "Chung-Lu 2^21 gamma 2.1 dmax 50k",
                       "schedule": "learned" if model is not None else "heuristic",
                       "graphs": info},
            "gpu_launches": launches // max(1, args.steps), "clocks": clk, "per_pattern": per}
    print(json.dumps(line), flush=True)
    ctx.close()


def patterns5_arm(args, dist: Dist) -> None:
    """GLUMIN's vertex-induced 5-vertex plans P6..P22 (set-operation programs) on an
    R-MAT graph (scale 12, edge factor 8, seed 3; maximum degree 941) and an Erdos-Renyi
    G(n = 2^16, average degree 16), seeded.  One step counts all 17 plans on both graphs;
    matches/s = total count / total device time.  CPU baseline: the oracle's restatement
    of the same plans on the host cores, every plan on the ER graph."""
    import torch

    xgm = load_engine()
    torch.cuda.set_device(dist.local)
    ctx = xgm.Context(dist.local)
    graphs = {"rmat_s12_ef8": xgm.gen_rmat(12, 8, seed=3),
              "er_2^16_deg16": xgm.gen_er(1 << 16, 1 << 19, seed=3)}
    per, total_ms, total_matches, info, launches = {}, 0.0, 0, {}, 0
    clocks = ClockSampler(dist.local)
    clocks.start()
    for gname, (nv, src, dst) in graphs.items():
        g = ctx.graph_from_edges(nv, src, dst)
        info[gname] = g.info()
        for pid in range(6, 23):
            pat = f"P{pid}"
            for _ in range(args.warmup):
                ctx.count(g, pat)
            _sync()
            ms, cnt = [], 0
            for _ in range(args.steps):
                cnt, st = ctx.count(g, pat, with_stats=True)
                ms.append(st["kernel_ms"] + st["prep_ms"])
                launches += st["launches"]
            per[f"{gname}/{pat}"] = {"count": cnt, "ms": statistics.mean(ms)}
            total_ms += statistics.mean(ms)
            total_matches += cnt
        g.close()
    clk = clocks.stop()
    line = {"metric": "matches_per_sec", "value": total_matches / (total_ms / 1e3),
            "unit": "matches/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32 ids / uint64 counts",
            "data": "synthetic (seeded R-MAT and Erdos-Renyi)",
            "config": {"workload": "GLUMIN P6-P22 (vertex-induced 5-vertex plans), R-MAT s12 "
                                   "ef8 and ER 2^16 deg 16", "graphs": info},
            "gpu_launches": launches // max(1, args.steps), "clocks": clk,
            "per_pattern": per}
    if dist.rank == 0 and not args.no_cpu_baseline:
        import oracle

        nv, src, dst = graphs["er_2^16_deg16"]
        rowptr, col = oracle.build_csr(nv, src, dst)
        cores = oracle.threads()
        t0 = time.perf_counter()
        c = sum(oracle.glumin5(pid, rowptr, col) for pid in range(6, 23))
        dt = time.perf_counter() - t0
        gpu_ms = sum(v["ms"] for k, v in per.items() if k.startswith("er_"))
        line["cpu_baseline"] = {"value": c / dt, "unit": "matches/s", "cores": cores,
                                "kind": "port",
                                "sample": f"P6-P22 on the ER graph ({c} matches in {dt:.2f} s, "
                                          f"OpenMP oracle port; the GPU took {gpu_ms:.1f} ms)"}
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            reference_arm(args, dist)
        elif args.workload == "batch":
            batch_arm(args, dist)
        elif args.workload == "motifs":
            motifs_arm(args, dist)
        elif args.workload == "patterns5":
            patterns5_arm(args, dist)
        else:
            engine_arm(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()

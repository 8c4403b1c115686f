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
count and the 8-byte result read inside the timed region.  Every count is checked
against the reference binaries' count of the same graph (tests/golden/config_counts.json)
where the fixture holds it.

The default line also carries `clique5` (the 5-clique half of the configuration, learned
vs plain heuristic schedule on the same resident graph) and `batch` (4096 Barabasi-Albert
graphs, triangle + 4-clique + diamond per graph in one replayed CUDA graph: plain
heuristic / autotuned / learned schedules, per-graph counts checked against the
committed fixture).

  python bench.py [--gpus N --steps K --warmup W] [--impl engine|reference]
                  [--pattern 4-clique|5-clique|triangle] [--policy learned|heuristic]
                  [--workload clique|batch|motifs|patterns5]

--impl reference times the reference's CPU counting algorithm (the oracle's restatement
of the G2Miner OpenMP path, all host threads) on a seeded uniform random sample of the
top-level vertices of the same graph, built by the oracle's own generator and CSR build
(the engine's library is not loaded).  The engine's `cpu_baseline` times the same sample.
"""
from __future__ import annotations

import argparse
import hashlib
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
CONFIG_FIXTURE = os.path.join(ROOT, "tests", "golden", "config_counts.json")
BATCH_FIXTURE = os.path.join(ROOT, "tests", "golden", "batch_counts.json")
L2_BYTES = 129 * 1024 * 1024
SAMPLE_SEED = 12345
# Fraction of the top-level vertices in the CPU sample, per (pattern, scale): about
# 4-5 s of the 16-core oracle per step at R-MAT scale 22.  Other cases calibrate.
SAMPLE_FRACTION = {("4-clique", 22): 1 / 16, ("triangle", 22): 1 / 2, ("5-clique", 22): 1 / 512,
                   ("4-clique", 16): 1.0, ("triangle", 16): 1.0}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="engine", choices=["engine", "reference"])
    p.add_argument("--pattern", default="4-clique", choices=list(PATTERN_KIND))
    p.add_argument("--policy", default="learned", choices=["learned", "heuristic"])
    p.add_argument("--scale", type=int, default=WORKLOAD["scale"])
    p.add_argument("--cpu-seconds", type=float, default=5.0,
                   help="target seconds of one CPU sample where no fraction is fixed")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-clique5", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--workload", default="clique",
                   choices=["clique", "batch", "motifs", "patterns5", "ablation"],
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
        return self

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


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_summary(pattern: str, scale: int) -> dict:
    """`key: value` lines of the committed ncu summary of the counting kernel
    (profiles/k_clique<k>_rmat_s<scale>.md): DRAM traffic per launch and issue rate."""
    name = {"4-clique": "k_clique4", "5-clique": "k_clique5", "triangle": "k_clique3"}[pattern]
    path = os.path.join(ROOT, "profiles", f"{name}_rmat_s{scale}.md")
    out = {"path": os.path.relpath(path, ROOT)}
    if not os.path.exists(path):
        return out
    for line in open(path):
        if ":" not in line or line.startswith(("|", "#", " ")):
            continue
        k, v = line.split(":", 1)
        k = k.strip()
        if k in ("traffic_bytes_per_launch", "issue_active_pct", "threads_per_warp_inst",
                 "l2_hit_pct", "kernel_ms_under_ncu"):
            try:
                out[k] = float(v.strip().split()[0])
            except (ValueError, IndexError):
                pass
    return out


def fixture_counts(scale: int, seed: int) -> dict:
    """Reference-binary counts of the R-MAT graph (tests/golden/config_counts.json)."""
    if not os.path.exists(CONFIG_FIXTURE):
        return {}
    with open(CONFIG_FIXTURE) as f:
        data = json.load(f)
    return data.get(f"rmat_s{scale}_ef16_seed{seed}", {})


def check_count(fx: dict, kind: str, got: int) -> bool:
    """True when the fixture holds this count (and then it must match)."""
    want = fx.get("counts", {}).get(kind)
    if want is None:
        return False
    assert got == want, f"{kind}: engine {got} != reference binaries {want}"
    return True


def workload_config(args, V, E, E_dag, max_deg, max_out, world) -> dict:
    """The workload description; both arms print the same dict for the same run."""
    return {"workload": f"{args.pattern} counting, R-MAT scale {args.scale} edge factor 16",
            "pattern": args.pattern, "graph": dict(WORKLOAD, scale=args.scale),
            "V": int(V), "E_undirected_entries": int(E), "E_dag": int(E_dag),
            "max_degree": int(max_deg), "max_out_degree": int(max_out),
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (adjacency %.0f MB > 129 MB)" % (E * 4 / 2**20)}


def sample_fraction(orc, pattern: str, scale: int, kind: str, drow, dcol, budget_s: float):
    """Fraction of top-level vertices in the CPU sample: fixed per (pattern, scale) so
    both arms time the same sample; otherwise doubled from 2^-16 until one sample takes
    at least half the budget."""
    if (pattern, scale) in SAMPLE_FRACTION:
        return SAMPLE_FRACTION[(pattern, scale)]
    nv = len(drow) - 1
    f = 2.0 ** -16
    while f < 1.0:
        smp = orc.vertex_sample(nv, f, SAMPLE_SEED)
        t0 = time.perf_counter()
        orc.count(kind, drow, dcol, sample=smp)
        if time.perf_counter() - t0 >= budget_s / 2:
            return f
        f *= 2
    return 1.0


def cpu_sample(orc, pattern: str, scale: int, drow, dcol, budget_s: float, total: int = None,
               repeat: int = 1):
    """Times the oracle port (all host threads) on a seeded uniform random vertex sample.
    Returns (matches in the sample, seconds per run, description dict)."""
    kind = PATTERN_KIND[pattern]
    nv = len(drow) - 1
    frac = sample_fraction(orc, pattern, scale, kind, drow, dcol, budget_s)
    smp = orc.vertex_sample(nv, frac, SAMPLE_SEED)
    times, c = [], 0
    for _ in range(repeat):
        t0 = time.perf_counter()
        c = orc.count(kind, drow, dcol, sample=smp)
        times.append(time.perf_counter() - t0)
    work = orc.algo_bytes(kind, drow, dcol, sample=smp)
    work_all = orc.algo_bytes(kind, drow, dcol) if frac < 1.0 else work
    desc = {"fraction": frac, "vertices": int(len(smp)), "seed": SAMPLE_SEED,
            "matches": int(c), "plan_bytes_share": work / work_all if work_all else None}
    if total:
        desc["match_share"] = c / total
    return c, times, desc


def host_cpu() -> dict:
    """The host CPU the baseline ran on: model string (from /proc/cpuinfo where the kernel
    gives one) and the online core count."""
    import platform
    fields = {}
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if ":" in line:
                    k, v = line.split(":", 1)
                    fields.setdefault(k.strip().lower(), v.strip())
    except OSError:
        pass
    model = fields.get("model name") or fields.get("hardware") or ""
    if not model and "cpu part" in fields:  # Arm: implementer / part ids
        impl, part = fields.get("cpu implementer", "?"), fields["cpu part"]
        known = {("0x41", "0xd4f"): "Arm Neoverse V2"}  # the Grace host CPU
        model = known.get((impl, part), f"arm implementer {impl} part {part}")
    return {"model": model or platform.machine(), "machine": platform.machine(),
            "nproc": os.cpu_count()}


def sample_text(desc: dict, scale: int, dt: float) -> str:
    share = desc.get("match_share")
    return (f"seeded uniform random sample of {desc['fraction']:.6g} of the top-level vertices "
            f"of the R-MAT s{scale} DAG ({desc['vertices']} vertices, seed {desc['seed']}): "
            f"{desc['matches']} matches"
            + (f" = {share:.4f} of all matches" if share is not None else "")
            + (f", {desc['plan_bytes_share']:.4f} of the plan's work"
               if desc.get("plan_bytes_share") is not None else "")
            + f", {dt:.2f} s per run; oracle port of the G2Miner OpenMP path")


def gen_graph(mod, scale):
    a, b, c, _ = WORKLOAD["abcd"]
    return mod.gen_rmat(scale, WORKLOAD["edge_factor"], a, b, c, seed=WORKLOAD["seed"])


# ------------------------------------------------------------------- engine arm
def timed_counts(ctx, g, pattern, n, kw):
    prep, kern, cnt = [], [], None
    for _ in range(n):
        cnt, st = ctx.count(g, pattern, with_stats=True, **kw)
        prep.append(st["prep_ms"])
        kern.append(st["kernel_ms"])
    return cnt, prep, kern


def clique5_sub(xgm, ctx, g, learned, fx, local) -> dict:
    """5-clique on the resident graph: learned vs plain heuristic schedule."""
    clocks = ClockSampler(local).start()
    out = {}
    for name, kw in (("learned", learned), ("heuristic", {})):
        if name == "learned" and not kw:
            continue
        timed_counts(ctx, g, "5-clique", 1, kw)
        _sync()
        cnt, prep, kern = timed_counts(ctx, g, "5-clique", 2, kw)
        ms = statistics.mean(p + k for p, k in zip(prep, kern))
        out[name] = {"ms_per_step": ms, "kernel_ms": statistics.mean(kern),
                     "matches_per_s": cnt / (ms / 1e3), "count": cnt}
    counts = {v["count"] for v in out.values()}
    assert len(counts) == 1, "schedules disagree on the 5-clique count"
    cnt = counts.pop()
    out["count_pinned"] = check_count(fx, "clique5", cnt)
    if "learned" in out:
        out["learned_speedup"] = out["heuristic"]["ms_per_step"] / out["learned"]["ms_per_step"]
    out["clocks"] = clocks.stop()
    return out


def batch_run(xgm, ctx, graphs, warmup, steps, local) -> dict:
    """4096 BA graphs: plain heuristic / autotuned / learned schedules of the batched
    CUDA-graph launch; per-graph counts checked against the committed fixture."""
    import numpy as np

    vo, eo, src, dst = xgm.gen_ba_batch(graphs, 100, 5000, 3, 8, seed=5)
    b = ctx.batch_from_edges(vo, src, dst)
    learned = xgm.trained_schedule(ctx)
    tune = ctx.autotune(b, BATCH_PATTERNS, reps=3)
    runs = {"heuristic": {}, "tuned": {"policy": xgm.SCHED_TUNED, "table": tune["table"]}}
    if learned:
        runs["learned"] = learned
    res, ref, kernels = {}, None, {}
    clocks = ClockSampler(local).start()
    for name, kw in runs.items():
        for _ in range(warmup):
            ctx.count_batched(b, BATCH_PATTERNS, **kw)
        _sync()
        ms = []
        for _ in range(steps):
            out, st = ctx.count_batched(b, BATCH_PATTERNS, with_stats=True, **kw)
            ms.append(st["kernel_ms"])
            kernels[name] = st["launches"]  # kernel nodes of the replayed CUDA graph
        if ref is None:
            ref = out
        assert np.array_equal(out, ref), f"{name} schedule changed a count"
        res[name] = statistics.mean(ms)
    clk = clocks.stop()
    per_graph = np.ascontiguousarray(ref, dtype="<u8")
    digest = hashlib.sha256(per_graph.tobytes()).hexdigest()
    totals = {p: int(per_graph[:, i].sum()) for i, p in enumerate(BATCH_PATTERNS)}
    pinned = False
    if graphs == 4096 and os.path.exists(BATCH_FIXTURE):
        with open(BATCH_FIXTURE) as f:
            fx = json.load(f)
        assert digest == fx["per_graph_sha256"], "per-graph batch counts differ from the fixture"
        assert totals == fx["totals"], "batch totals differ from the fixture"
        pinned = True
    total = float(per_graph.astype(np.float64).sum())
    best = min(res, key=res.get)
    out = {"graphs": graphs, "vertices": int(vo[-1]), "samples": int(len(src)),
           "patterns": BATCH_PATTERNS, "schedules_ms": res, "best": best,
           "matches_per_s": {k: total / (v / 1e3) for k, v in res.items()},
           "tuned_variants": tune["variants"], "totals": totals, "per_graph_sha256": digest,
           "counts_pinned": pinned, "kernel_nodes": kernels, "clocks": clk}
    if "learned" in res:
        out["learned_vs_heuristic"] = res["heuristic"] / res["learned"]
        out["learned_vs_tuned"] = res["tuned"] / res["learned"]
    b.close()
    return out


def engine_arm(args, dist: Dist) -> None:
    import torch

    xgm = load_engine()
    torch.cuda.set_device(dist.local)
    ctx = xgm.Context(dist.local)
    nv, src, dst = gen_graph(xgm, args.scale)
    g = ctx.graph_from_edges(nv, src, dst)
    del src, dst
    info = g.info()
    fx = fixture_counts(args.scale, WORKLOAD["seed"])
    if fx:
        assert (info["V"], info["E"]) == (fx["V"], fx["E"]), "not the fixture's graph"
    learned = xgm.trained_schedule(ctx) if args.policy == "learned" else {}
    kw = learned

    timed_counts(ctx, g, args.pattern, args.warmup, kw)
    dist.barrier()
    _sync()
    clocks = ClockSampler(dist.local).start()
    t0 = time.perf_counter()
    count, prep, kern = timed_counts(ctx, g, args.pattern, args.steps, kw)
    _sync()
    wall = time.perf_counter() - t0
    dist.barrier()
    clk = clocks.stop()
    pinned = check_count(fx, PATTERN_KIND[args.pattern], count)
    step_ms = [p + k for p, k in zip(prep, kern)]
    ms_per_step = dist.reduce(sum(step_ms) / args.steps, "max")
    total_matches = dist.reduce(float(count), "sum")
    value = total_matches / (ms_per_step / 1e3)
    kern_ms = statistics.mean(kern)

    # plain heuristic schedule on the same graph and steps (the baseline of the learned one)
    plain = None
    if learned:
        timed_counts(ctx, g, args.pattern, 1, {})
        c2, p2, k2 = timed_counts(ctx, g, args.pattern, args.steps, {})
        assert c2 == count, "schedules disagree on the count"
        pms = dist.reduce(sum(p + k for p, k in zip(p2, k2)) / args.steps, "max")
        plain = {"matches_per_s": total_matches / (pms / 1e3), "ms_per_step": pms,
                 "kernel_ms": statistics.mean(k2)}

    launches = ctx.count_kernels(g, args.pattern, **kw)
    peaks = measured_peaks()
    plan = ctx.algo_bytes(g, args.pattern)
    prof = profile_summary(args.pattern, args.scale)
    traffic = prof.get("traffic_bytes_per_launch")
    achieved = traffic / (kern_ms / 1e3) / 1e9 if traffic else None
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": achieved / peaks["hbm_gbs"] if achieved else None,
        "traffic": int(traffic) if traffic else None,
        "traffic_source": (f"{prof['path']} (ncu dram__bytes_read.sum + dram__bytes_write.sum "
                           "of this launch, committed capture; divided by this run's "
                           "CUDA-event kernel time)") if traffic else "no committed capture",
        "peak_source": peaks["source"],
        # the reference plan's algorithmic bytes (4 B per list element it reads + 8 B per
        # task): this kernel reads each list once per vertex task instead, so the plan's
        # bytes over the launch time exceed the copy peak
        "plan_bytes_per_launch": plan,
        "plan_gbs": plan / (kern_ms / 1e3) / 1e9,
        "issue_active_pct": prof.get("issue_active_pct"),
        "threads_per_warp_inst": prof.get("threads_per_warp_inst"),
        "l2_hit_pct": prof.get("l2_hit_pct"),
    }
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
        "config": workload_config(args, info["V"], info["E"], info["E_dag"],
                                  info["max_degree"], info["max_out_degree"], dist.world),
        "schedule": "learned" if learned else "heuristic",
        "count": count,
        "count_pinned": pinned,
        "gteps": info["E_dag"] / (ms_per_step / 1e3) / 1e9,
        "kernel_ms": kern_ms,
        "prep_ms": statistics.mean(prep),
        "wall_ms_per_step": wall * 1e3 / args.steps,
        "plain_heuristic": plain,
        "gpu_launches": launches * args.steps,
        "roofline": roofline,
        "clocks": clk,
    }

    if args.pattern == "4-clique" and not args.no_clique5 and dist.rank == 0:
        line["clique5"] = clique5_sub(xgm, ctx, g, learned, fx, dist.local)

    # end to end through the C ABI from pinned host buffers
    rp = cp = None
    if not args.no_e2e:
        rowptr, col = g.download()
        rp = torch.empty(len(rowptr), dtype=torch.int64, pin_memory=True)
        cp = torch.empty(len(col), dtype=torch.int32, pin_memory=True)
        rp.numpy()[:] = rowptr
        cp.numpy()[:] = col
        del rowptr, col
        g.close()
        g = None
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

    if args.pattern == "4-clique" and not args.no_batch and dist.rank == 0:
        line["batch"] = batch_run(xgm, ctx, args.graphs, 2, 5, dist.local)

    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        import oracle

        if g is None:
            rowptr, col = rp.numpy(), cp.numpy()
        else:
            rowptr, col = g.download()
        drow, dcol = oracle.orient(rowptr, col)
        c, times, desc = cpu_sample(oracle, args.pattern, args.scale, drow, dcol,
                                    args.cpu_seconds, total=count)
        line["cpu_baseline"] = {"value": c / times[0], "unit": "matches/s",
                                "cores": oracle.threads(), "kind": "port",
                                "sample": sample_text(desc, args.scale, times[0]),
                                "sample_detail": desc, "host": host_cpu()}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    if g is not None:
        g.close()
    ctx.close()


# ------------------------------------------------------------------- batch arm
BATCH_PATTERNS = ["triangle", "4-clique", "diamond"]


def batch_arm(args, dist: Dist) -> None:
    """Batched multi-graph counting: Barabasi-Albert graphs, n log-uniform in
    [100, 5000], m uniform in {3..8}, seed 5; triangle + 4-clique + diamond per graph in
    one persistent launch replayed as a CUDA graph.  Compared with the same counts made
    by one xgm_count call per (graph, pattern) on a sample of the graphs."""
    import torch

    xgm = load_engine()
    torch.cuda.set_device(dist.local)
    ctx = xgm.Context(dist.local)
    res = batch_run(xgm, ctx, args.graphs, args.warmup, args.steps, dist.local)
    vo, eo, src, dst = xgm.gen_ba_batch(args.graphs, 100, 5000, 3, 8, seed=5)
    sample = list(range(0, args.graphs, max(1, args.graphs // 256)))
    loop_s, loop_graphs = 0.0, 0
    for gi in sample:
        lo, hi = int(vo[gi]), int(vo[gi + 1])
        g = ctx.graph_from_edges(hi - lo, src[eo[gi]:eo[gi + 1]] - lo, dst[eo[gi]:eo[gi + 1]] - lo)
        _sync()
        t0 = time.perf_counter()
        for pat in BATCH_PATTERNS:
            ctx.count(g, pat)
        loop_s += time.perf_counter() - t0
        loop_graphs += 1
        g.close()
    loop_ms_full = loop_s * 1e3 * args.graphs / loop_graphs
    best = res["best"]
    ms = res["schedules_ms"][best]
    total = sum(res["totals"].values())
    line = {"metric": "matches_per_sec", "value": total / (ms / 1e3), "unit": "matches/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 ids / uint64 counts", "data": "synthetic (seeded Barabasi-Albert)",
            "config": {"workload": f"batched counting, {args.graphs} BA graphs, "
                                   "triangle + 4-clique + diamond per graph",
                       "graphs": args.graphs, "vertices": res["vertices"],
                       "samples": res["samples"]},
            "schedule": best, "batch": res,
            "per_graph_calls_ms_estimate": loop_ms_full,
            "speedup_vs_per_graph_calls": loop_ms_full / ms,
            "count_total": total,
            "gpu_launches": res["kernel_nodes"][best] * args.steps, "clocks": res["clocks"]}
    print(json.dumps(line), flush=True)
    ctx.close()


# ---------------------------------------------------------------- reference arm
def reference_arm(args, dist: Dist) -> None:
    """The reference's CPU counting algorithm (oracle restatement of the G2Miner OpenMP
    path, all host threads) on the seeded uniform vertex sample of the same graph.  The
    graph is generated and built by the oracle alone (the engine is not loaded)."""
    if dist.rank != 0:
        return
    import numpy as np

    import oracle

    nv, src, dst = gen_graph(oracle, args.scale)
    rowptr, col = oracle.build_csr(nv, src, dst)
    del src, dst
    drow, dcol = oracle.orient(rowptr, col)
    max_deg = int(np.diff(rowptr).max())
    E = len(col)
    del rowptr, col
    max_out = int(np.diff(drow).max())
    fx = fixture_counts(args.scale, WORKLOAD["seed"])
    total = fx.get("counts", {}).get(PATTERN_KIND[args.pattern])
    c, times, desc = cpu_sample(oracle, args.pattern, args.scale, drow, dcol, args.cpu_seconds,
                                total=total, repeat=args.warmup + args.steps)
    times = times[args.warmup:]
    ms = statistics.mean(times) * 1e3
    value = c / (ms / 1e3)
    cores = oracle.threads()
    line = {"metric": "matches_per_sec", "value": value, "unit": "matches/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 ids / uint64 counts", "data": "synthetic (seeded R-MAT, oracle generator)",
            "config": workload_config(args, nv, E, len(dcol), max_deg, max_out, dist.world),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "matches/s", "cores": cores, "kind": "port",
                             "sample": sample_text(desc, args.scale, ms / 1e3),
                             "sample_detail": desc, "host": host_cpu()},
            "e2e": {"value": value, "unit": "matches/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


MOTIF_PATTERNS = ["diamond", "rectangle", "tailedtriangle", "4-clique"]
MOTIF_KIND = {"diamond": "diamond", "rectangle": "cycle4", "tailedtriangle": "tailed",
              "4-clique": "clique4"}


def motifs_arm(args, dist: Dist) -> None:
    """Edge-induced diamond / 4-cycle / tailed triangle / 4-clique on an Erdos-Renyi
    G(n = 2^21, average degree 32), seed 3, and a Chung-Lu power-law graph (n = 2^21,
    exponent 2.1, maximum expected degree 50,000, average degree 32), seed 4.  One step
    counts all four patterns on both graphs; matches/s = total count / total device
    time.  Counts are checked against the reference binaries' fixture."""
    import torch

    xgm = load_engine()
    torch.cuda.set_device(dist.local)
    ctx = xgm.Context(dist.local)
    n = 1 << 21
    graphs = {"er_n2097152_deg32_seed3": xgm.gen_er(n, n * 16, seed=3),
              "chung_lu_n2097152_g2.1_w50000_deg32_seed4":
                  xgm.gen_chung_lu(n, 2.1, 50000.0, 32.0, seed=4)}
    fixtures = json.load(open(CONFIG_FIXTURE)) if os.path.exists(CONFIG_FIXTURE) else {}
    kw = xgm.trained_schedule(ctx) if args.policy == "learned" else {}
    per, total_ms, total_matches, info, launches, pinned = {}, 0.0, 0, {}, 0, 0
    clocks = ClockSampler(dist.local).start()
    for gname, (nv, src, dst) in graphs.items():
        g = ctx.graph_from_edges(nv, src, dst)
        info[gname] = g.info()
        fx = fixtures.get(gname, {})
        for pat in MOTIF_PATTERNS:
            for _ in range(args.warmup):
                ctx.count(g, pat, **kw)
            _sync()
            ms, cnt = [], 0
            for _ in range(args.steps):
                cnt, st = ctx.count(g, pat, with_stats=True, **kw)
                ms.append(st["kernel_ms"] + st["prep_ms"])
                launches += st["launches"]
            pinned += check_count(fx, MOTIF_KIND[pat], cnt)
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
                                   "Chung-Lu 2^21 gamma 2.1 dmax 50k", "graphs": info},
            "schedule": "learned" if kw else "heuristic",
            "counts_pinned": f"{pinned} of {len(per)}",
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
    clocks = ClockSampler(dist.local).start()
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
                                "kind": "port", "host": host_cpu(),
                                "sample": f"P6-P22 on the ER graph ({c} matches in {dt:.2f} s, "
                                          f"OpenMP oracle port; the GPU took {gpu_ms:.1f} ms)"}
    print(json.dumps(line), flush=True)
    ctx.close()


def ablation_arm(args, dist: Dist) -> None:
    """What the learned schedule gains, and from what: on the same kernels, (1) the plain
    degree-threshold heuristic (WARP <= 32 < WIDE <= 128 < CTA <= 1024 < split), (2) that
    heuristic extended with the per-task variants by thresholds alone (GROUP <= 8 <
    BUCKET <= 32), (3) the autotuned per-out-degree-bucket variant table (no model), (4)
    the trained MLP's per-task choice.  4-clique on R-MAT scale 22 seed 2 (a training
    scale, other seed) and on the held-out R-MAT scale 23 seed 99; the 4096-graph BA batch
    (triangle + 4-clique + diamond).  Counts must agree across the arms."""
    import numpy as np
    import torch

    xgm = load_engine()
    torch.cuda.set_device(dist.local)
    ctx = xgm.Context(dist.local)
    learned = xgm.trained_schedule(ctx)
    ext = {"group_max": 8, "bucket_max": 32}

    def best_ms(fn, reps):
        fn()
        out, ms = None, []
        for _ in range(reps):
            out, t = fn()
            ms.append(t)
        return out, min(ms)

    res = {}
    clocks = ClockSampler(dist.local).start()
    for scale, seed in ((22, 2), (23, 99)):
        nv, src, dst = xgm.gen_rmat(scale, 16, seed=seed)
        g = ctx.graph_from_edges(nv, src, dst)
        del src, dst
        tune = ctx.autotune(g, "4-clique", reps=2)
        arms = {"heuristic": {}, "extended_heuristic": ext,
                "autotuned": {"policy": xgm.SCHED_TUNED, "table": tune["table"]}}
        if learned:
            arms["learned"] = learned
        row, want = {}, None
        for name, kw in arms.items():
            def run(kw=kw):
                c, st = ctx.count(g, "4-clique", with_stats=True, **kw)
                return c, st["kernel_ms"] + st["prep_ms"]
            c, ms = best_ms(run, max(2, args.steps))
            want = c if want is None else want
            assert c == want, f"{name} changed the count"
            row[name] = ms
        row["count"] = want
        res[f"4-clique rmat s{scale} seed {seed}"] = row
        g.close()
    vo, eo, src, dst = xgm.gen_ba_batch(4096, 100, 5000, 3, 8, seed=5)
    b = ctx.batch_from_edges(vo, src, dst)
    tune = ctx.autotune(b, BATCH_PATTERNS, reps=3)
    arms = {"heuristic": {}, "extended_heuristic": ext,
            "autotuned": {"policy": xgm.SCHED_TUNED, "table": tune["table"]}}
    if learned:
        arms["learned"] = learned
    row, want = {}, None
    for name, kw in arms.items():
        def run(kw=kw):
            out, st = ctx.count_batched(b, BATCH_PATTERNS, with_stats=True, **kw)
            return out, st["kernel_ms"]
        out, ms = best_ms(run, max(3, args.steps))
        want = out if want is None else want
        assert np.array_equal(out, want), f"{name} changed a count"
        row[name] = ms
    res["batch 4096 BA graphs, triangle + 4-clique + diamond"] = row
    b.close()
    clk = clocks.stop()
    line = {"workload": "schedule ablation (ms per count, best of the steps)", "results": res,
            "schedule_definitions": {"heuristic": "WARP <= 32 < WIDE <= 128 < CTA <= 1024 < split",
                                     "extended_heuristic": "GROUP <= 8 < BUCKET <= 32 < WIDE <= 128 < CTA <= 1024 < split",
                                     "autotuned": "per out-degree bucket variant table (xgm_autotune)",
                                     "learned": "MLP per task (costmodel.json)"},
            "clocks": clk}
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
        elif args.workload == "ablation":
            ablation_arm(args, dist)
        else:
            engine_arm(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()

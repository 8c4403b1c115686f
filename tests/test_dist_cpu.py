"""The multi-rank path of bench.py on CPU: two gloo ranks (no GPU, no data-path collective).

bench.py --gpus N runs N independent replicas (the counting path shards by graph, with
no exchange step); the only collectives are the barrier and the max/sum reductions of
the timing, which these tests run over gloo."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
import textwrap

from conftest import ROOT


def _port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_port())] + args
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_two_rank_reductions(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(textwrap.dedent(f"""
        import sys
        sys.path.insert(0, {ROOT!r})
        import bench
        d = bench.Dist()
        assert d.world == 2
        d.barrier()
        mx = d.reduce(float(d.rank + 1), "max")
        sm = d.reduce(float(d.rank + 1), "sum")
        assert (mx, sm) == (2.0, 3.0), (mx, sm)
        print("rank", d.rank, "ok")
        d.close()
    """))
    r = _torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.count("ok") == 2


def test_reference_arm_two_ranks_prints_once():
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--scale", "12",
                   "--steps", "1", "--warmup", "0", "--cpu-seconds", "1"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1  # rank 0 only
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference")


def test_reference_arm_loads_only_the_oracle(tmp_path):
    """The reference arm builds its graph with the oracle's generator and CSR build and
    times the oracle on a seeded uniform vertex sample: the engine's library is never
    mapped into the process."""
    script = tmp_path / "ref_only.py"
    script.write_text(textwrap.dedent(f"""
        import json, sys
        sys.path.insert(0, {ROOT!r})
        sys.argv = ["bench.py", "--impl", "reference", "--scale", "12", "--steps", "1",
                    "--warmup", "0", "--cpu-seconds", "0.5"]
        import bench
        bench.main()
        maps = open("/proc/self/maps").read()
        assert "libxgm" not in maps, "the reference arm loaded the engine"
        assert "liborc" in maps
        print("maps ok")
    """))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, str(script)], cwd=ROOT, capture_output=True, text=True,
                       timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "maps ok" in r.stdout
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    d = line["cpu_baseline"]["sample_detail"]
    assert 0 < d["fraction"] <= 1 and d["vertices"] > 0 and d["matches"] > 0
    assert line["config"]["V"] == 1 << 12 and "schedule" not in line["config"]

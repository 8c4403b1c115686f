"""xgm_count_cli, the command-line front end over the C ABI with xgminer's flags."""
from __future__ import annotations

import os
import re
import subprocess
import tempfile

import numpy as np
import pytest


@pytest.fixture(scope="module")
def cli(xgm):
    path = os.path.join(os.path.dirname(xgm.LIB_PATH), "xgm_count_cli")
    if not os.path.exists(path):
        import importlib

        importlib.import_module("x-gminer_gb300.build").build()
    return path


def _run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True)


def test_cli_arguments(cli):
    # argument errors are reported before any device is touched
    assert _run(cli, "--help").returncode == 0
    r = _run(cli, "--graph", "x", "--algorithm", "cpu_baseline")
    assert r.returncode == 2 and "GPU" in r.stderr
    assert _run(cli, "--graph", "x", "--algorithm", "no_such_algo").returncode == 2
    r = _run(cli, "--graph", "x", "--patternID", "99")
    assert r.returncode == 2 and "patternID 99" in r.stderr
    assert _run(cli, "--graph", "x", "--bogus").returncode == 2


@pytest.mark.gpu
def test_cli_counts_match_the_library(xgm, ctx, orc, cli):
    nv, s, d = xgm.gen_rmat(10, 8, seed=5)
    rowptr, col = orc.build_csr(nv, s, d)
    g = ctx.graph_from_csr(rowptr, col)
    with tempfile.TemporaryDirectory() as tmp:
        prefix = os.path.join(tmp, "graph")
        orc.write_graph(prefix, rowptr, col)
        cases = [(["--patternID", "20"], ctx.count(g, "4-clique")),          # GLUMIN P4
                 (["--patternID", "22", "--algorithm", "glumin_g2miner_lut"],
                  ctx.count(g, "P6")),
                 (["--patternID", "1"], ctx.count(g, "triangle")),
                 (["--pattern-name", "diamond", "--vert-induced", "1"],
                  ctx.count(g, xgm.plan("diamond", induced=True))),
                 (["--pattern-size", "3", "--pattern-adj-mat", "011101110"],
                  ctx.count(g, "triangle")),
                 (["--pattern-name", "5-house"], ctx.count(g, "5-house"))]
        for args, want in cases:
            r = _run(cli, "--graph", prefix, *args)
            assert r.returncode == 0, (args, r.stderr)
            m = re.search(r"count: (\d+)", r.stdout)
            assert m and int(m.group(1)) == want, (args, r.stdout)
    g.close()

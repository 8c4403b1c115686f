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
    for bad in ("99", "16"):  # 16: GraphPi's Clique_7_Minus, seven vertices
        r = _run(cli, "--graph", "x", "--patternID", bad)
        assert r.returncode == 2 and f"patternID {bad}" in r.stderr
    assert _run(cli, "--graph", "x", "--bogus").returncode == 2


@pytest.mark.gpu
def test_cli_counts_match_the_library(xgm, ctx, orc, cli):
    nv, s, d = xgm.gen_rmat(10, 8, seed=5)
    rowptr, col = orc.build_csr(nv, s, d)
    g = ctx.graph_from_csr(rowptr, col)

    def adj(edges):
        a = np.zeros((6, 6), np.uint8)
        for u, v in edges:
            a[u, v] = a[v, u] = 1
        return a

    # GraphPi's 6-vertex shapes (xgminer/src/pattern_graphpi.cpp)
    hourglass = adj([(0, 1), (0, 2), (0, 4), (1, 2), (1, 5), (2, 3), (3, 4), (3, 5), (4, 5)])
    cycle6tri = adj([(0, 1), (0, 2), (1, 2), (1, 3), (1, 4), (2, 3), (2, 5), (0, 4), (0, 5)])
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
                 (["--pattern-name", "5-house"], ctx.count(g, "5-house")),
                 (["--patternID", "10"], ctx.count(g, "diamond")),
                 (["--patternID", "14"], ctx.count(g, ctx.plan(hourglass))),
                 (["--patternID", "15", "--vert-induced", "1"],
                  ctx.count(g, ctx.plan(cycle6tri, induced=True)))]
        for args, want in cases:
            r = _run(cli, "--graph", prefix, *args)
            assert r.returncode == 0, (args, r.stderr)
            m = re.search(r"count: (\d+)", r.stdout)
            assert m and int(m.group(1)) == want, (args, r.stdout)
    g.close()

"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on a CPU host."""
from __future__ import annotations

import hashlib
import importlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden_counts.json")
# the reference tree (X-GMiner checkout), where present; same variable as
# oracle/build_ref.sh
REFERENCE_ROOT = os.environ.get("XGM_REFERENCE_ROOT", "/root/reference")
REFERENCE_GRAPHS = os.path.join(REFERENCE_ROOT, "codes", "GraphMiner", "inputs")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def xgm():
    mod = importlib.import_module("x-gminer_gb300")
    if not os.path.exists(mod.LIB_PATH):
        importlib.import_module("x-gminer_gb300.build").build()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ctx(xgm):
    c = xgm.Context(0)
    yield c
    c.close()


def csr_digest(rowptr, col) -> str:
    h = hashlib.sha256()
    h.update(np.asarray(rowptr, dtype="<i8").tobytes())
    h.update(np.asarray(col, dtype="<i4").tobytes())
    return h.hexdigest()


def golden_samples(xgm, case):
    g, a, seed = case["gen"], case["args"], case["seed"]
    if g == "rmat":
        return xgm.gen_rmat(a[0], a[1], seed=seed)
    if g == "er":
        return xgm.gen_er(a[0], a[1], seed=seed)
    if g == "ba":
        return xgm.gen_ba(a[0], a[1], seed=seed)
    raise ValueError(g)


DAG_KINDS = ("tc", "clique4", "clique5")
KIND_TO_PATTERN = {"tc": "triangle", "clique4": "4-clique", "clique5": "5-clique",
                   "diamond": "diamond", "cycle4": "rectangle", "tailed": "tailedtriangle"}


def oracle_counts(orc, rowptr, col):
    drow, dcol = orc.orient(rowptr, col)
    out = {}
    for k in KIND_TO_PATTERN:
        out[k] = orc.count(k, drow, dcol) if k in DAG_KINDS else orc.count(k, rowptr, col)
    return out


def relabel_by_degree(rowptr, col):
    """The graph renumbered by (degree, id) rank, rows sorted: the id space the engine's
    kernels walk (its orientation rule is rank(v) > rank(u))."""
    nv = len(rowptr) - 1
    deg = np.diff(rowptr)
    perm = np.lexsort((np.arange(nv), deg))  # rank -> original
    rank = np.empty(nv, dtype=np.int64)
    rank[perm] = np.arange(nv)
    src = np.repeat(np.arange(nv), deg)
    ns, nd = rank[src], rank[col]
    order = np.lexsort((nd, ns))
    r2 = np.zeros(nv + 1, dtype=np.int64)
    np.add.at(r2, ns + 1, 1)
    return np.cumsum(r2), nd[order].astype(np.int32)

"""The C-ABI library: loads without a GPU, exports what include/xgm.h declares."""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REFERENCE_ROOT, ROOT


def header_functions():
    txt = open(os.path.join(ROOT, "include", "xgm.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(xgm_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol(xgm):
    names = header_functions()
    assert len(names) >= 30
    so = ctypes.CDLL(xgm.LIB_PATH)
    for n in names:
        assert hasattr(so, n), n
    assert sorted(xgm.EXPORTED) == names


def test_python_constants_match_header(xgm):
    """The Python mirror's constants (schedule policies and flags, variants, statuses,
    build flags, ...) equal the enum values include/xgm.h declares."""
    txt = open(os.path.join(ROOT, "include", "xgm.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    pairs = re.findall(r"\bXGM_(\w+)\s*=\s*(-?\d+|0x[0-9a-fA-F]+)", txt)
    checked = 0
    for name, val in pairs:
        if hasattr(xgm, name):
            assert getattr(xgm, name) == int(val, 0), name
            checked += 1
    assert checked >= 10
    assert xgm.SCHED_HASH_ONLY == 2 and xgm.SCHED_NO_GRAPH == 1


def test_generators_deterministic(xgm):
    a = xgm.gen_rmat(12, 8, seed=11)
    b = xgm.gen_rmat(12, 8, seed=11)
    c = xgm.gen_rmat(12, 8, seed=12)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert not np.array_equal(a[1], c[1])
    assert a[1].min() >= 0 and a[1].max() < 4096
    n, s, d = xgm.gen_er(1000, 5000, seed=3)
    assert s.max() < 1000 and d.max() < 1000
    n, s, d = xgm.gen_ba(500, 4, seed=3)
    assert len(s) == 4 * (500 - 4)
    assert np.all(s > d)  # each new vertex attaches to earlier ones
    vo, eo, s, d = xgm.gen_ba_batch(16, 100, 300, 3, 8, seed=5)
    for g in range(16):
        lo, hi = vo[g], vo[g + 1]
        es, ed = s[eo[g]:eo[g + 1]], d[eo[g]:eo[g + 1]]
        assert es.min() >= lo and es.max() < hi and ed.min() >= lo and ed.max() < hi


def test_chung_lu_degrees(xgm):
    n, s, d = xgm.gen_chung_lu(1 << 14, 2.1, 2000.0, 16.0, seed=4)
    deg = np.bincount(np.concatenate([s, d]), minlength=n)
    assert abs(deg.mean() - 16.0) < 0.5
    assert deg.max() > 1000  # power-law head near w_max


def test_bad_generator_arguments(xgm):
    lib = xgm.lib()
    assert lib.xgm_gen_rmat(0, 16, 0.57, 0.19, 0.19, 1, None, None) == -1
    assert lib.xgm_gen_rmat(10, 16, 0.7, 0.3, 0.3, 1, None, None) == -1
    assert lib.xgm_gen_ba(3, 5, 1, None, None) == -1


def test_status_strings(xgm):
    for s in range(10):
        assert xgm.lib().xgm_status_string(s)


def test_no_device_is_an_error_not_a_fallback(xgm):
    import subprocess
    if subprocess.run(["sh", "-c", "command -v nvidia-smi && nvidia-smi -L"],
                      capture_output=True).returncode == 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(xgm.XgmError) as e:
        xgm.Context(0)
    assert e.value.status == xgm.ERR_NO_DEVICE


def test_mlp_reference_gradient_is_consistent():
    import oracle.mlp_ref as M
    rng = np.random.default_rng(0)
    p = (rng.standard_normal(M.NPARAM) * 0.3).astype(np.float16).astype(np.float64)
    X = rng.random((64, M.F))
    y = rng.random(64) * 4
    loss, g = M.loss_grad(p, X, y)
    eps = 1e-6
    for i in rng.choice(M.NPARAM, 25, replace=False):
        q = p.copy()
        q[i] += eps
        w1, b1, w2, b2 = [a.astype(np.float64) for a in M.unpack(q)]
        # finite difference in float64 without fp16 rounding of the perturbed weight
        z = X @ (q[: M.H * M.F].reshape(M.H, M.F)).T + q[M.H * M.F: M.H * M.F + M.H]
        yh = np.maximum(z, 0) @ q[M.H * M.F + M.H: M.H * M.F + 2 * M.H] + q[-1]
        lp = np.mean((yh - y) ** 2)
        assert abs((lp - loss) / eps - g[i]) < 1e-3 * max(1.0, abs(g[i]))


def _spec(edges):
    # the layout of a GLUMIN pattern description (codegen/codegen/patterns/*.yml)
    return "pattern:\n  name: x\n  edges: [" + ", ".join(edges) + "]\n  orientation: []\n"


def test_plan_names_and_ids(xgm):
    # count-app names (edge-induced) and GLUMIN ids (vertex-induced); no GPU needed
    for name, pat, ind in [("triangle", xgm.TRIANGLE, 0), ("4-diamond", xgm.DIAMOND, 0),
                           ("rectangle", xgm.CYCLE4, 0), ("4-star", xgm.STAR3, 0),
                           ("4-path", xgm.PATH4, 0), ("3-path", xgm.WEDGE, 0),
                           ("P1", xgm.STAR3, 1), ("P2", xgm.DIAMOND, 1),
                           ("P3", xgm.TAILED_TRIANGLE, 1), ("P4", xgm.CLIQUE4, 1),
                           ("P5", xgm.CLIQUE5, 1), ("6-clique", xgm.CLIQUE6, 0),
                           ("P23", xgm.CLIQUE6, 1), ("P24", xgm.CLIQUE7, 1)]:
        p = xgm.plan(name)
        assert (p.pattern, int(p.induced)) == (pat, ind), name
    for pid in range(6, 23):  # GLUMIN's generated 5-vertex plans: set-operation programs
        p = xgm.plan(f"P{pid}")
        assert (p.pattern, p.induced) == (xgm.PROGRAM, True), pid
        w = p.program
        assert w is not None and len(w) == xgm.PROGRAM_WORDS and w[0] == 2 and w[1] == 5
    for name in xgm.YML5_EDGES:  # GLUMIN's 5-vertex .yml names: compiled, edge-induced
        p = xgm.plan(name)
        assert (p.pattern, p.induced) == (xgm.PROGRAM, False), name
        assert xgm.plan(name, induced=True).induced
    assert xgm.plan("P5").program is None
    for bad in ("P25", "P0", "P6x", "6-star"):
        with pytest.raises(xgm.XgmError) as e:
            xgm.plan(bad)
        assert e.value.status == xgm.ERR_UNSUPPORTED, bad


def test_plan_from_spec(xgm):
    cases = [(["AB", "BC", "AC"], xgm.TRIANGLE), (["AB", "AC", "AD"], xgm.STAR3),
             (["AB", "BC", "CD"], xgm.PATH4), (["AB", "BC"], xgm.WEDGE),
             (["AB", "BC", "CD", "AD"], xgm.CYCLE4), (["AB", "AC", "AD", "BC", "CD"], xgm.DIAMOND),
             (["AB", "AC", "BC", "CD"], xgm.TAILED_TRIANGLE),
             (["AB", "AC", "AD", "BC", "BD", "CD"], xgm.CLIQUE4)]
    for edges, pat in cases:
        p = xgm.plan_from_spec(_spec(edges))
        assert p.pattern == pat and p.induced, edges
        assert not xgm.plan_from_spec(_spec(edges), induced=False).induced
    # a 5-vertex pattern without a builtin compiles to a set-operation program
    p = xgm.plan_from_spec(_spec(["AB", "BC", "CD", "DE", "AE"]))  # 5-cycle
    assert p.pattern == xgm.PROGRAM and p.induced and p.program is not None
    for bad, st in [(_spec(["AB", "A"]), xgm.ERR_INVALID), (_spec(["AA", "AB"]), xgm.ERR_INVALID),
                    ("pattern:\n  name: x\n", xgm.ERR_INVALID), (_spec([]), xgm.ERR_INVALID),
                    (_spec(["AB", "CD"]), xgm.ERR_UNSUPPORTED),  # disconnected
                    (_spec(["AB", "BC", "CD", "DE", "EF", "FG"]), xgm.ERR_UNSUPPORTED)]:  # 7-path
        with pytest.raises(xgm.XgmError) as e:
            xgm.plan_from_spec(bad)
        assert e.value.status == st, bad


GLUMIN_PATTERNS = os.path.join(REFERENCE_ROOT, "codes", "GLUMIN", "codegen", "codegen",
                               "patterns")


@pytest.mark.skipif(not os.path.isdir(GLUMIN_PATTERNS), reason="reference tree absent")
def test_reference_pattern_files(xgm):
    want = {"3-triangle": xgm.TRIANGLE, "3-path": xgm.WEDGE, "4-clique": xgm.CLIQUE4,
            "4-cycle": xgm.CYCLE4, "4-diamond": xgm.DIAMOND, "4-path": xgm.PATH4,
            "4-star": xgm.STAR3, "4-tailed-triangle": xgm.TAILED_TRIANGLE,
            "5-clique": xgm.CLIQUE5}
    want.update({name: xgm.PROGRAM for name in xgm.YML5_EDGES})
    for f in sorted(os.listdir(GLUMIN_PATTERNS)):
        name = f[:-4]
        if name in want:
            assert xgm.plan_from_spec(os.path.join(GLUMIN_PATTERNS, f)).pattern == want[name], f
        else:  # the empty template is not a plan
            with pytest.raises(xgm.XgmError):
                xgm.plan_from_spec(os.path.join(GLUMIN_PATTERNS, f))
    # the engine's copies of the 5-vertex edge lists are the files' own
    for name, edges in xgm.YML5_EDGES.items():
        text = open(os.path.join(GLUMIN_PATTERNS, name + ".yml")).read()
        assert "edges: [" + edges + "]" in text, name


def test_oracle_generators_match_engine(xgm, orc):
    """The oracle's generators (used by the CPU legs, which never load the engine)
    give the engine's samples bit for bit, Chung-Lu and the BA batch sizes included."""
    cases = [("gen_rmat", (12, 16, 0.57, 0.19, 0.19, 3)), ("gen_er", (5000, 40000, 4)),
             ("gen_chung_lu", (1 << 15, 2.1, 3000.0, 16.0, 4)), ("gen_ba", (3000, 5, 4))]
    for name, args in cases:
        a, b = getattr(orc, name)(*args), getattr(xgm, name)(*args)
        assert a[0] == b[0], name
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), name
    a = orc.gen_ba_batch(96, 100, 5000, 3, 8, seed=5)
    b = xgm.gen_ba_batch(96, 100, 5000, 3, 8, seed=5)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_chung_lu_weights_are_host_independent(orc):
    """Chung-Lu samples depend only on integer and correctly rounded IEEE steps: a
    fixed digest of a small graph's samples (the same on x86-64 and aarch64)."""
    import hashlib

    nv, s, d = orc.gen_chung_lu(1 << 12, 2.1, 500.0, 8.0, seed=4)
    h = hashlib.sha256(s.astype("<i4").tobytes() + d.astype("<i4").tobytes()).hexdigest()
    assert h == CHUNG_LU_4096_DIGEST


CHUNG_LU_4096_DIGEST = "ba625a565a6675d02c816b09587f574bfb0f4df61009565bee756230663a7413"

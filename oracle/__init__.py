"""CPU oracle for the GB300 counting engine.

TEST INFRASTRUCTURE ONLY.  Loaded by the tests, by __graft_entry__.smoke() and by the
CPU-baseline leg of bench.py as the checker; the engine never imports or calls it.

 - oracle.c: plain-C restatement of the reference's OpenMP counting path (each
   function cites the reference lines it follows), built here into liborc.so.
 - gen.c: the seeded graph generators (same samples as the engine's), so the CPU
   legs build their graphs without loading the engine.
 - _ref/: the reference's own OpenMP binaries built from its sources by build_ref.sh
   (only where the reference tree is present); run_ref() runs them on graph files.
 - mlp_ref.py: numpy forward/backward of the cost model, the gradient checker.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import shutil
import subprocess
from typing import Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.c")
GEN_SRC = os.path.join(HERE, "gen.c")
LIB = os.path.join(HERE, "liborc.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build() -> str:
    """Compiles oracle.c and gen.c (OpenMP when the compiler has it)."""
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                                             os.path.getmtime(GEN_SRC)):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB + ".tmp"
    base = [cc, "-O3", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", SRC, GEN_SRC,
            "-o", tmp, "-lm"]
    r = subprocess.run(base[:2] + ["-fopenmp"] + base[2:], capture_output=True, text=True)
    if r.returncode != 0:
        r = subprocess.run(base, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


def build_ref() -> bool:
    """Builds the reference's own OpenMP binaries into _ref/ when the tree is present."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], capture_output=True,
                       text=True)
    return r.returncode == 0 and os.path.exists(os.path.join(REF_DIR, "tc_omp_base"))


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P, I64, U64 = C.c_void_p, C.c_int64, C.c_uint64
        L.orc_max_threads.restype = C.c_int
        L.orc_has_openmp.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_free.argtypes = [P]
        L.orc_build_csr.restype = C.c_int
        L.orc_build_csr.argtypes = [I64, P, P, I64, C.c_int, C.POINTER(P), C.POINTER(P),
                                    C.POINTER(I64)]
        L.orc_orient.restype = C.c_int
        L.orc_orient.argtypes = [I64, P, P, C.POINTER(P), C.POINTER(P), C.POINTER(I64)]
        for name in ("orc_tc", "orc_diamond", "orc_cycle4", "orc_tailed_triangle"):
            f = getattr(L, name)
            f.restype = U64
            f.argtypes = [I64, P, P, I64, I64, I64]
        for name in ("orc_clique4", "orc_clique5"):
            f = getattr(L, name)
            f.restype = U64
            f.argtypes = [I64, P, P, I64, I64, I64, I64]
        L.orc_clique_k.restype = U64
        L.orc_clique_k.argtypes = [C.c_int, I64, P, P, I64, I64, I64, I64]
        L.orc_motif.restype = C.c_int
        L.orc_motif.argtypes = [C.c_int, I64, P, P, I64, P]
        L.orc_algo_bytes.restype = U64
        L.orc_algo_bytes.argtypes = [C.c_int, I64, P, P, I64]
        L.orc_glumin5.restype = C.c_int
        L.orc_glumin5.argtypes = [C.c_int, I64, P, P, I64, P]
        L.orc_setprog.restype = C.c_int
        L.orc_setprog.argtypes = [P, C.c_int, I64, P, P, I64, P]
        L.orc_occurrences.restype = C.c_int
        L.orc_occurrences.argtypes = [C.c_int, P, C.c_int, I64, P, P, P]
        L.orc_set_sample.argtypes = [P, I64]
        D = C.c_double
        L.orc_gen_rmat.restype = I64
        L.orc_gen_rmat.argtypes = [C.c_int, C.c_int, D, D, D, U64, P, P]
        L.orc_gen_er.restype = I64
        L.orc_gen_er.argtypes = [I64, I64, U64, P, P]
        L.orc_gen_chung_lu.restype = I64
        L.orc_gen_chung_lu.argtypes = [I64, D, D, D, U64, P, P]
        L.orc_gen_ba.restype = I64
        L.orc_gen_ba.argtypes = [I64, C.c_int, U64, P, P]
        L.orc_gen_ba_batch.restype = I64
        L.orc_gen_ba_batch.argtypes = [C.c_int, I64, I64, C.c_int, C.c_int, U64, P, P, P, P]
        _lib = L
    return _lib


# ------------------------------------------------------------ seeded generators
def _samples(m: int):
    if m < 0:
        raise ValueError("invalid generator parameters")
    return np.empty(m, dtype=np.int32), np.empty(m, dtype=np.int32)


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, seed: int = 1):
    """R-MAT edge samples (same samples as the engine's xgm_gen_rmat)."""
    s, d = _samples(lib().orc_gen_rmat(scale, edge_factor, a, b, c, seed, None, None))
    lib().orc_gen_rmat(scale, edge_factor, a, b, c, seed, s.ctypes.data, d.ctypes.data)
    return 1 << scale, s, d


def gen_er(n: int, m: int, seed: int = 1):
    s, d = _samples(lib().orc_gen_er(n, m, seed, None, None))
    lib().orc_gen_er(n, m, seed, s.ctypes.data, d.ctypes.data)
    return n, s, d


def gen_chung_lu(n: int, gamma: float = 2.1, w_max: float = 50000.0, avg_deg: float = 32.0,
                 seed: int = 1):
    s, d = _samples(lib().orc_gen_chung_lu(n, gamma, w_max, avg_deg, seed, None, None))
    if lib().orc_gen_chung_lu(n, gamma, w_max, avg_deg, seed, s.ctypes.data, d.ctypes.data) < 0:
        raise MemoryError("oracle Chung-Lu generator failed")
    return n, s, d


def gen_ba(n: int, m: int, seed: int = 1):
    s, d = _samples(lib().orc_gen_ba(n, m, seed, None, None))
    if lib().orc_gen_ba(n, m, seed, s.ctypes.data, d.ctypes.data) < 0:
        raise MemoryError("oracle BA generator failed")
    return n, s, d


def gen_ba_batch(num_graphs: int, n_lo: int = 100, n_hi: int = 5000, m_lo: int = 3,
                 m_hi: int = 8, seed: int = 5):
    vo = np.empty(num_graphs + 1, dtype=np.int64)
    eo = np.empty(num_graphs + 1, dtype=np.int64)
    ne = lib().orc_gen_ba_batch(num_graphs, n_lo, n_hi, m_lo, m_hi, seed, vo.ctypes.data,
                                eo.ctypes.data, None, None)
    s, d = _samples(ne)
    lib().orc_gen_ba_batch(num_graphs, n_lo, n_hi, m_lo, m_hi, seed, vo.ctypes.data,
                           eo.ctypes.data, s.ctypes.data, d.ctypes.data)
    return vo, eo, s, d


def vertex_sample(nv: int, fraction: float, seed: int = 12345) -> np.ndarray:
    """A seeded uniform random sample of vertex ids (each vertex kept with probability
    `fraction`, by a hash of (seed, id)), sorted; int64."""
    ids = np.arange(nv, dtype=np.uint64)
    with np.errstate(over="ignore"):  # 64-bit wrap-around is the hash
        x = ids * np.uint64(0x9E3779B97F4A7C15) + np.uint64(seed) * np.uint64(0xD1B54A32D192ED03)
        x ^= x >> np.uint64(31)
        x *= np.uint64(0xBF58476D1CE4E5B9)
        x ^= x >> np.uint64(29)
    keep = (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) < fraction
    return np.nonzero(keep)[0].astype(np.int64)


def _take(p, n, dtype):
    arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(np.ctypeslib.as_ctypes_type(dtype))),
                                shape=(max(n, 1),))[:n].copy()
    lib().orc_free(p)
    return arr


def threads(n: int = 0) -> int:
    if n > 0:
        lib().orc_set_threads(n)
    return lib().orc_max_threads()


def build_csr(nv: int, src: np.ndarray, dst: np.ndarray, flags: int = 7) -> Tuple[np.ndarray, np.ndarray]:
    src = np.ascontiguousarray(src, dtype=np.int32)
    dst = np.ascontiguousarray(dst, dtype=np.int32)
    rp, cp, ne = C.c_void_p(), C.c_void_p(), C.c_int64()
    st = lib().orc_build_csr(nv, src.ctypes.data, dst.ctypes.data, len(src), flags, C.byref(rp),
                             C.byref(cp), C.byref(ne))
    if st != 0:
        raise ValueError(f"oracle CSR build failed ({st})")
    return _take(rp, nv + 1, np.int64), _take(cp, ne.value, np.int32)


def orient(rowptr: np.ndarray, col: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    nv = len(rowptr) - 1
    rp, cp, ne = C.c_void_p(), C.c_void_p(), C.c_int64()
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    if lib().orc_orient(nv, rowptr.ctypes.data, col.ctypes.data, C.byref(rp), C.byref(cp),
                        C.byref(ne)) != 0:
        raise MemoryError("oracle orientation failed")
    return _take(rp, nv + 1, np.int64), _take(cp, ne.value, np.int32)


def _args(rowptr, col):
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    return len(rowptr) - 1, rowptr, col


def count(kind: str, rowptr: np.ndarray, col: np.ndarray, lo: int = 0, hi: int = -1,
          stride: int = 1, sample: np.ndarray = None) -> int:
    """kind: tc / clique4 .. clique7 (on a DAG) or diamond / cycle4 / tailed (undirected).
    With `sample` (int64 vertex ids; triangle and clique kinds only), the top-level
    loop runs over sample[lo:hi:stride] instead of the vertex range."""
    if sample is not None:
        if kind not in ("tc", "clique4", "clique5", "clique6", "clique7"):
            raise ValueError("vertex samples cover the triangle and clique counts")
        sample = np.ascontiguousarray(sample, dtype=np.int64)
        lib().orc_set_sample(sample.ctypes.data, len(sample))
        try:
            return count(kind, rowptr, col, lo, len(sample) if hi < 0 else hi, stride)
        finally:
            lib().orc_set_sample(None, 0)
    nv, rowptr, col = _args(rowptr, col)
    hi = nv if hi < 0 else hi
    L = lib()
    if kind in ("clique6", "clique7"):
        md = int(np.max(np.diff(rowptr))) if nv else 0
        return int(L.orc_clique_k(int(kind[-1]), nv, rowptr.ctypes.data, col.ctypes.data, md,
                                  lo, hi, stride))
    if kind in ("clique4", "clique5"):
        md = int(np.max(np.diff(rowptr))) if nv else 0
        f = L.orc_clique4 if kind == "clique4" else L.orc_clique5
        return int(f(nv, rowptr.ctypes.data, col.ctypes.data, md, lo, hi, stride))
    f = {"tc": L.orc_tc, "diamond": L.orc_diamond, "cycle4": L.orc_cycle4,
         "tailed": L.orc_tailed_triangle}[kind]
    return int(f(nv, rowptr.ctypes.data, col.ctypes.data, lo, hi, stride))


ALGO_KIND = {"tc": 3, "clique4": 4, "clique5": 5, "diamond": 6, "cycle4": 7, "tailed": 8}


def motif(k: int, rowptr: np.ndarray, col: np.ndarray) -> list:
    """Vertex-induced k-motif census (k = 3: [wedges, triangles]; k = 4: [3-stars,
    4-paths, tailed triangles, 4-cycles, diamonds, 4-cliques]) on the undirected CSR."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    nv = len(rowptr) - 1
    md = int(np.diff(rowptr).max()) if nv else 0
    out = np.zeros(6, dtype=np.uint64)
    if lib().orc_motif(k, nv, rowptr.ctypes.data, col.ctypes.data, md, out.ctypes.data) != 0:
        raise ValueError("motif census covers k = 3 and k = 4")
    return [int(x) for x in out[: 2 if k == 3 else 6]]


def glumin5(pid: int, rowptr: np.ndarray, col: np.ndarray) -> int:
    """GLUMIN's P<pid> count (6 <= pid <= 22) on the undirected CSR: the generated plan
    restated as CPU loops, GLUMIN's set semantics included."""
    nv, rowptr, col = _args(rowptr, col)
    md = int(np.diff(rowptr).max()) if nv else 0
    out = np.zeros(1, dtype=np.uint64)
    if lib().orc_glumin5(pid, nv, rowptr.ctypes.data, col.ctypes.data, md, out.ctypes.data) != 0:
        raise ValueError("GLUMIN 5-vertex plans are P6 .. P22")
    return int(out[0])


def program(words, rowptr: np.ndarray, col: np.ndarray) -> int:
    """Runs an engine set-operation program (xgm_plan_program words) on the CPU."""
    w = np.ascontiguousarray(words, dtype=np.int32)
    nv, rowptr, col = _args(rowptr, col)
    md = int(np.diff(rowptr).max()) if nv else 0
    out = np.zeros(1, dtype=np.uint64)
    if lib().orc_setprog(w.ctypes.data, len(w), nv, rowptr.ctypes.data, col.ctypes.data, md,
                         out.ctypes.data) != 0:
        raise ValueError("malformed program words")
    return int(out[0])


def occurrences(adj, induced: bool, rowptr: np.ndarray, col: np.ndarray) -> int:
    """Occurrences of a connected pattern (k x k 0/1 adjacency, k <= 6) by brute force:
    injective embeddings over the automorphism count.  Small graphs only."""
    a = np.ascontiguousarray(np.asarray(adj, dtype=np.uint8))
    k = a.shape[0]
    nv, rowptr, col = _args(rowptr, col)
    out = np.zeros(1, dtype=np.uint64)
    if lib().orc_occurrences(k, a.ctypes.data, 1 if induced else 0, nv, rowptr.ctypes.data,
                             col.ctypes.data, out.ctypes.data) != 0:
        raise ValueError("pattern must be connected, 2 .. 6 vertices")
    return int(out[0])


def algo_bytes(kind: str, rowptr: np.ndarray, col: np.ndarray, sample: np.ndarray = None) -> int:
    """Algorithmic adjacency bytes of the reference plan (4 B per list element read +
    8 B per task); with `sample`, only the tasks of those top-level vertices."""
    nv, rowptr, col = _args(rowptr, col)
    md = int(np.max(np.diff(rowptr))) if nv else 0
    if sample is not None:
        sample = np.ascontiguousarray(sample, dtype=np.int64)
        lib().orc_set_sample(sample.ctypes.data, len(sample))
    try:
        return int(lib().orc_algo_bytes(ALGO_KIND[kind], nv, rowptr.ctypes.data,
                                        col.ctypes.data, md))
    finally:
        if sample is not None:
            lib().orc_set_sample(None, 0)


# ------------------------------------------------------ reference binaries (_ref)
def ref_available(name: str = "tc_omp_base") -> bool:
    return os.access(os.path.join(REF_DIR, name), os.X_OK)


def run_ref(kind: str, prefix: str, threads_: int = 0) -> Tuple[int, float]:
    """Runs a reference binary on <prefix>.* graph files; returns (count, seconds)."""
    env = dict(os.environ)
    if threads_ > 0:
        env["OMP_NUM_THREADS"] = str(threads_)
    if kind == "tc":
        cmd, pat = [os.path.join(REF_DIR, "tc_omp_base"), prefix], r"total_num_triangles = (\d+)"
    elif kind in ("clique4", "clique5"):
        cmd = [os.path.join(REF_DIR, "clique_omp_base"), prefix, kind[-1]]
        pat = r"num_\d-cliques = (\d+)"
    else:
        name = {"diamond": "diamond", "cycle4": "rectangle", "tailed": "tailedtriangle"}[kind]
        cmd, pat = [os.path.join(REF_DIR, "count_omp_base"), prefix, name], r"total_num = (\d+)"
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd[0]} failed: {r.stderr[-500:]}")
    m = re.search(pat, r.stdout)
    t = re.search(r"runtime[^=]*= ([0-9.eE+-]+)", r.stdout)
    if not m:
        raise RuntimeError("unexpected reference output:\n" + r.stdout[-800:])
    return int(m.group(1)), float(t.group(1)) if t else float("nan")


def run_ref_motif(k: int, prefix: str, threads_: int = 0) -> list:
    """Runs the reference's motif_omp_formula (k = 3 or 4); returns its counts in order."""
    env = dict(os.environ)
    if threads_ > 0:
        env["OMP_NUM_THREADS"] = str(threads_)
    cmd = [os.path.join(REF_DIR, "motif_omp_formula"), prefix, str(k)]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd[0]} failed: {r.stderr[-500:]}")
    found = dict((int(i), int(v)) for i, v in re.findall(r"pattern (\d+): (\d+)", r.stdout))
    n = 2 if k == 3 else 6
    if sorted(found) != list(range(n)):
        raise RuntimeError("unexpected reference output:\n" + r.stdout[-800:])
    return [found[i] for i in range(n)]


# GLUMIN's 5-vertex CPU plans (codes/GLUMIN/src/pattern/cpu_serials.cc:57-81): the
# selector of the list form (BS_vertex_*, cpu_kernels/*-BSE.yml.h) and of the LUT form
# (LUT_*, *-BSV.yml.h) for the P id whose generated GPU plan each restates.
GLUMIN5_CPU = {10: (4, 3), 15: (6, 5), 7: (8, 7), 13: (10, 9), 20: (12, 11)}


def run_ref_glumin5(pid: int, prefix: str, lut: bool = False) -> Tuple[int, float]:
    """Runs GLUMIN's CPU plan for P<pid> (7, 10, 13, 15, 20) on <prefix>.* graph files;
    returns (count, seconds)."""
    sel = GLUMIN5_CPU[pid][1 if lut else 0]
    cmd = [os.path.join(REF_DIR, "glumin_pattern_cpu"), prefix, str(sel)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd[0]} failed: {r.stderr[-500:]}")
    m = re.search(r"pattern 0: (\d+)", r.stdout)
    t = re.search(r"runtime \[omp_base\] = ([0-9.eE+-]+)", r.stdout)
    if not m:
        raise RuntimeError("unexpected reference output:\n" + r.stdout[-800:])
    return int(m.group(1)), float(t.group(1)) if t else float("nan")


def write_graph(prefix: str, rowptr: np.ndarray, col: np.ndarray) -> None:
    """Writes <prefix>.meta.txt/.vertex.bin/.edge.bin (scripts/graph_format_conversion.py:47-80)."""
    nv = len(rowptr) - 1
    maxd = int(np.max(np.diff(rowptr))) if nv else 0
    with open(prefix + ".meta.txt", "w") as f:
        f.write(f"{nv}\n{len(col)}\n4 8 1 2\n{maxd}\n0\n0\n0\n")
    np.ascontiguousarray(rowptr, dtype="<i8").tofile(prefix + ".vertex.bin")
    np.ascontiguousarray(col, dtype="<i4").tofile(prefix + ".edge.bin")


def read_graph(prefix: str) -> Tuple[np.ndarray, np.ndarray]:
    with open(prefix + ".meta.txt") as f:
        nv, ne = int(f.readline()), int(f.readline())
    rowptr = np.fromfile(prefix + ".vertex.bin", dtype="<i8", count=nv + 1)
    col = np.fromfile(prefix + ".edge.bin", dtype="<i4", count=ne)
    return rowptr, col

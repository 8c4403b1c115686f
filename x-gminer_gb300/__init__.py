"""Python host binding of the GB300 pattern-counting engine (ctypes over include/xgm.h).

Mirrors the reference's solver interface for the counting path:

  TCSolver(g)          <- TCSolver(Graph&, uint64_t&, int, int)
                          codes/GraphMiner/src/triangle/main.cc:5
  CliqueSolver(g, k)   <- CliqueSolver(Graph&, int k, uint64_t&, int, int)
                          codes/GraphMiner/src/clique/main.cc:6
  ScSolver(g, name)    <- ScSolver(Graph&, Pattern&, uint64_t&, int, int)
                          codes/GraphMiner/src/count/main.cc:7
  Graph.load(prefix)   <- Graph(prefix, use_dag) / Graph_V2(prefix, use_dag)
                          codes/GraphMiner/src/common/graph.cc:4, xgminer/src/graph_v2.cpp:5

The counting itself runs in libxgm.so (hand-written sm_103a CUDA behind a C ABI).  There
is no CPU fallback: without the built library or a GPU the calls raise XgmError.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from typing import Optional, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libxgm.so")

# status codes (xgm_status)
OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_DEVICE, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_IO, \
    ERR_GRAPH, ERR_NO_DEVICE = range(10)

BUILD_SYMMETRIZE, BUILD_DEDUP, BUILD_DROP_SELF, BUILD_VALIDATE = 1, 2, 4, 8
BUILD_CLEAN = 7
VIEW_UNDIRECTED, VIEW_DAG = 0, 1

TRIANGLE, CLIQUE4, CLIQUE5, DIAMOND, CYCLE4, TAILED_TRIANGLE = 1, 2, 3, 4, 5, 6
WEDGE, STAR3, PATH4, CLIQUE6, CLIQUE7 = 7, 8, 9, 10, 11
PROGRAM = 12  # set-operation program: GLUMIN P6..P22 or a compiled pattern of up to 6 vertices
PROGRAM_WORDS = 162
GLUMIN5_IDS = [f"P{i}" for i in range(6, 23)]
# GLUMIN's 5-vertex .yml patterns (codegen/codegen/patterns/5-*.yml), `edges:` lists
YML5_EDGES = {"5-cycle": "AB, BC, CD, DE, AE", "5-double-triangle": "AB, AC, BC, AD, AE, DE",
              "5-house": "AB, AC, BC, BD, DE, CE", "5-path": "AB, BC, CD, DE",
              "5-solid-house": "AB, AC, BC, BD, BE, CD, CE, DE", "5-star": "AB, AC, AD, AE",
              "5-tailed-square": "AB, BC, CD, AD, AE"}
PATTERN_NAMES = {"triangle": TRIANGLE, "4-clique": CLIQUE4, "5-clique": CLIQUE5,
                 "diamond": DIAMOND, "rectangle": CYCLE4, "4-cycle": CYCLE4,
                 "tailedtriangle": TAILED_TRIANGLE, "wedge": WEDGE, "3-star": STAR3,
                 "4-path": PATH4, "6-clique": CLIQUE6, "7-clique": CLIQUE7}
# order of the motif census (MotifSolver output)
MOTIF3_NAMES = ["wedge", "triangle"]
MOTIF4_NAMES = ["3-star", "4-path", "tailed-triangle", "4-cycle", "diamond", "4-clique"]

SCHED_HEURISTIC, SCHED_LEARNED, SCHED_FIXED, SCHED_TUNED = 0, 1, 2, 3
SCHED_NO_GRAPH = 1
SCHED_HASH_ONLY = 2  # CTA tasks use the Bloom filter + hash, never the span bitmap
TUNE_BUCKETS = 16
VAR_WARP, VAR_CTA, VAR_SPLIT, VAR_WIDE, VAR_SEARCH, VAR_BUCKET, VAR_GROUP = 0, 1, 2, 3, 4, 5, 6
NUM_VARIANTS = 7
ALL_VARIANTS = (VAR_WARP, VAR_CTA, VAR_SPLIT, VAR_WIDE, VAR_SEARCH, VAR_BUCKET, VAR_GROUP)

MODEL_FEATURES, MODEL_HIDDEN = 12, 32
COLLECT_MULTI = 0x100  # xgm_model_collect: time the batched multi-pattern launch
MODEL_PARAMS = MODEL_HIDDEN * MODEL_FEATURES + 2 * MODEL_HIDDEN + 1


class XgmError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"xgm status {status}: {message}")
        self.status = status
        self.message = message


class CsrHost(C.Structure):
    _fields_ = [("num_vertices", C.c_int64), ("num_edges", C.c_int64),
                ("rowptr", C.c_void_p), ("colidx", C.c_void_p)]


class GraphInfo(C.Structure):
    _fields_ = [("num_vertices", C.c_int64), ("num_edges", C.c_int64),
                ("num_dag_edges", C.c_int64), ("max_degree", C.c_int64),
                ("max_out_degree", C.c_int64), ("num_triangles_hint", C.c_int64)]


class PlanDesc(C.Structure):
    _fields_ = [("builtin", C.c_int), ("num_vertices", C.c_int),
                ("adj", (C.c_uint8 * 8) * 8), ("induced", C.c_int)]


class TuneTable(C.Structure):
    _fields_ = [("variant", C.c_uint8 * 16)]


class Sched(C.Structure):
    _fields_ = [("policy", C.c_int), ("variant", C.c_int), ("model", C.c_void_p),
                ("warp_max", C.c_int), ("cta_max", C.c_int), ("order_by_cost", C.c_int),
                ("table", C.c_void_p), ("flags", C.c_int), ("wide_max", C.c_int),
                ("search_max", C.c_int), ("bucket_max", C.c_int), ("group_max", C.c_int),
                ("margin", C.c_float), ("hub_max", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("table", TuneTable), ("best_ms", C.c_double), ("heuristic_ms", C.c_double),
                ("trials", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("prep_ms", C.c_double), ("tasks", C.c_int64),
                ("variant_tasks", C.c_int64 * NUM_VARIANTS), ("algo_bytes", C.c_uint64),
                ("device_error", C.c_uint32), ("launches", C.c_int)]

    def as_dict(self) -> dict:
        return {"kernel_ms": self.kernel_ms, "prep_ms": self.prep_ms, "tasks": self.tasks,
                "variant_tasks": list(self.variant_tasks), "device_error": self.device_error,
                "launches": self.launches}


# (name, restype, argtypes) of every entry point declared in include/xgm.h
_P, _I, _I64, _U64 = C.c_void_p, C.c_int, C.c_int64, C.c_uint64
_SIGS = [
    ("xgm_status_string", C.c_char_p, [_I]),
    ("xgm_create", _I, [C.POINTER(_P), _P]),
    ("xgm_destroy", None, [_P]),
    ("xgm_last_error", C.c_char_p, [_P]),
    ("xgm_stream", _P, [_P]),
    ("xgm_graph_upload", _I, [_P, C.POINTER(CsrHost), _I, C.POINTER(_P)]),
    ("xgm_graph_build_from_edges", _I, [_P, _I64, _P, _P, _I64, _I, C.POINTER(_P)]),
    ("xgm_graph_load", _I, [_P, C.c_char_p, _I, C.POINTER(_P)]),
    ("xgm_graph_info_get", _I, [_P, C.POINTER(GraphInfo)]),
    ("xgm_graph_download", _I, [_P, _P, _I, _P, _P]),
    ("xgm_graph_destroy", None, [_P]),
    ("xgm_graph_write_files", _I, [C.c_char_p, C.POINTER(CsrHost)]),
    ("xgm_plan_compile", _I, [_P, C.POINTER(PlanDesc), C.POINTER(_P)]),
    ("xgm_plan_from_name", _I, [_P, C.c_char_p, C.POINTER(_P)]),
    ("xgm_plan_from_spec", _I, [_P, C.c_char_p, _I, C.POINTER(_P)]),
    ("xgm_plan_pattern", _I, [_P]),
    ("xgm_plan_program", _I, [_P, _P, _I]),
    ("xgm_plan_induced", _I, [_P]),
    ("xgm_plan_destroy", None, [_P]),
    ("xgm_count", _I, [_P, _P, _P, C.POINTER(Sched), C.POINTER(_U64), C.POINTER(Stats)]),
    ("xgm_motif_count", _I, [_P, _P, _I, C.POINTER(Sched), C.POINTER(_U64), _I,
                             C.POINTER(Stats)]),
    ("xgm_count_kernels", _I, [_P, _P, _P, C.POINTER(Sched), C.POINTER(_I)]),
    ("xgm_tc_solver", _I, [_P, _P, C.POINTER(_U64)]),
    ("xgm_tc_solver_static", _I, [_P, _P, C.POINTER(_U64)]),
    ("xgm_clique_solver", _I, [_P, _P, _I, C.POINTER(_U64)]),
    ("xgm_sc_solver", _I, [_P, _P, C.c_char_p, C.POINTER(_U64)]),
    ("xgm_algo_bytes", _I, [_P, _P, _P, C.POINTER(_U64)]),
    ("xgm_autotune", _I, [_P, _P, _P, _P, _I, _I, C.POINTER(TuneResult)]),
    ("xgm_batch_build_from_edges", _I, [_P, _I, _P, _P, _P, _I64, _I, C.POINTER(_P)]),
    ("xgm_batch_upload", _I, [_P, _I, _P, C.POINTER(CsrHost), _I, C.POINTER(_P)]),
    ("xgm_batch_num_graphs", _I, [_P]),
    ("xgm_batch_graph", _P, [_P]),
    ("xgm_count_batched", _I, [_P, _P, _P, _I, C.POINTER(Sched), _P, C.POINTER(Stats)]),
    ("xgm_batch_destroy", None, [_P]),
    ("xgm_model_create", _I, [_P, _U64, C.POINTER(_P)]),
    ("xgm_model_destroy", None, [_P]),
    ("xgm_model_set_params", _I, [_P, _P]),
    ("xgm_model_get_params", _I, [_P, _P]),
    ("xgm_model_collect", _I, [_P, _P, _P, _I, _I, _P, _P, _I64, C.POINTER(_I64),
                               C.POINTER(_U64)]),
    ("xgm_model_train", _I, [_P, _P, _P, _P, _I64, _I, _I, C.c_float, _U64,
                             C.POINTER(C.c_float)]),
    ("xgm_model_predict", _I, [_P, _P, _P, _I64, _P]),
    ("xgm_model_loss_grad", _I, [_P, _P, _P, _P, _I64, C.POINTER(C.c_float), _P]),
    ("xgm_gen_rmat", _I64, [_I, _I, C.c_double, C.c_double, C.c_double, _U64, _P, _P]),
    ("xgm_gen_er", _I64, [_I64, _I64, _U64, _P, _P]),
    ("xgm_gen_chung_lu", _I64, [_I64, C.c_double, C.c_double, C.c_double, _U64, _P, _P]),
    ("xgm_gen_ba", _I64, [_I64, _I, _U64, _P, _P]),
    ("xgm_gen_ba_batch", _I64, [_I, _I64, _I64, _I, _I, _U64, _P, _P, _P, _P]),
]
EXPORTED = [s[0] for s in _SIGS]

_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    """Loads libxgm.so (built in-tree by __graft_entry__.build() / build.py)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise XgmError(ERR_INVALID, f"{LIB_PATH} is not built; run build.py first")
        L = C.CDLL(LIB_PATH)
        for name, res, args in _SIGS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _check(st: int, ctx: Optional["Context"] = None) -> None:
    if st != OK:
        msg = lib().xgm_last_error(ctx._h if ctx is not None else None)
        raise XgmError(st, (msg or b"").decode() or lib().xgm_status_string(st).decode())


class Context:
    """A device context (one CUDA stream); mirrors one GPU of the reference's solvers."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        cfg = (C.c_int * 2)(device, 0)
        st = lib().xgm_create(C.byref(h), C.cast(cfg, C.c_void_p))
        _check(st)
        self._h = h
        # graphs and models of this context; the C ABI requires them to be destroyed
        # before the context, so close() releases them first
        self._children: "weakref.WeakSet" = weakref.WeakSet()

    def _adopt(self, obj):
        self._children.add(obj)
        return obj

    def close(self) -> None:
        if self._h:
            for child in list(self._children):
                child.close()
            lib().xgm_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # graphs -------------------------------------------------------------
    def graph_from_edges(self, num_vertices: int, src: np.ndarray, dst: np.ndarray,
                         flags: int = BUILD_CLEAN) -> "Graph":
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        h = C.c_void_p()
        _check(lib().xgm_graph_build_from_edges(self._h, int(num_vertices), _ptr(src), _ptr(dst),
                                                 len(src), flags, C.byref(h)), self)
        return self._adopt(Graph(self, h))

    def graph_from_csr(self, rowptr: np.ndarray, colidx: np.ndarray, flags: int = 0) -> "Graph":
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        colidx = np.ascontiguousarray(colidx, dtype=np.int32)
        csr = CsrHost(len(rowptr) - 1, len(colidx), _ptr(rowptr), _ptr(colidx) if len(colidx) else 0)
        h = C.c_void_p()
        _check(lib().xgm_graph_upload(self._h, C.byref(csr), flags, C.byref(h)), self)
        return self._adopt(Graph(self, h))

    def load_graph(self, prefix: str, flags: int = 0) -> "Graph":
        h = C.c_void_p()
        _check(lib().xgm_graph_load(self._h, prefix.encode(), flags, C.byref(h)), self)
        return self._adopt(Graph(self, h))

    # plans / counting -----------------------------------------------------
    def plan(self, pattern, induced: bool = False, program: bool = False) -> "Plan":
        return plan(pattern, induced, self, program)

    def plan_from_spec(self, spec: str, induced: bool = True) -> "Plan":
        """Plan from a GLUMIN pattern .yml (text or path); GLUMIN counts vertex-induced."""
        return plan_from_spec(spec, induced, self)

    @staticmethod
    def _sched(policy=SCHED_HEURISTIC, variant=0, model=None, warp_max=0, cta_max=0,
               order_by_cost=1, table=None, flags=0, wide_max=0, search_max=0, bucket_max=0,
               group_max=0, margin=0.0, hub_max=0):
        sp = Sched(policy, variant, model._h if model is not None else None, warp_max, cta_max,
                   order_by_cost, C.cast(C.pointer(table), C.c_void_p) if table is not None
                   else None, flags, wide_max, search_max, bucket_max, group_max, margin,
                   hub_max)
        sp._keep = table  # keep the table alive with the struct
        return sp

    def count(self, graph: "Graph", pattern, policy: int = SCHED_HEURISTIC, variant: int = 0,
              model: Optional["Model"] = None, warp_max: int = 0, cta_max: int = 0,
              order_by_cost: int = 1, table: Optional[TuneTable] = None,
              wide_max: int = 0, search_max: int = 0, bucket_max: int = 0,
              group_max: int = 0, margin: float = 0.0, hub_max: int = 0,
              hash_only: bool = False, with_stats: bool = False):
        plan = pattern if isinstance(pattern, Plan) else self.plan(pattern)
        sp = self._sched(policy, variant, model, warp_max, cta_max, order_by_cost, table,
                         SCHED_HASH_ONLY if hash_only else 0, wide_max=wide_max,
                         search_max=search_max, bucket_max=bucket_max,
                         group_max=group_max, margin=margin, hub_max=hub_max)
        out = C.c_uint64()
        st = Stats()
        _check(lib().xgm_count(self._h, graph._h, plan._h, C.byref(sp), C.byref(out),
                               C.byref(st)), self)
        return (int(out.value), st.as_dict()) if with_stats else int(out.value)

    def motif_count(self, graph: "Graph", k: int, policy: int = SCHED_HEURISTIC,
                    variant: int = 0, model: Optional["Model"] = None,
                    with_stats: bool = False):
        """Vertex-induced k-motif census, k = 3 or 4 (MOTIF3_NAMES / MOTIF4_NAMES order)."""
        sp = self._sched(policy, variant, model)
        out = (C.c_uint64 * 6)()
        st = Stats()
        _check(lib().xgm_motif_count(self._h, graph._h, k, C.byref(sp), out, 6, C.byref(st)),
               self)
        res = [int(x) for x in out[: 2 if k == 3 else 6]]
        return (res, st.as_dict()) if with_stats else res

    def count_kernels(self, graph: "Graph", pattern, policy: int = SCHED_HEURISTIC,
                      model: Optional["Model"] = None, order_by_cost: int = 1,
                      margin: float = 0.0) -> int:
        plan = pattern if isinstance(pattern, Plan) else self.plan(pattern)
        sp = self._sched(policy, 0, model, 0, 0, order_by_cost, margin=margin)
        n = C.c_int()
        _check(lib().xgm_count_kernels(self._h, graph._h, plan._h, C.byref(sp), C.byref(n)), self)
        return int(n.value)

    # batches --------------------------------------------------------------
    def batch_from_edges(self, vtx_off: np.ndarray, src: np.ndarray, dst: np.ndarray,
                         flags: int = BUILD_CLEAN) -> "Batch":
        vtx_off = np.ascontiguousarray(vtx_off, dtype=np.int64)
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        h = C.c_void_p()
        _check(lib().xgm_batch_build_from_edges(self._h, len(vtx_off) - 1, _ptr(vtx_off),
                                                 _ptr(src), _ptr(dst), len(src), flags,
                                                 C.byref(h)), self)
        return self._adopt(Batch(self, h))

    def batch_from_csr(self, vtx_off: np.ndarray, rowptr: np.ndarray, colidx: np.ndarray,
                       flags: int = 0) -> "Batch":
        vtx_off = np.ascontiguousarray(vtx_off, dtype=np.int64)
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        colidx = np.ascontiguousarray(colidx, dtype=np.int32)
        csr = CsrHost(len(rowptr) - 1, len(colidx), _ptr(rowptr), _ptr(colidx) if len(colidx) else 0)
        h = C.c_void_p()
        _check(lib().xgm_batch_upload(self._h, len(vtx_off) - 1, _ptr(vtx_off), C.byref(csr),
                                      flags, C.byref(h)), self)
        return self._adopt(Batch(self, h))

    def count_batched(self, batch: "Batch", patterns, policy: int = SCHED_HEURISTIC,
                      model: Optional["Model"] = None, table: Optional[TuneTable] = None,
                      use_graph: bool = True, order_by_cost: int = 1, margin: float = 0.0,
                      group_max: int = 0, bucket_max: int = 0, search_max: int = 0,
                      hub_max: int = 0, hash_only: bool = False, with_stats: bool = False):
        plans = [p if isinstance(p, Plan) else self.plan(p) for p in patterns]
        arr = (C.c_void_p * len(plans))(*[p._h.value for p in plans])
        sp = self._sched(policy, 0, model, 0, 0, order_by_cost, table,
                         (0 if use_graph else SCHED_NO_GRAPH) |
                         (SCHED_HASH_ONLY if hash_only else 0), search_max=search_max,
                         bucket_max=bucket_max, group_max=group_max, margin=margin,
                         hub_max=hub_max)
        out = np.empty(batch.num_graphs * len(plans), dtype=np.uint64)
        st = Stats()
        _check(lib().xgm_count_batched(self._h, batch._h, C.cast(arr, C.c_void_p), len(plans),
                                       C.byref(sp), _ptr(out), C.byref(st)), self)
        res = out.reshape(batch.num_graphs, len(plans))
        return (res, st.as_dict()) if with_stats else res

    def autotune(self, target, patterns, reps: int = 3) -> dict:
        """Per out-degree bucket variant table for a graph (one pattern) or a batch."""
        if isinstance(patterns, (str, int, Plan)):
            patterns = [patterns]
        plans = [p if isinstance(p, Plan) else self.plan(p) for p in patterns]
        arr = (C.c_void_p * len(plans))(*[p._h.value for p in plans])
        res = TuneResult()
        g = target._h if isinstance(target, Graph) else None
        b = target._h if isinstance(target, Batch) else None
        _check(lib().xgm_autotune(self._h, g, b, C.cast(arr, C.c_void_p), len(plans), reps,
                                  C.byref(res)), self)
        table = TuneTable()
        C.memmove(C.byref(table), C.byref(res.table), C.sizeof(TuneTable))
        return {"table": table, "variants": list(res.table.variant), "best_ms": res.best_ms,
                "heuristic_ms": res.heuristic_ms, "trials": res.trials}

    def algo_bytes(self, graph: "Graph", pattern) -> int:
        plan = pattern if isinstance(pattern, Plan) else self.plan(pattern)
        out = C.c_uint64()
        _check(lib().xgm_algo_bytes(self._h, graph._h, plan._h, C.byref(out)), self)
        return int(out.value)


def plan(pattern, induced: bool = False, ctx: Optional["Context"] = None,
         program: bool = False) -> "Plan":
    """Plan from a name, a builtin id or a pattern adjacency matrix (no GPU needed);
    program=True compiles an adjacency matrix to a set-operation program even where a
    builtin plan exists."""
    h = C.c_void_p()
    ch = ctx._h if ctx is not None else None
    if isinstance(pattern, str):
        if induced and pattern in YML5_EDGES:
            return plan_from_spec(f"edges: [{YML5_EDGES[pattern]}]", True, ctx)
        _check(lib().xgm_plan_from_name(ch, pattern.encode(), C.byref(h)), ctx)
        if induced and lib().xgm_plan_pattern(h) == PROGRAM:
            if not lib().xgm_plan_induced(h):
                lib().xgm_plan_destroy(h)
                raise XgmError(ERR_UNSUPPORTED, f"{pattern}: no vertex-induced form by name")
            return Plan(h)
        if induced:  # names carry no induced flag: rebuild through the descriptor
            p = lib().xgm_plan_pattern(h)
            lib().xgm_plan_destroy(h)
            return plan(p, induced, ctx)
        return Plan(h)
    d = PlanDesc()
    d.induced = 1 if induced else 0
    if isinstance(pattern, int):
        d.builtin = pattern
    else:
        adj = np.asarray(pattern, dtype=np.uint8)
        d.builtin = PROGRAM if program else 0
        d.num_vertices = adj.shape[0]
        for i in range(adj.shape[0]):
            for j in range(adj.shape[1]):
                d.adj[i][j] = int(adj[i, j])
    _check(lib().xgm_plan_compile(ch, C.byref(d), C.byref(h)), ctx)
    return Plan(h)


def plan_from_spec(spec: str, induced: bool = True, ctx: Optional["Context"] = None) -> "Plan":
    if os.path.exists(spec):
        spec = open(spec).read()
    h = C.c_void_p()
    _check(lib().xgm_plan_from_spec(ctx._h if ctx is not None else None, spec.encode(),
                                    1 if induced else 0, C.byref(h)), ctx)
    return Plan(h)


class Plan:
    def __init__(self, h):
        self._h = h

    @property
    def pattern(self) -> int:
        return lib().xgm_plan_pattern(self._h)

    @property
    def induced(self) -> bool:
        return bool(lib().xgm_plan_induced(self._h))

    @property
    def program(self) -> Optional[np.ndarray]:
        """Flat words of a set-operation program plan (None for a builtin)."""
        n = lib().xgm_plan_program(self._h, None, 0)
        if n == 0:
            return None
        w = np.zeros(n, dtype=np.int32)
        lib().xgm_plan_program(self._h, w.ctypes.data, n)
        return w

    def __del__(self):
        try:
            if self._h:
                lib().xgm_plan_destroy(self._h)
                self._h = None
        except Exception:
            pass


class Graph:
    """A device-resident graph (undirected CSR + degree-oriented DAG)."""

    def __init__(self, ctx: Context, h):
        self.ctx = ctx
        self._h = h

    @classmethod
    def load(cls, ctx: Context, prefix: str) -> "Graph":
        return ctx.load_graph(prefix)

    def info(self) -> dict:
        i = GraphInfo()
        _check(lib().xgm_graph_info_get(self._h, C.byref(i)))
        return {"V": i.num_vertices, "E": i.num_edges, "E_dag": i.num_dag_edges,
                "max_degree": i.max_degree, "max_out_degree": i.max_out_degree}

    def download(self, view: int = VIEW_UNDIRECTED) -> Tuple[np.ndarray, np.ndarray]:
        inf = self.info()
        rowptr = np.empty(inf["V"] + 1, dtype=np.int64)
        col = np.empty(max(1, inf["E"] if view == VIEW_UNDIRECTED else inf["E_dag"]), dtype=np.int32)
        _check(lib().xgm_graph_download(self.ctx._h, self._h, view, _ptr(rowptr), _ptr(col)),
               self.ctx)
        return rowptr, col[: int(rowptr[-1])]

    def close(self) -> None:
        if self._h and self.ctx._h:
            lib().xgm_graph_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many small graphs in one packed id space (graph i owns [vtx_off[i], vtx_off[i+1]))."""

    def __init__(self, ctx: Context, h):
        self.ctx = ctx
        self._h = h
        self.num_graphs = lib().xgm_batch_num_graphs(h)

    def download(self):
        """Packed undirected CSR (global ids)."""
        gh = lib().xgm_batch_graph(self._h)
        view = Graph.__new__(Graph)
        view.ctx, view._h = self.ctx, C.c_void_p(gh)
        try:
            return view.download()
        finally:
            view._h = None  # owned by the batch

    def close(self) -> None:
        if self._h and self.ctx._h:
            lib().xgm_batch_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Model:
    """Learned cost model (12 -> 32 -> 1 MLP, fp16 weights) trained on the GPU."""

    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        h = C.c_void_p()
        _check(lib().xgm_model_create(ctx._h, seed, C.byref(h)), ctx)
        self._h = h
        ctx._adopt(self)

    def close(self) -> None:
        if self._h and self.ctx._h:
            lib().xgm_model_destroy(self._h)
        self._h = None

    def params(self) -> np.ndarray:
        p = np.empty(MODEL_PARAMS, dtype=np.float32)
        _check(lib().xgm_model_get_params(self._h, _ptr(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().xgm_model_set_params(self._h, _ptr(p)))

    def collect(self, graph: Graph, pattern, variant: int, stride: int = 1,
                max_rows: int = 1 << 20, multi: bool = False):
        """Per-task features and log2 warp-cycles with every task forced to `variant`;
        multi=True times the batched multi-pattern launch (pattern "triangle")."""
        plan = pattern if isinstance(pattern, Plan) else self.ctx.plan(pattern)
        if multi:
            variant |= COLLECT_MULTI
        X = np.empty((max_rows, MODEL_FEATURES), dtype=np.float32)
        y = np.empty(max_rows, dtype=np.float32)
        n = C.c_int64()
        cnt = C.c_uint64()
        _check(lib().xgm_model_collect(self.ctx._h, graph._h, plan._h, variant, stride, _ptr(X),
                                       _ptr(y), max_rows, C.byref(n), C.byref(cnt)), self.ctx)
        return X[: n.value].copy(), y[: n.value].copy(), int(cnt.value)

    def train(self, X: np.ndarray, y: np.ndarray, epochs: int = 20, batch: int = 1024,
              lr: float = 3e-3, seed: int = 1) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = C.c_float()
        _check(lib().xgm_model_train(self.ctx._h, self._h, _ptr(X), _ptr(y), len(y), epochs, batch,
                                     lr, seed, C.byref(loss)), self.ctx)
        return float(loss.value)

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.empty(len(X), dtype=np.float32)
        _check(lib().xgm_model_predict(self.ctx._h, self._h, _ptr(X), len(X), _ptr(y)), self.ctx)
        return y

    def loss_grad(self, X: np.ndarray, y: np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = C.c_float()
        g = np.empty(MODEL_PARAMS, dtype=np.float32)
        _check(lib().xgm_model_loss_grad(self.ctx._h, self._h, _ptr(X), _ptr(y), len(y),
                                         C.byref(loss), _ptr(g)), self.ctx)
        return float(loss.value), g

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------- reference-shaped solvers
def TCSolver(g: Graph) -> int:
    out = C.c_uint64()
    _check(lib().xgm_tc_solver(g.ctx._h, g._h, C.byref(out)), g.ctx)
    return int(out.value)


def CliqueSolver(g: Graph, k: int) -> int:
    out = C.c_uint64()
    _check(lib().xgm_clique_solver(g.ctx._h, g._h, k, C.byref(out)), g.ctx)
    return int(out.value)


def MotifSolver(g: Graph, k: int) -> list:
    """Vertex-induced k-motif census in the reference's output order (MOTIF3_NAMES /
    MOTIF4_NAMES)."""
    return g.ctx.motif_count(g, k)


def ScSolver(g: Graph, pattern: str) -> int:
    out = C.c_uint64()
    _check(lib().xgm_sc_solver(g.ctx._h, g._h, pattern.encode(), C.byref(out)), g.ctx)
    return int(out.value)


# ------------------------------------------------------------- trained schedule
COSTMODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "costmodel.json")


def trained_schedule(ctx: "Context", path: Optional[str] = None) -> dict:
    """count() keyword arguments for the learned schedule with the trained cost model
    (costmodel.json: parameters, queue order and margin); {} when the file is absent
    or was trained for another feature layout, i.e. the plain heuristic schedule."""
    import json

    path = path or COSTMODEL_PATH
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        spec = json.load(f)
    if (spec.get("features") != MODEL_FEATURES or spec.get("variants") != NUM_VARIANTS
            or len(spec.get("params", ())) != MODEL_PARAMS):
        return {}
    m = Model(ctx)
    m.set_params(np.asarray(spec["params"], dtype=np.float32))
    return {"policy": SCHED_LEARNED, "model": m,
            "order_by_cost": int(spec.get("order_by_cost", 1)),
            "margin": float(spec.get("margin", 0.0))}


# ------------------------------------------------------------------ generators
def _two(m: int):
    return np.empty(m, dtype=np.int32), np.empty(m, dtype=np.int32)


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, seed: int = 1):
    m = lib().xgm_gen_rmat(scale, edge_factor, a, b, c, seed, None, None)
    if m < 0:
        raise XgmError(ERR_INVALID, "bad R-MAT parameters")
    s, d = _two(m)
    lib().xgm_gen_rmat(scale, edge_factor, a, b, c, seed, _ptr(s), _ptr(d))
    return 1 << scale, s, d


def gen_er(n: int, m: int, seed: int = 1):
    if lib().xgm_gen_er(n, m, seed, None, None) < 0:
        raise XgmError(ERR_INVALID, "bad G(n,m) parameters")
    s, d = _two(m)
    lib().xgm_gen_er(n, m, seed, _ptr(s), _ptr(d))
    return n, s, d


def gen_chung_lu(n: int, gamma: float = 2.1, w_max: float = 50000.0, avg_deg: float = 32.0,
                 seed: int = 1):
    m = lib().xgm_gen_chung_lu(n, gamma, w_max, avg_deg, seed, None, None)
    if m < 0:
        raise XgmError(ERR_INVALID, "bad Chung-Lu parameters")
    s, d = _two(m)
    lib().xgm_gen_chung_lu(n, gamma, w_max, avg_deg, seed, _ptr(s), _ptr(d))
    return n, s, d


def gen_ba(n: int, m: int, seed: int = 1):
    ne = lib().xgm_gen_ba(n, m, seed, None, None)
    if ne < 0:
        raise XgmError(ERR_INVALID, "bad Barabasi-Albert parameters")
    s, d = _two(ne)
    lib().xgm_gen_ba(n, m, seed, _ptr(s), _ptr(d))
    return n, s, d


def gen_ba_batch(num_graphs: int, n_lo: int = 100, n_hi: int = 5000, m_lo: int = 3,
                 m_hi: int = 8, seed: int = 5):
    vo = np.empty(num_graphs + 1, dtype=np.int64)
    eo = np.empty(num_graphs + 1, dtype=np.int64)
    ne = lib().xgm_gen_ba_batch(num_graphs, n_lo, n_hi, m_lo, m_hi, seed, _ptr(vo), _ptr(eo),
                                None, None)
    if ne < 0:
        raise XgmError(ERR_INVALID, "bad batch parameters")
    s, d = _two(ne)
    lib().xgm_gen_ba_batch(num_graphs, n_lo, n_hi, m_lo, m_hi, seed, _ptr(vo), _ptr(eo), _ptr(s),
                           _ptr(d))
    return vo, eo, s, d

/*
 * xgm.h - C ABI of the GB300 pattern-counting engine.
 *
 * The engine takes a graph plus a pattern plan and returns exact uint64 counts.
 * It replaces the counting call of X-GMiner / GLUMIN / G2Miner:
 *
 *   TCSolver(Graph&, uint64_t& total, int n_gpu, int chunk)
 *       codes/GraphMiner/src/triangle/main.cc:5, impl gpu_base.cu:25-74
 *   CliqueSolver(Graph&, int k, uint64_t& total, int, int)
 *       codes/GraphMiner/src/clique/main.cc:6, impl clique/gpu_base.cu:16
 *   ScSolver(Graph&, Pattern&, uint64_t& total, int, int)
 *       codes/GraphMiner/src/count/main.cc:7, impl count/omp_base.cc:5-58
 *   GLUMIN::CliqueSolver_[LUT_]on_G2Miner(Graph_V2&) writing total[0]
 *       xgminer/include/glumin.h:82-86, xgminer/src/glumin/glumin_GM_solver.cu:1083-1235
 *
 * Conventions.
 *  - Every call returns an xgm_status; nothing exits or aborts.  A device-side error
 *    flag (bounds, bounded-wait timeout) is reported as XGM_ERR_DEVICE / XGM_ERR_TIMEOUT.
 *  - Host buffers belong to the caller and are copied; device memory and the CUDA
 *    stream belong to the context and are released by the matching *_destroy call.
 *  - A context is used by one host thread at a time; contexts are independent.
 *  - Vertex ids are int32 (vidType, codes/GraphMiner/include/common.h:36), row
 *    pointers int64 (eidType, common.h:37), counts uint64 (AccType, common.h:40).
 */
#ifndef XGM_H_
#define XGM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum {
  XGM_OK = 0,
  XGM_ERR_INVALID = 1,     /* bad argument */
  XGM_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  XGM_ERR_OOM = 3,         /* device allocation failed */
  XGM_ERR_DEVICE = 4,      /* a kernel raised its error flag (bounds check) */
  XGM_ERR_TIMEOUT = 5,     /* a bounded device-side wait ran out */
  XGM_ERR_UNSUPPORTED = 6, /* pattern / option not implemented */
  XGM_ERR_IO = 7,          /* graph file missing or malformed */
  XGM_ERR_GRAPH = 8,       /* CSR failed validation (unsorted, self-loop, id out of range) */
  XGM_ERR_NO_DEVICE = 9    /* no CUDA device visible */
} xgm_status;

const char* xgm_status_string(xgm_status s);

typedef struct xgm_ctx xgm_ctx;
typedef struct xgm_graph xgm_graph;
typedef struct xgm_plan xgm_plan;
typedef struct xgm_batch xgm_batch;
typedef struct xgm_model xgm_model;

/* ----------------------------------------------------------------- context */
typedef struct {
  int device;        /* CUDA ordinal */
  int reserved_flags;
} xgm_config;

/* Creates a context on cfg->device (NULL: device 0) with its own stream. */
xgm_status xgm_create(xgm_ctx** out, const xgm_config* cfg);
void xgm_destroy(xgm_ctx* ctx);
/* Text of the last error raised on this context (never NULL). */
const char* xgm_last_error(const xgm_ctx* ctx);
/* The context's CUDA stream, as a void* cudaStream_t. */
void* xgm_stream(xgm_ctx* ctx);

/* ------------------------------------------------------------------- graph */
/* Host CSR in the reference's binary layout: rowptr int64[V+1] (graph.vertex.bin),
 * colidx int32[E] (graph.edge.bin); graph_v2.cpp:23-49, graph.cc:20-45. */
typedef struct {
  int64_t num_vertices;
  int64_t num_edges;
  const int64_t* rowptr;
  const int32_t* colidx;
} xgm_csr_host;

enum {
  XGM_BUILD_SYMMETRIZE = 1,  /* add (v,u) for every (u,v) */
  XGM_BUILD_DEDUP = 2,       /* drop repeated edges */
  XGM_BUILD_DROP_SELF = 4,   /* drop (v,v) */
  XGM_BUILD_VALIDATE = 8,    /* upload only: reject unsorted/duplicate/self/out-of-range */
  XGM_BUILD_CLEAN = 7        /* SYMMETRIZE|DEDUP|DROP_SELF */
};

typedef struct {
  int64_t num_vertices;
  int64_t num_edges;      /* undirected CSR entries (2 x undirected edges) */
  int64_t num_dag_edges;  /* edges kept by the degree orientation */
  int64_t max_degree;
  int64_t max_out_degree; /* of the oriented DAG */
  int64_t num_triangles_hint; /* reserved, 0 */
} xgm_graph_info;

/* Uploads an undirected CSR (as Graph_V2 loads it) and builds on the GPU the degree
 * orientation (graph_v2.cpp:243-289), the vertex ranking used by the kernels and the
 * task lists.  The CSR must be symmetric with sorted rows (as the reference's inputs
 * are); flags: XGM_BUILD_VALIDATE checks that on the GPU; XGM_BUILD_CLEAN bits re-run
 * the CSR build over the given entries (symmetrising them). */
xgm_status xgm_graph_upload(xgm_ctx* ctx, const xgm_csr_host* csr, int flags,
                            xgm_graph** out);
/* Builds the CSR on the GPU from raw edge samples (the offline step of
 * scripts/graph_format_conversion.py:20-44 plus dedupe and self-loop removal),
 * then the same as xgm_graph_upload.  Ids must lie in [0, num_vertices); without
 * XGM_BUILD_SYMMETRIZE the samples must already hold both directions of every edge. */
xgm_status xgm_graph_build_from_edges(xgm_ctx* ctx, int64_t num_vertices,
                                      const int32_t* src, const int32_t* dst,
                                      int64_t num_samples, int flags, xgm_graph** out);
/* Loads <prefix>.meta.txt / .vertex.bin / .edge.bin (graph_v2.cpp:5-134). */
xgm_status xgm_graph_load(xgm_ctx* ctx, const char* prefix, int flags, xgm_graph** out);
xgm_status xgm_graph_info_get(const xgm_graph* g, xgm_graph_info* out);
enum { XGM_VIEW_UNDIRECTED = 0, XGM_VIEW_DAG = 1 };
/* Copies a CSR view back to host arrays sized from xgm_graph_info (original ids). */
xgm_status xgm_graph_download(xgm_ctx* ctx, const xgm_graph* g, int view, int64_t* rowptr,
                              int32_t* colidx);
/* Graphs (and models) must be destroyed before the context they were created on. */
void xgm_graph_destroy(xgm_graph* g);

/* Host-side file helpers in the reference layout. */
xgm_status xgm_graph_write_files(const char* prefix, const xgm_csr_host* csr);

/* -------------------------------------------------------------------- plan */
/* Builtin patterns.  Cliques and the triangle run on the degree-oriented DAG
 * (USE_DAG, codes/GraphMiner/include/defines.h:12); the other motifs are
 * edge-induced counts on the undirected graph (count/omp_base.cc:5-58) unless the
 * plan is vertex-induced. */
typedef enum {
  XGM_PATTERN_TRIANGLE = 1,
  XGM_PATTERN_CLIQUE4 = 2,
  XGM_PATTERN_CLIQUE5 = 3,
  XGM_PATTERN_DIAMOND = 4,          /* diamond.h; GLUMIN 4-diamond.yml */
  XGM_PATTERN_CYCLE4 = 5,           /* rectangle.h; GLUMIN 4-cycle.yml */
  XGM_PATTERN_TAILED_TRIANGLE = 6,  /* tailedtriangle.h; GLUMIN 4-tailed-triangle.yml */
  XGM_PATTERN_WEDGE = 7,            /* 2-edge path; GLUMIN 3-path.yml, motif k = 3 */
  XGM_PATTERN_STAR3 = 8,            /* K_{1,3}; GLUMIN 4-star.yml (P1) */
  XGM_PATTERN_PATH4 = 9,            /* 3-edge path; GLUMIN 4-path.yml */
  XGM_PATTERN_CLIQUE6 = 10,         /* GLUMIN P23 (clique6_warp_edge*.cuh) */
  XGM_PATTERN_CLIQUE7 = 11,         /* GLUMIN P24 (clique7_warp_edge*.cuh) */
  XGM_PATTERN_PROGRAM = 12          /* set-operation program: GLUMIN's P6..P22, or a
                                       compiled connected pattern of up to 6 vertices */
} xgm_pattern;

/* Words of a set-operation program in flat form (xgm_plan_program). */
#define XGM_PROGRAM_WORDS 162

typedef struct {
  int builtin;            /* xgm_pattern, or 0 to match `adj`: a builtin when one has this
                             shape, else a compiled set-operation program (connected
                             patterns of up to 6 vertices, each occurrence counted once);
                             XGM_PATTERN_PROGRAM compiles `adj` even where a builtin exists */
  int num_vertices;       /* pattern size when builtin == 0 (3..6; 7 for the 7-clique) */
  uint8_t adj[8][8];      /* pattern adjacency when builtin == 0 */
  int induced;            /* 0: edge-induced; 1: vertex-induced (the non-clique motifs are
                             derived from edge-induced counts, the 4-clique count and the
                             4-cycle count through exact identities; cliques are the same
                             either way) */
} xgm_plan_desc;

xgm_status xgm_plan_compile(xgm_ctx* ctx, const xgm_plan_desc* desc, xgm_plan** out);
/* Plan for a reference pattern name: the count app's names ("triangle", "4-clique",
 * "5-clique", "diamond", "rectangle", "tailedtriangle"; Pattern(name),
 * count/main.cc:17) and GLUMIN's .yml names ("3-triangle", "4-cycle", "4-diamond",
 * "4-tailed-triangle", "3-path", "4-path", "4-star"), all edge-induced; and GLUMIN's
 * pattern ids (codes/GLUMIN/src/G2Miner/main.cc:13-60), vertex-induced: "P1" (4-star),
 * "P2" (4-diamond, reported as GLUMIN does: each diamond once per direction of its
 * shared edge, i.e. twice), "P3" (4-tailed-triangle), "P4"/"P5"/"P23"/"P24"
 * (4/5/6/7-clique), and "P6".."P22", GLUMIN's generated 5-vertex plans
 * (G2Miner/gpu_GM_LUT_kernels/GM_kernels/P*-GM.yml.cuh) run as set-operation
 * programs with GLUMIN's own set semantics: the count is the reference's, including
 * the embeddings with a repeated vertex that P12, P13, P19 and P22 admit.  The
 * 5-vertex .yml names ("5-cycle", "5-double-triangle", "5-house", "5-path",
 * "5-solid-house", "5-star", "5-tailed-square") give compiled edge-induced programs. */
xgm_status xgm_plan_from_name(xgm_ctx* ctx, const char* name, xgm_plan** out);
/* Plan from a GLUMIN pattern description, the text of one of
 * the .yml files in codes/GLUMIN/codegen/codegen/patterns: its `edges: [AB, AC, ...]` list (vertices
 * named by letters) is matched against the builtins, else compiled to a set-operation
 * program (up to 6 vertices).  GLUMIN's plans count vertex-induced embeddings (pass
 * induced = 1 for the same meaning). */
xgm_status xgm_plan_from_spec(xgm_ctx* ctx, const char* spec, int induced, xgm_plan** out);
int xgm_plan_pattern(const xgm_plan* p);
/* A program plan's flat form: [2 (format version), k, slots, flat, v1 < v0 task filter,
 * ops per level (4), v2 / v3 / v4 candidate operands, then 25 operations of six words
 * (out slot, kind 0 intersect /
 * 1 difference / 2 filter, operand a, operand b, bound mask, exclusion mask); an
 * operand >= 16 is N(v_(operand-16)), below it a slot].  Returns XGM_PROGRAM_WORDS
 * (writing words[] when n_words is at least that), 0 for a builtin plan. */
int xgm_plan_program(const xgm_plan* p, int32_t* words, int n_words);
int xgm_plan_induced(const xgm_plan* p);
void xgm_plan_destroy(xgm_plan* p);

/* ---------------------------------------------------------------- schedule */
typedef enum {
  XGM_SCHED_HEURISTIC = 0, /* degree-threshold split (common.h:114-116 analogue) */
  XGM_SCHED_LEARNED = 1,   /* MLP cost model picks variant + order; needs a model */
  XGM_SCHED_FIXED = 2,     /* force `variant` for every task (tuning / logging) */
  XGM_SCHED_TUNED = 3      /* per out-degree bucket variant table from xgm_autotune */
} xgm_sched_policy;

/* Kernel variants a task can run with. */
typedef enum {
  XGM_VAR_WARP = 0,   /* one warp per task, frontier bitmap in shared memory */
  XGM_VAR_CTA = 1,    /* one CTA per task, frontier bitmap in shared memory */
  XGM_VAR_SPLIT = 2,  /* task split into per-edge sub-tasks (hub vertices) */
  XGM_VAR_WIDE = 3,   /* one warp per task, 4-word frontier bitmap rows (out-degree <= 128) */
  XGM_VAR_SEARCH = 4, /* one warp per task (out-degree <= 32), rows by binary search */
  XGM_VAR_BUCKET = 5, /* as SEARCH, behind X-GMiner's bucket-bitmap pre-filter: 16 buckets
                         per out-list, only common buckets searched
                         (xgminer/include/xgminer_bitmap.cuh:161-278, 661-813) */
  XGM_VAR_GROUP = 6,  /* eight lanes per task, four tasks per warp (out-degree <= 8), rows
                         by binary search */
  XGM_NUM_VARIANTS = 7
} xgm_variant;

/* Autotuned schedule: the variant for each out-degree bucket.  Bucket b holds
 * out-degrees s with floor(log2(s)) == b - 1 (bucket 0: s == 0), the last bucket
 * everything above.  A variant that cannot hold a task falls back by capacity. */
#define XGM_TUNE_BUCKETS 16
typedef struct {
  uint8_t variant[XGM_TUNE_BUCKETS];
} xgm_tune_table;

typedef struct {
  int policy;             /* xgm_sched_policy */
  int variant;            /* for XGM_SCHED_FIXED */
  const xgm_model* model; /* for XGM_SCHED_LEARNED */
  int warp_max;           /* heuristic: out-degree <= warp_max -> WARP (0: default 32) */
  int cta_max;            /* heuristic: out-degree <= cta_max -> CTA, else SPLIT (0: default 1024) */
  int order_by_cost;      /* learned: 1 = heaviest predicted tasks first */
  const xgm_tune_table* table; /* for XGM_SCHED_TUNED */
  int flags;              /* XGM_SCHED_NO_GRAPH: batched calls launch directly, no CUDA graph;
                             XGM_SCHED_HASH_ONLY: CTA tasks test membership with the Bloom
                             filter and hash even where the span bitmap fits (same counts) */
  int wide_max;           /* heuristic: out-degree <= wide_max -> WIDE (0: default 128; -1: none) */
  int search_max;         /* heuristic: out-degree <= search_max -> SEARCH (0: none) */
  int bucket_max;         /* heuristic: out-degree <= bucket_max -> BUCKET (0: none) */
  int group_max;          /* heuristic: out-degree <= group_max -> GROUP (0: none; <= 8) */
  float margin;           /* learned: predicted log2-cost saving a task needs to leave the
                             heuristic's variant (0: default 0.2) */
  int hub_max;            /* 3- to 5-clique counts: a hub task (out-degree above the CTA
                             capacity, 1024) of out-degree <= hub_max runs whole in the hub kernel
                             (one 1024-thread CTA, shared-memory bitmap) instead of being
                             split into one sub-task per out-edge (0: default, 1536 for
                             3- and 4-cliques and every hub split for 5-cliques; -1: every
                             hub split) */
} xgm_sched;

enum { XGM_SCHED_NO_GRAPH = 1, XGM_SCHED_HASH_ONLY = 2 };

typedef struct {
  double kernel_ms;        /* device time of the counting launch(es) */
  double prep_ms;          /* device time of task generation / scheduling */
  int64_t tasks;           /* top-level tasks */
  int64_t variant_tasks[XGM_NUM_VARIANTS];
  uint64_t algo_bytes;     /* algorithmic adjacency bytes of the plan (0 unless requested) */
  uint32_t device_error;   /* raw device error flag */
  int launches;            /* kernels launched by the call */
} xgm_stats;

/* Counts `plan` on `g`.  out_count receives the exact uint64 total. */
xgm_status xgm_count(xgm_ctx* ctx, const xgm_graph* g, const xgm_plan* plan,
                     const xgm_sched* sched, uint64_t* out_count, xgm_stats* stats);

/* Vertex-induced k-motif census, replaces MotifSolver(g, k, total)
 * (codes/GraphMiner/src/motif/omp_formula.cc:8, main.cc:8-31), same output order:
 * k = 3 (n_counts >= 2): [wedges, triangles];
 * k = 4 (n_counts >= 6): [3-stars, 4-paths, tailed triangles, 4-cycles, diamonds,
 * 4-cliques]. */
xgm_status xgm_motif_count(xgm_ctx* ctx, const xgm_graph* g, int k, const xgm_sched* sched,
                           uint64_t* counts, int n_counts, xgm_stats* stats);

/* Reference-shaped convenience entry points (same meaning as the solvers cited in the
 * file header; n_gpu / chunk arguments are dropped: one GPU, persistent queue). */
xgm_status xgm_tc_solver(xgm_ctx* ctx, const xgm_graph* g, uint64_t* total);
xgm_status xgm_clique_solver(xgm_ctx* ctx, const xgm_graph* g, int k, uint64_t* total);
xgm_status xgm_sc_solver(xgm_ctx* ctx, const xgm_graph* g, const char* pattern,
                         uint64_t* total);

/* Number of kernels one xgm_count call with these arguments launches (the call's
 * device work is captured once into a CUDA graph and its kernel nodes counted). */
xgm_status xgm_count_kernels(xgm_ctx* ctx, const xgm_graph* g, const xgm_plan* plan,
                             const xgm_sched* sched, int* n_kernels);

/* Triangle count that allocates no device memory.  No counterpart in the reference.
 * For callers that cannot allocate while they count (a host framework that owns all
 * device memory through its own allocator, a hot loop with no room for cudaMalloc):
 * the task lists and counters live in a 48 MiB file-scope device array instead of
 * memory allocated per call, so graphs of up to 2^21 vertices are accepted (larger:
 * XGM_ERR_UNSUPPORTED).  Same result as xgm_tc_solver; the graph must belong to ctx.
 * All calls share the array and it keeps the last call's contents (each call clears
 * what it reuses), so calls whose GPU work overlaps race.  The first call on a device
 * resolves the array's address and should come before any stream capture.  The call
 * waits for ctx's stream and leaves the caller's current device unchanged. */
xgm_status xgm_tc_solver_static(xgm_ctx* ctx, const xgm_graph* g, uint64_t* total);

/* Algorithmic adjacency bytes the plan reads on g (host pass over the downloaded
 * graph; 4 B per int32 element + 8 B per task), used as the roofline numerator. */
xgm_status xgm_algo_bytes(xgm_ctx* ctx, const xgm_graph* g, const xgm_plan* plan,
                          uint64_t* bytes);

/* ----------------------------------------------------------------- autotuner */
/* Empirical search of the per-bucket variant table for `plan` on g (or on a batch when
 * g is NULL and b is set): coordinate descent over buckets, each candidate timed as
 * the median of `reps` counts; the counts are checked equal to the first.  `best_ms` /
 * `heuristic_ms` report the tuned and plain per-call times.  No counterpart in the
 * reference (its thresholds are compile-time constants, common.h:114-116). */
typedef struct {
  xgm_tune_table table;
  double best_ms;
  double heuristic_ms;
  int trials;
} xgm_tune_result;
xgm_status xgm_autotune(xgm_ctx* ctx, const xgm_graph* g, xgm_batch* b, const xgm_plan* const* plans,
                        int n_plans, int reps, xgm_tune_result* out);

/* ------------------------------------------------------------------- batches */
/* Many small graphs counted together.  Graph i owns vertices [vtx_off[i], vtx_off[i+1])
 * of one packed id space; edge samples (or CSR entries) use those global ids and never
 * cross graphs.  The reference counts one graph per process run (GLUMIN::run,
 * xgminer/include/glumin.h:56); this is the batched form of that call. */
xgm_status xgm_batch_build_from_edges(xgm_ctx* ctx, int num_graphs, const int64_t* vtx_off,
                                      const int32_t* src, const int32_t* dst,
                                      int64_t num_samples, int flags, xgm_batch** out);
xgm_status xgm_batch_upload(xgm_ctx* ctx, int num_graphs, const int64_t* vtx_off,
                            const xgm_csr_host* csr, int flags, xgm_batch** out);
int xgm_batch_num_graphs(const xgm_batch* b);
/* The batch's packed graph (for xgm_graph_download / xgm_graph_info_get); owned by b. */
const xgm_graph* xgm_batch_graph(const xgm_batch* b);
/* Counts every plan on every graph of the batch: out[i * n_plans + p].  Triangle,
 * 4-clique, diamond and tailed-triangle plans run in one persistent launch (plus a
 * per-graph reduction); 5-clique and 4-cycle add one launch each.  The device work is
 * captured into a CUDA graph on the first call for a (plan set, schedule) and replayed
 * afterwards, unless sched->flags has XGM_SCHED_NO_GRAPH. */
xgm_status xgm_count_batched(xgm_ctx* ctx, xgm_batch* b, const xgm_plan* const* plans,
                             int n_plans, const xgm_sched* sched, uint64_t* out,
                             xgm_stats* stats);
void xgm_batch_destroy(xgm_batch* b);

/* -------------------------------------------------------------- cost model */
/* Learned scheduler: a 12 -> 32 (ReLU) -> 1 MLP with fp16 weights and fp32
 * accumulation that predicts log2(warp-cycles) of a task under a kernel variant.  It is
 * trained by the engine's own forward/backward kernels on per-task timings the engine
 * logs (xgm_model_collect), and used by XGM_SCHED_LEARNED to pick each task's variant
 * and to order the queues heaviest-first.  It changes the schedule only, never a count.
 * No counterpart in the reference (its schedule is the fixed heuristic of
 * xgminer/include/glumin/common.h:114-116). */
#define XGM_MODEL_FEATURES 12
#define XGM_MODEL_HIDDEN 32
#define XGM_MODEL_PARAMS (XGM_MODEL_HIDDEN * XGM_MODEL_FEATURES + 2 * XGM_MODEL_HIDDEN + 1)

/* Parameter layout (fp32 view): W1[32][12] row-major, b1[32], w2[32], b2. */
xgm_status xgm_model_create(xgm_ctx* ctx, uint64_t seed, xgm_model** out);
void xgm_model_destroy(xgm_model* m);
xgm_status xgm_model_set_params(xgm_model* m, const float* params);
xgm_status xgm_model_get_params(const xgm_model* m, float* params);
/* Runs `plan` on g with every task forced to `variant` (tasks the variant cannot hold
 * fall back by capacity) and per-task timing on, and returns samples of the tasks that
 * ran with `variant`: features X[n][12], targets y[n] = log2(cycles * warps used), for
 * every `stride`-th such task, at most max_rows.  count_out (optional) gets the count.
 * With XGM_COLLECT_MULTI or-ed into `variant` (plan: triangle) the timed launch is the
 * batched multi-pattern one (triangles + 4-cliques + triangle participation per task,
 * xgm_count_batched), its tasks described as 4-clique tasks. */
#define XGM_COLLECT_MULTI 0x100
xgm_status xgm_model_collect(xgm_ctx* ctx, const xgm_graph* g, const xgm_plan* plan, int variant,
                             int stride, float* X, float* y, int64_t max_rows, int64_t* n_rows,
                             uint64_t* count_out);
/* Adam on mean squared error, minibatches of `batch`, on the GPU. */
xgm_status xgm_model_train(xgm_ctx* ctx, xgm_model* m, const float* X, const float* y, int64_t n,
                           int epochs, int batch, float lr, uint64_t seed, float* final_loss);
xgm_status xgm_model_predict(xgm_ctx* ctx, const xgm_model* m, const float* X, int64_t n,
                             float* y);
/* Mean squared error and its gradient with respect to the (fp16-rounded) parameters. */
xgm_status xgm_model_loss_grad(xgm_ctx* ctx, const xgm_model* m, const float* X, const float* y,
                               int64_t n, float* loss, float* grad);

/* ------------------------------------------------------ generators (host) */
/* Write `m` raw samples to caller arrays; with src == NULL return the sample count.
 * Returns -1 on bad arguments. */
int64_t xgm_gen_rmat(int scale, int edge_factor, double a, double b, double c,
                     uint64_t seed, int32_t* src, int32_t* dst);
int64_t xgm_gen_er(int64_t n, int64_t m, uint64_t seed, int32_t* src, int32_t* dst);
int64_t xgm_gen_chung_lu(int64_t n, double gamma, double w_max, double avg_deg,
                         uint64_t seed, int32_t* src, int32_t* dst);
int64_t xgm_gen_ba(int64_t n, int m, uint64_t seed, int32_t* src, int32_t* dst);
int64_t xgm_gen_ba_batch(int num_graphs, int64_t n_lo, int64_t n_hi, int m_lo, int m_hi,
                         uint64_t seed, int64_t* vtx_off, int64_t* edge_off, int32_t* src,
                         int32_t* dst);

#ifdef __cplusplus
}
#endif
#endif /* XGM_H_ */

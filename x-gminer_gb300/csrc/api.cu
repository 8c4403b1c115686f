// C ABI of the engine (include/xgm.h): contexts, graphs, plans and the counting calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"
#include "io.h"
#include "measure.cuh"
#include "motif.cuh"
#include "prim.cuh"

namespace xgm {

thread_local std::string g_thread_error;

void set_thread_error(const std::string& msg) { g_thread_error = msg; }

xgm_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  set_thread_error(std::string("CUDA error '") + cudaGetErrorString(e) + "' in " + what + " at " +
                   file + ":" + std::to_string(line));
  cudaGetLastError();  // clear a sticky launch error where possible
  return e == cudaErrorMemoryAllocation ? XGM_ERR_OOM : XGM_ERR_CUDA;
}

namespace {

__global__ void k_csr_to_samples(const int64_t* rowptr, const int32_t* col, int64_t nv,
                                 int32_t* src, int32_t* dst) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < nv; u += warps)
    for (int64_t e = rowptr[u] + lane; e < rowptr[u + 1]; e += 32) {
      src[e] = (int32_t)u;
      dst[e] = col[e];
    }
}

inline unsigned warp_grid(int64_t nv) {
  int64_t b = (nv * 32 + 255) / 256;
  if (b < 1) b = 1;
  if (b > 65536) b = 65536;
  return (unsigned)b;
}

}  // namespace

xgm_status finish_status(xgm_ctx* ctx, xgm_status st) {
  if (st != XGM_OK && ctx) ctx->last_error = g_thread_error;
  return st;
}

xgm_status check_device_flag(xgm_ctx* ctx, uint32_t flag) {
  if (flag == 0) return XGM_OK;
  std::string m = "device error flag 0x" + std::to_string(flag) + ":";
  if (flag & ERR_CAPACITY) m += " task exceeded its variant's capacity;";
  if (flag & ERR_BOUNDS) m += " index or input validation check failed;";
  if (flag & ERR_TIMEOUT) m += " bounded wait ran out;";
  set_thread_error(m);
  if (ctx) ctx->last_error = m;
  return (flag & ERR_TIMEOUT) ? XGM_ERR_TIMEOUT : XGM_ERR_DEVICE;
}

xgm_status ctx_sync_scalars(xgm_ctx* ctx) {
  XGM_CUDA_TRY(cudaMemcpyAsync(ctx->h_sc, ctx->d_sc, sizeof(Scalars), cudaMemcpyDeviceToHost,
                               ctx->stream));
  XGM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return XGM_OK;
}

xgm_status graph_finish_common(xgm_ctx* ctx, DevGraph& g) {
  XGM_CUDA_TRY(finish_graph(g, nullptr, 0, ctx->stream));
  XGM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return XGM_OK;
}

}  // namespace xgm

using namespace xgm;

extern "C" {

const char* xgm_status_string(xgm_status s) {
  switch (s) {
    case XGM_OK: return "ok";
    case XGM_ERR_INVALID: return "invalid argument";
    case XGM_ERR_CUDA: return "CUDA error";
    case XGM_ERR_OOM: return "out of device memory";
    case XGM_ERR_DEVICE: return "device-side check failed";
    case XGM_ERR_TIMEOUT: return "device-side wait timed out";
    case XGM_ERR_UNSUPPORTED: return "unsupported";
    case XGM_ERR_IO: return "I/O error";
    case XGM_ERR_GRAPH: return "graph failed validation";
    case XGM_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

xgm_status xgm_create(xgm_ctx** out, const xgm_config* cfg) {
  if (!out) return XGM_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_thread_error("no CUDA device visible");
    return XGM_ERR_NO_DEVICE;
  }
  const int dev = cfg ? cfg->device : 0;
  if (dev < 0 || dev >= ndev) return XGM_ERR_INVALID;
  XGM_CUDA_TRY(cudaSetDevice(dev));
  xgm_ctx* c = new xgm_ctx();
  c->device = dev;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_sc, sizeof(Scalars));
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_sc, sizeof(Scalars));
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
  if (e == cudaSuccess) {
    // keep freed stream-ordered allocations cached in the pool between calls
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  if (e != cudaSuccess) {
    xgm_status st = cuda_fail(e, "xgm_create", __FILE__, __LINE__);
    xgm_destroy(c);
    return st;
  }
  *out = c;
  return XGM_OK;
}

void xgm_destroy(xgm_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) {
    taskbuf_free(c->tb, c->stream);
    motif_buffers_free(c);
    program_buffers_free(c);
    cudaStreamSynchronize(c->stream);
  }
  if (c->d_sc) cudaFree(c->d_sc);
  if (c->h_sc) cudaFreeHost(c->h_sc);
  for (int i = 0; i < 4; ++i)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* xgm_last_error(const xgm_ctx* ctx) {
  if (ctx && !ctx->last_error.empty()) return ctx->last_error.c_str();
  return g_thread_error.c_str();
}

void* xgm_stream(xgm_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

// ------------------------------------------------------------------- graphs
xgm_status xgm_graph_build_from_edges(xgm_ctx* ctx, int64_t nv, const int32_t* src,
                                      const int32_t* dst, int64_t m, int flags, xgm_graph** out) {
  if (!ctx || !out || nv <= 0 || nv > (int64_t(1) << 31) - 1 || m < 0 || (m > 0 && (!src || !dst)))
    return XGM_ERR_INVALID;
  *out = nullptr;
  cudaStream_t s = ctx->stream;
  int32_t *ds = nullptr, *dd = nullptr;
  auto fail = [&](xgm_status st) {
    if (ds) cudaFreeAsync(ds, s);
    if (dd) cudaFreeAsync(dd, s);
    return finish_status(ctx, st);
  };
  cudaError_t e = cudaMallocAsync(&ds, sizeof(int32_t) * (m > 0 ? m : 1), s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dd, sizeof(int32_t) * (m > 0 ? m : 1), s);
  if (e == cudaSuccess && m > 0)
    e = cudaMemcpyAsync(ds, src, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && m > 0)
    e = cudaMemcpyAsync(dd, dst, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_sc, 0, sizeof(Scalars), s);
  xgm_graph* g = new xgm_graph();
  g->ctx = ctx;
  if (e == cudaSuccess)
    e = build_csr_from_samples(nv, ds, dd, m, flags & XGM_BUILD_CLEAN, g->g, &ctx->d_sc->err, s);
  if (e != cudaSuccess) {
    free_graph(g->g, s);
    delete g;
    return fail(cuda_fail(e, "xgm_graph_build_from_edges", __FILE__, __LINE__));
  }
  xgm_status st = ctx_sync_scalars(ctx);
  if (st == XGM_OK && ctx->h_sc->err) {
    set_thread_error("edge sample ids outside [0, num_vertices)");
    st = XGM_ERR_GRAPH;
  }
  if (st == XGM_OK) st = graph_finish_common(ctx, g->g);
  cudaFreeAsync(ds, s);
  cudaFreeAsync(dd, s);
  ds = dd = nullptr;
  if (st != XGM_OK) {
    free_graph(g->g, s);
    delete g;
    return fail(st);
  }
  *out = g;
  return XGM_OK;
}

xgm_status xgm_graph_upload(xgm_ctx* ctx, const xgm_csr_host* csr, int flags, xgm_graph** out) {
  if (!ctx || !csr || !out || csr->num_vertices <= 0 ||
      csr->num_vertices > (int64_t(1) << 31) - 1 || csr->num_edges < 0 || !csr->rowptr ||
      (csr->num_edges > 0 && !csr->colidx))
    return XGM_ERR_INVALID;
  *out = nullptr;
  cudaStream_t s = ctx->stream;
  const int64_t nv = csr->num_vertices, ne = csr->num_edges;
  if (csr->rowptr[0] != 0 || csr->rowptr[nv] != ne) {
    set_thread_error("rowptr must start at 0 and end at num_edges");
    return finish_status(ctx, XGM_ERR_GRAPH);
  }
  xgm_graph* g = new xgm_graph();
  g->ctx = ctx;
  DevGraph& G = g->g;
  G.nv = nv;
  G.ne = ne;
  cudaError_t e = cudaMallocAsync(&G.rowptr_o, sizeof(int64_t) * (nv + 1), s);
  if (e == cudaSuccess) e = cudaMallocAsync(&G.col_o, sizeof(int32_t) * (ne > 0 ? ne : 1), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(G.rowptr_o, csr->rowptr, sizeof(int64_t) * (nv + 1), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && ne > 0)
    e = cudaMemcpyAsync(G.col_o, csr->colidx, sizeof(int32_t) * ne, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_sc, 0, sizeof(Scalars), s);
  xgm_status st = XGM_OK;
  if (e == cudaSuccess && (flags & XGM_BUILD_CLEAN)) {
    // rebuild over the given entries as raw samples
    int32_t *ds = nullptr, *dd = nullptr;
    e = cudaMallocAsync(&ds, sizeof(int32_t) * (ne > 0 ? ne : 1), s);
    if (e == cudaSuccess) e = cudaMallocAsync(&dd, sizeof(int32_t) * (ne > 0 ? ne : 1), s);
    if (e == cudaSuccess && ne > 0) {
      k_csr_to_samples<<<warp_grid(nv), 256, 0, s>>>(G.rowptr_o, G.col_o, nv, ds, dd);
      e = cudaGetLastError();
    }
    DevGraph B;
    if (e == cudaSuccess)
      e = build_csr_from_samples(nv, ds, dd, ne, flags & XGM_BUILD_CLEAN, B, &ctx->d_sc->err, s);
    if (ds) cudaFreeAsync(ds, s);
    if (dd) cudaFreeAsync(dd, s);
    if (e == cudaSuccess) {
      free_graph(G, s);
      G = B;
    } else {
      free_graph(B, s);
    }
  } else if (e == cudaSuccess && (flags & XGM_BUILD_VALIDATE)) {
    e = validate_csr(G, &ctx->d_sc->err, s);
  }
  if (e != cudaSuccess) st = cuda_fail(e, "xgm_graph_upload", __FILE__, __LINE__);
  if (st == XGM_OK) st = ctx_sync_scalars(ctx);
  if (st == XGM_OK && ctx->h_sc->err) {
    set_thread_error((flags & XGM_BUILD_CLEAN)
                         ? "entries outside [0, num_vertices)"
                         : "CSR validation failed: rows must be sorted, duplicate-free, "
                           "symmetric, without self-loops, with ids in [0, num_vertices)");
    st = XGM_ERR_GRAPH;
  }
  if (st == XGM_OK) st = graph_finish_common(ctx, G);
  if (st != XGM_OK) {
    free_graph(G, s);
    delete g;
    return finish_status(ctx, st);
  }
  *out = g;
  return XGM_OK;
}

xgm_status xgm_graph_load(xgm_ctx* ctx, const char* prefix, int flags, xgm_graph** out) {
  if (!ctx || !prefix || !out) return XGM_ERR_INVALID;
  std::vector<int64_t> rowptr;
  std::vector<int32_t> col;
  std::string msg;
  xgm_status st = read_graph_files(prefix, rowptr, col, msg);
  if (st != XGM_OK) {
    set_thread_error(msg);
    return finish_status(ctx, st);
  }
  xgm_csr_host h{(int64_t)rowptr.size() - 1, (int64_t)col.size(), rowptr.data(), col.data()};
  return xgm_graph_upload(ctx, &h, flags, out);
}

xgm_status xgm_graph_info_get(const xgm_graph* g, xgm_graph_info* out) {
  if (!g || !out) return XGM_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  out->num_vertices = g->g.nv;
  out->num_edges = g->g.ne;
  out->num_dag_edges = g->g.ne_dag;
  out->max_degree = g->g.max_deg;
  out->max_out_degree = g->g.max_out;
  return XGM_OK;
}

xgm_status xgm_graph_download(xgm_ctx* ctx, const xgm_graph* g, int view, int64_t* rowptr,
                              int32_t* colidx) {
  if (!ctx || !g || !rowptr || !colidx) return XGM_ERR_INVALID;
  cudaStream_t s = ctx->stream;
  const DevGraph& G = g->g;
  if (view == XGM_VIEW_UNDIRECTED) {
    XGM_CUDA_TRY(cudaMemcpyAsync(rowptr, G.rowptr_o, sizeof(int64_t) * (G.nv + 1),
                                 cudaMemcpyDeviceToHost, s));
    if (G.ne > 0)
      XGM_CUDA_TRY(cudaMemcpyAsync(colidx, G.col_o, sizeof(int32_t) * G.ne, cudaMemcpyDeviceToHost, s));
    XGM_CUDA_TRY(cudaStreamSynchronize(s));
    return XGM_OK;
  }
  if (view != XGM_VIEW_DAG) return XGM_ERR_INVALID;
  int64_t* dr = nullptr;
  int32_t* dc = nullptr;
  cudaError_t e = dag_original(G, &dr, &dc, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(rowptr, dr, sizeof(int64_t) * (G.nv + 1), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && G.ne_dag > 0)
    e = cudaMemcpyAsync(colidx, dc, sizeof(int32_t) * G.ne_dag, cudaMemcpyDeviceToHost, s);
  if (dr) cudaFreeAsync(dr, s);
  if (dc) cudaFreeAsync(dc, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return finish_status(ctx, cuda_fail(e, "xgm_graph_download", __FILE__, __LINE__));
  return XGM_OK;
}

void xgm_graph_destroy(xgm_graph* g) {
  if (!g) return;
  cudaStream_t s = g->ctx ? g->ctx->stream : 0;
  free_graph(g->g, s);
  if (s) cudaStreamSynchronize(s);
  delete g;
}

// -------------------------------------------------------------------- plans
xgm_status xgm_plan_compile(xgm_ctx* ctx, const xgm_plan_desc* d, xgm_plan** out) {
  if (!d || !out) return XGM_ERR_INVALID;
  *out = nullptr;
  int pat = d->builtin;
  const bool force_program = pat == XGM_PATTERN_PROGRAM;
  if (pat == 0 || force_program) {
    pat = match_pattern(d);
    if (pat < 0) {
      set_thread_error("pattern adjacency is malformed");
      return finish_status(ctx, XGM_ERR_INVALID);
    }
    if (pat == 0 || force_program) {
      // no builtin: a set-operation program (connected patterns of up to 6 vertices)
      Prog prog;
      std::string why;
      if (d->num_vertices > kProgMaxK) {
        set_thread_error("pattern not supported (builtins, or any connected pattern of up to "
                         "6 vertices)");
        return finish_status(ctx, XGM_ERR_UNSUPPORTED);
      }
      if (!prog_compile(d->num_vertices, d->adj, d->induced != 0, &prog, &why)) {
        set_thread_error("pattern not supported: " + why);
        return finish_status(ctx, XGM_ERR_UNSUPPORTED);
      }
      xgm_plan* p = new xgm_plan();
      p->pattern = XGM_PATTERN_PROGRAM;
      p->induced = d->induced ? 1 : 0;
      p->prog = prog;
      *out = p;
      return XGM_OK;
    }
  }
  if (pat < XGM_PATTERN_TRIANGLE || pat > XGM_PATTERN_CLIQUE7) return XGM_ERR_INVALID;
  xgm_plan* p = new xgm_plan();
  p->pattern = pat;
  p->induced = d->induced ? 1 : 0;
  *out = p;
  return XGM_OK;
}

xgm_status xgm_plan_from_spec(xgm_ctx* ctx, const char* spec, int induced, xgm_plan** out) {
  if (!spec || !out) return XGM_ERR_INVALID;
  *out = nullptr;
  // the `edges:` list: [AB, AC, ...]; vertices are letters A..H
  const char* e = std::strstr(spec, "edges:");
  const char* lb = e ? std::strchr(e, '[') : nullptr;
  const char* rb = lb ? std::strchr(lb, ']') : nullptr;
  if (!rb) {
    set_thread_error("pattern description has no `edges: [...]` list");
    return finish_status(ctx, XGM_ERR_INVALID);
  }
  xgm_plan_desc d;
  std::memset(&d, 0, sizeof(d));
  int nv = 0;
  for (const char* c = lb + 1; c < rb;) {
    while (c < rb && (*c == ' ' || *c == ',' || *c == '\n' || *c == '\t')) ++c;
    if (c >= rb) break;
    if (c + 1 >= rb || *c < 'A' || *c > 'H' || c[1] < 'A' || c[1] > 'H') {
      set_thread_error("pattern edges must be pairs of letters A..H");
      return finish_status(ctx, XGM_ERR_INVALID);
    }
    const int a = *c - 'A', b = c[1] - 'A';
    if (a == b) {
      set_thread_error("pattern edge joins a vertex to itself");
      return finish_status(ctx, XGM_ERR_INVALID);
    }
    d.adj[a][b] = d.adj[b][a] = 1;
    nv = std::max(nv, std::max(a, b) + 1);
    c += 2;
  }
  d.num_vertices = nv;
  d.induced = induced;
  return xgm_plan_compile(ctx, &d, out);
}

int xgm_plan_induced(const xgm_plan* p) { return p ? p->induced : 0; }

xgm_status xgm_plan_from_name(xgm_ctx* ctx, const char* name, xgm_plan** out) {
  if (!name || !out) return XGM_ERR_INVALID;
  *out = nullptr;
  // GLUMIN's 5-vertex plans P6..P22, as generated
  if (name[0] == 'P' && name[1] >= '0' && name[1] <= '9') {
    char* end = nullptr;
    const long pid = std::strtol(name + 1, &end, 10);
    Prog prog;
    if (end && *end == '\0' && pid >= 6 && pid <= 22 && prog_glumin((int)pid, &prog)) {
      xgm_plan* p = new xgm_plan();
      p->pattern = XGM_PATTERN_PROGRAM;
      p->induced = 1;
      p->prog = prog;
      *out = p;
      return XGM_OK;
    }
  }
  // GLUMIN's 5-vertex .yml names (codegen/codegen/patterns/5-*.yml), edge-induced like
  // the other .yml names
  static const struct {
    const char* name;
    const char* edges;
  } kYml5[] = {{"5-cycle", "edges: [AB, BC, CD, DE, AE]"},
               {"5-double-triangle", "edges: [AB, AC, BC, AD, AE, DE]"},
               {"5-house", "edges: [AB, AC, BC, BD, DE, CE]"},
               {"5-path", "edges: [AB, BC, CD, DE]"},
               {"5-solid-house", "edges: [AB, AC, BC, BD, BE, CD, CE, DE]"},
               {"5-star", "edges: [AB, AC, AD, AE]"},
               {"5-tailed-square", "edges: [AB, BC, CD, AD, AE]"}};
  for (const auto& y : kYml5)
    if (std::strcmp(name, y.name) == 0) return xgm_plan_from_spec(ctx, y.edges, 0, out);
  int induced = 0;
  uint64_t scale = 1;
  const int pat = pattern_from_name(name, &induced, &scale);
  if (pat <= 0) {
    set_thread_error(std::string("unknown pattern name '") + name + "'");
    return finish_status(ctx, XGM_ERR_UNSUPPORTED);
  }
  xgm_plan_desc d;
  std::memset(&d, 0, sizeof(d));
  d.builtin = pat;
  d.induced = induced;
  xgm_status st = xgm_plan_compile(ctx, &d, out);
  if (st == XGM_OK) (*out)->scale = scale;
  return st;
}

int xgm_plan_pattern(const xgm_plan* p) { return p ? p->pattern : 0; }

int xgm_plan_program(const xgm_plan* p, int32_t* words, int n_words) {
  if (!p || p->pattern != XGM_PATTERN_PROGRAM) return 0;
  static_assert(kProgWords == XGM_PROGRAM_WORDS, "program word count");
  if (words && n_words >= kProgWords) prog_to_words(p->prog, words);
  return kProgWords;
}
void xgm_plan_destroy(xgm_plan* p) { delete p; }

// ----------------------------------------------------------------- counting
xgm_status xgm_count(xgm_ctx* ctx, const xgm_graph* g, const xgm_plan* plan, const xgm_sched* sched,
                     uint64_t* out_count, xgm_stats* stats) {
  if (!ctx || !g || !plan || !out_count) return XGM_ERR_INVALID;
  xgm_sched def;
  std::memset(&def, 0, sizeof(def));
  const xgm_sched& sp = sched ? *sched : def;
  xgm_stats st_local;
  xgm_stats& st = stats ? *stats : st_local;
  std::memset(&st, 0, sizeof(st));
  xgm_status r = plan->pattern == XGM_PATTERN_PROGRAM
                     ? count_program(ctx, g->g, plan->prog, out_count, st)
                     : count_plan(ctx, g->g, plan->pattern, plan->induced, sp, out_count, st);
  if (r == XGM_OK) *out_count *= plan->scale;
  return finish_status(ctx, r);
}

xgm_status xgm_motif_count(xgm_ctx* ctx, const xgm_graph* g, int k, const xgm_sched* sched,
                           uint64_t* counts, int n_counts, xgm_stats* stats) {
  if (!ctx || !g || !counts) return XGM_ERR_INVALID;
  if ((k == 3 && n_counts < 2) || (k == 4 && n_counts < 6)) {
    set_thread_error("counts[] too short: k = 3 gives 2 counts, k = 4 gives 6");
    return finish_status(ctx, XGM_ERR_INVALID);
  }
  xgm_sched def;
  std::memset(&def, 0, sizeof(def));
  xgm_stats st_local;
  xgm_stats& st = stats ? *stats : st_local;
  std::memset(&st, 0, sizeof(st));
  return finish_status(ctx, count_motifs(ctx, g->g, k, sched ? *sched : def, counts, st));
}

xgm_status xgm_count_kernels(xgm_ctx* ctx, const xgm_graph* g, const xgm_plan* plan,
                             const xgm_sched* sched, int* n_kernels) {
  if (!ctx || !g || !plan || !n_kernels) return XGM_ERR_INVALID;
  if (plan->pattern == XGM_PATTERN_PROGRAM) {  // bitmap launch (where eligible), tasks, splits
    ProgLut lut;
    *n_kernels = plan->prog.k == 3 ? 1
                                   : (prog_lut(plan->prog, &lut) ? (lut.stream >= 0 ? 4 : 3) : 2);
    return XGM_OK;
  }
  xgm_sched def;
  std::memset(&def, 0, sizeof(def));
  return finish_status(ctx, count_kernels(ctx, g->g, plan->pattern, sched ? *sched : def, n_kernels));
}

xgm_status xgm_tc_solver(xgm_ctx* ctx, const xgm_graph* g, uint64_t* total) {
  xgm_plan p;
  p.pattern = XGM_PATTERN_TRIANGLE;
  return xgm_count(ctx, g, &p, nullptr, total, nullptr);
}

xgm_status xgm_clique_solver(xgm_ctx* ctx, const xgm_graph* g, int k, uint64_t* total) {
  if (k < 3 || k > 7) {
    set_thread_error("k-clique counting supports k = 3 .. 7");
    return finish_status(ctx, XGM_ERR_UNSUPPORTED);
  }
  static const int kPat[8] = {0, 0, 0, XGM_PATTERN_TRIANGLE, XGM_PATTERN_CLIQUE4,
                              XGM_PATTERN_CLIQUE5, XGM_PATTERN_CLIQUE6, XGM_PATTERN_CLIQUE7};
  xgm_plan p;
  p.pattern = kPat[k];
  return xgm_count(ctx, g, &p, nullptr, total, nullptr);
}

xgm_status xgm_sc_solver(xgm_ctx* ctx, const xgm_graph* g, const char* pattern, uint64_t* total) {
  xgm_plan* p = nullptr;
  xgm_status st = xgm_plan_from_name(ctx, pattern, &p);
  if (st != XGM_OK) return st;
  st = xgm_count(ctx, g, p, nullptr, total, nullptr);
  xgm_plan_destroy(p);
  return st;
}

xgm_status xgm_algo_bytes(xgm_ctx* ctx, const xgm_graph* g, const xgm_plan* plan, uint64_t* bytes) {
  if (!ctx || !g || !plan || !bytes) return XGM_ERR_INVALID;
  if (plan->pattern == XGM_PATTERN_PROGRAM) {
    set_thread_error("algorithmic bytes are defined for the builtin plans only");
    return finish_status(ctx, XGM_ERR_UNSUPPORTED);
  }
  return finish_status(ctx, algo_bytes_dispatch(ctx, g->g, plan->pattern, bytes));
}

}  // extern "C"

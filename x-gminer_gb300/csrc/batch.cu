// Batched multi-graph counting and the schedule autotuner.
//
// A batch packs many small graphs into one id space (graph i owns a contiguous vertex
// range).  The CSR build ranks vertices by (graph, degree, id), so every graph stays
// contiguous in rank order and the orientation inside each graph is the reference's
// rule (graph.cc:233-275).  One persistent launch of the counting kernel in its
// multi-pattern mode counts triangles and 4-cliques of every task and credits
// triangle participation; a per-graph reduction turns participation into diamonds and
// tailed triangles.  5-cliques and 4-cycles add one launch each.  Every task adds its
// totals to out[graph * n_plans + plan].  The whole sequence is stream-ordered with no
// host round trip, captured once into a CUDA graph per (plan set, schedule) and
// replayed.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"
#include "learned.cuh"
#include "motif.cuh"
#include "prim.cuh"

namespace xgm {

namespace {

struct CachedExec {
  std::string key;
  cudaGraphExec_t exec = nullptr;
  int kernels = 0;  // kernel nodes of the captured graph
};

}  // namespace
}  // namespace xgm

struct xgm_batch {
  xgm_ctx* ctx = nullptr;
  int num_graphs = 0;
  xgm_graph graph;  // packed graph (graph.g.gid: rank -> graph id)
  std::vector<int64_t> vtx_off;
  unsigned long long* d_out = nullptr;
  unsigned long long* h_out = nullptr;  // pinned
  int64_t out_cap = 0;
  xgm::Scalars* d_sc = nullptr;
  xgm::Scalars* h_sc = nullptr;  // pinned
  xgm::TaskBuf tb;
  unsigned long long* vpart = nullptr;
  unsigned* epart = nullptr;
  // 4-cycle buffers
  uint32_t* c4_scratch = nullptr;
  long long* wedges = nullptr;
  uint8_t* fl_large = nullptr;
  uint8_t* fl_small = nullptr;
  int64_t* c4_pos = nullptr;
  int32_t* c4_large = nullptr;
  int32_t* c4_small = nullptr;
  int64_t* c4_n = nullptr;
  std::vector<xgm::CachedExec> cache;
};

namespace xgm {

namespace {

__global__ void k_group_ids(const int64_t* vtx_off, int num_graphs, int64_t nv, int32_t* group) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = num_graphs;  // last i with vtx_off[i] <= v
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (vtx_off[mid] <= v) lo = mid; else hi = mid;
    }
    group[v] = lo;
  }
}

__global__ void k_check_samples_in_graph(const int64_t* vtx_off, int num_graphs, const int32_t* src,
                                         const int32_t* dst, int64_t m, uint32_t* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = src[i], v = dst[i];
    int lo = 0, hi = num_graphs;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (vtx_off[mid] <= u) lo = mid; else hi = mid;
    }
    if (v < vtx_off[lo] || v >= vtx_off[lo + 1]) atomicOr(err, ERR_BOUNDS);
  }
}

inline unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 65536));
}

void batch_free(xgm_batch* b) {
  cudaStream_t s = b->ctx->stream;
  for (auto& c : b->cache)
    if (c.exec) cudaGraphExecDestroy(c.exec);
  b->cache.clear();
  taskbuf_free(b->tb, s);
  void* ps[] = {b->d_out, b->vpart, b->epart, b->c4_scratch, b->wedges, b->fl_large,
                b->fl_small, b->c4_pos, b->c4_large, b->c4_small, b->c4_n};
  for (void* p : ps)
    if (p) cudaFreeAsync(p, s);
  free_graph(b->graph.g, s);
  cudaStreamSynchronize(s);
  if (b->d_sc) cudaFree(b->d_sc);
  if (b->h_sc) cudaFreeHost(b->h_sc);
  if (b->h_out) cudaFreeHost(b->h_out);
}

// Finishes a batch whose packed CSR (original ids) is in b->graph.g.
xgm_status batch_finish(xgm_ctx* ctx, xgm_batch* b) {
  cudaStream_t s = ctx->stream;
  DevGraph& g = b->graph.g;
  int64_t* d_off = nullptr;
  int32_t* group = nullptr;
  XGM_CUDA_TRY(cudaMallocAsync(&d_off, sizeof(int64_t) * (b->num_graphs + 1), s));
  XGM_CUDA_TRY(cudaMallocAsync(&group, sizeof(int32_t) * (g.nv > 0 ? g.nv : 1), s));
  XGM_CUDA_TRY(cudaMemcpyAsync(d_off, b->vtx_off.data(), sizeof(int64_t) * (b->num_graphs + 1),
                               cudaMemcpyHostToDevice, s));
  k_group_ids<<<grid_for(g.nv), 256, 0, s>>>(d_off, b->num_graphs, g.nv, group);
  XGM_CUDA_TRY(cudaGetLastError());
  XGM_CUDA_TRY(finish_graph(g, group, b->num_graphs, s));
  cudaFreeAsync(d_off, s);
  cudaFreeAsync(group, s);
  XGM_CUDA_TRY(taskbuf_reserve(b->tb, g.nv, s));
  XGM_CUDA_TRY(cudaMalloc(&b->d_sc, sizeof(Scalars)));
  XGM_CUDA_TRY(cudaMallocHost(&b->h_sc, sizeof(Scalars)));
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  return XGM_OK;
}

xgm_status check_offsets(int num_graphs, const int64_t* vtx_off) {
  if (num_graphs <= 0 || !vtx_off || vtx_off[0] != 0) return XGM_ERR_INVALID;
  for (int i = 0; i < num_graphs; ++i)
    if (vtx_off[i + 1] <= vtx_off[i]) return XGM_ERR_INVALID;
  if (vtx_off[num_graphs] > (int64_t(1) << 31) - 1) return XGM_ERR_INVALID;
  return XGM_OK;
}

struct Slots {
  int tri = -1, k4 = -1, k5 = -1, dia = -1, tail = -1, c4 = -1;
};

xgm_status slots_of(const xgm_plan* const* plans, int n, Slots& sl) {
  for (int p = 0; p < n; ++p) {
    if (!plans[p]) return XGM_ERR_INVALID;
    if (plans[p]->induced || plans[p]->scale != 1) {
      set_thread_error("vertex-induced plans are counted one graph at a time (xgm_count)");
      return XGM_ERR_UNSUPPORTED;
    }
    int* t = nullptr;
    switch (plans[p]->pattern) {
      case XGM_PATTERN_TRIANGLE: t = &sl.tri; break;
      case XGM_PATTERN_CLIQUE4: t = &sl.k4; break;
      case XGM_PATTERN_CLIQUE5: t = &sl.k5; break;
      case XGM_PATTERN_DIAMOND: t = &sl.dia; break;
      case XGM_PATTERN_TAILED_TRIANGLE: t = &sl.tail; break;
      case XGM_PATTERN_CYCLE4: t = &sl.c4; break;
      default:
        set_thread_error("batched counting covers the clique, diamond, 4-cycle and tailed "
                         "triangle plans");
        return XGM_ERR_UNSUPPORTED;
    }
    if (*t >= 0) {
      set_thread_error("a plan appears twice in the batched call");
      return XGM_ERR_INVALID;
    }
    *t = p;
  }
  return XGM_OK;
}

template <class T>
cudaError_t alloc_once(T** p, int64_t n, cudaStream_t s, bool zero = false) {
  if (*p) return cudaSuccess;
  cudaError_t e = cudaMallocAsync((void**)p, sizeof(T) * (size_t)(n > 0 ? n : 1), s);
  if (e == cudaSuccess && zero) e = cudaMemsetAsync(*p, 0, sizeof(T) * (size_t)(n > 0 ? n : 1), s);
  return e;
}

// Allocations a sequence needs, made before any capture.
xgm_status batch_prepare(xgm_ctx* ctx, xgm_batch* b, const Slots& sl, int P,
                         const xgm_sched& sp) {
  cudaStream_t s = ctx->stream;
  const DevGraph& g = b->graph.g;
  const int64_t need = (int64_t)b->num_graphs * P;
  if (b->out_cap < need) {
    if (b->d_out) cudaFreeAsync(b->d_out, s);
    if (b->h_out) cudaFreeHost(b->h_out);
    b->d_out = nullptr;
    b->h_out = nullptr;
    XGM_CUDA_TRY(cudaMallocAsync(&b->d_out, sizeof(unsigned long long) * need, s));
    XGM_CUDA_TRY(cudaMallocHost(&b->h_out, sizeof(unsigned long long) * need));
    b->out_cap = need;
    for (auto& c : b->cache)
      if (c.exec) cudaGraphExecDestroy(c.exec);
    b->cache.clear();
  }
  if (sl.dia >= 0 || sl.tail >= 0) {
    XGM_CUDA_TRY(alloc_once(&b->vpart, g.nv, s));
    XGM_CUDA_TRY(alloc_once(&b->epart, g.ne, s));
  }
  if (sl.c4 >= 0) {
    XGM_CUDA_TRY(alloc_once(&b->c4_scratch, (int64_t)cycle4_grid(ctx->num_sms) * g.nv, s, true));
    XGM_CUDA_TRY(alloc_once(&b->wedges, g.nv, s));
    XGM_CUDA_TRY(alloc_once(&b->fl_large, g.nv, s));
    XGM_CUDA_TRY(alloc_once(&b->fl_small, g.nv, s));
    XGM_CUDA_TRY(alloc_once(&b->c4_pos, g.nv, s));
    XGM_CUDA_TRY(alloc_once(&b->c4_large, g.nv, s));
    XGM_CUDA_TRY(alloc_once(&b->c4_small, g.nv, s));
    XGM_CUDA_TRY(alloc_once(&b->c4_n, 2, s));
  }
  ensure_clique_grid(ctx);
  if (sched_may_bucket(sp)) XGM_CUDA_TRY(ensure_bucket_index(g, s));  // before any capture
  if (sp.policy == XGM_SCHED_LEARNED) XGM_CUDA_TRY(ensure_task_stats(g, s));
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  return XGM_OK;
}

// The device work of one batched count: stream operations only.
xgm_status batch_sequence(xgm_ctx* ctx, xgm_batch* b, const Slots& sl, int P,
                          const xgm_sched& sp) {
  cudaStream_t s = ctx->stream;
  const DevGraph& g = b->graph.g;
  const GView view = g.view();
  const int64_t nout = (int64_t)b->num_graphs * P;
  const int grid = ensure_clique_grid(ctx);
  XGM_CUDA_TRY(cudaMemsetAsync(b->d_out, 0, sizeof(unsigned long long) * nout, s));
  XGM_CUDA_TRY(cudaMemsetAsync(b->d_sc, 0, sizeof(Scalars), s));
  if (sl.tri >= 0 || sl.k4 >= 0 || sl.dia >= 0 || sl.tail >= 0) {
    const bool part = sl.dia >= 0 || sl.tail >= 0;
    if (part) {
      XGM_CUDA_TRY(cudaMemsetAsync(b->vpart, 0, sizeof(unsigned long long) * (g.nv > 0 ? g.nv : 1), s));
      XGM_CUDA_TRY(cudaMemsetAsync(b->epart, 0, sizeof(unsigned) * (g.ne > 0 ? g.ne : 1), s));
    }
    // roots from out-degree 2 on (triangles); the learned model describes the tasks as
    // tasks of this multi-pattern launch (kFeatMulti)
    xgm_status r = schedule_into(b->tb, g, 3, sp, s, kFeatMulti);
    if (r != XGM_OK) return r;
    // without a participation plan the counters go to a dummy-free path: the multi
    // kernel always credits participation, so give it real buffers
    if (!part) {
      XGM_CUDA_TRY(alloc_once(&b->vpart, g.nv, s));
      XGM_CUDA_TRY(alloc_once(&b->epart, g.ne, s));
    }
    GOut o{g.gid, b->d_out, P, sl.tri, sl.k4};
    XGM_CUDA_TRY(launch_multi(view, b->tb.lists(false), &b->d_sc->q, b->vpart, b->epart,
                              &b->d_sc->err, grid, s, o));
    // the multi launch's task lists, for the stats
    XGM_CUDA_TRY(cudaMemcpyAsync(b->d_sc->n, b->tb.n, sizeof(int64_t) * 8,
                                 cudaMemcpyDeviceToDevice, s));
    if (part)
      XGM_CUDA_TRY(launch_part_reduce_graphs(view, g.gid, b->vpart, b->epart, b->d_out, P, sl.dia,
                                             sl.tail, s));
  }
  if (sl.k5 >= 0) {
    XGM_CUDA_TRY(cudaMemsetAsync(&b->d_sc->q, 0, sizeof(QueueHeads), s));
    xgm_status r = schedule_into(b->tb, g, 5, sp, s, 0, true);
    if (r != XGM_OK) return r;
    GOut o{g.gid, b->d_out, P, sl.k5, -1};
    XGM_CUDA_TRY(launch_clique(5, view, b->tb.lists(false), &b->d_sc->q, nullptr, &b->d_sc->err,
                               grid, s, o));
  }
  if (sl.c4 >= 0) {
    XGM_CUDA_TRY(launch_wedge_count(view, b->wedges, b->fl_large, b->fl_small, s));
    XGM_CUDA_TRY(scan_excl(b->fl_large, b->c4_pos, g.nv, b->c4_n + 0, s));
    XGM_CUDA_TRY(launch_scatter_flags(b->fl_large, b->c4_pos, g.nv, b->c4_large, s));
    XGM_CUDA_TRY(scan_excl(b->fl_small, b->c4_pos, g.nv, b->c4_n + 1, s));
    XGM_CUDA_TRY(launch_scatter_flags(b->fl_small, b->c4_pos, g.nv, b->c4_small, s));
    GOut o{g.gid, b->d_out, P, sl.c4, -1};
    XGM_CUDA_TRY(launch_cycle4(view, b->c4_large, b->c4_small, b->c4_n, b->d_sc->c4heads,
                               b->c4_scratch, nullptr, &b->d_sc->err, cycle4_grid(ctx->num_sms), s,
                               o));
  }
  XGM_CUDA_TRY(cudaMemcpyAsync(b->h_out, b->d_out, sizeof(unsigned long long) * nout,
                               cudaMemcpyDeviceToHost, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(b->h_sc, b->d_sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  return XGM_OK;
}

std::string sched_key(const Slots& sl, const xgm_sched& sp) {
  std::string k(reinterpret_cast<const char*>(&sl), sizeof(sl));
  k.append(reinterpret_cast<const char*>(&sp.policy), sizeof(int) * 2);
  k.append(reinterpret_cast<const char*>(&sp.model), sizeof(void*));
  k.append(reinterpret_cast<const char*>(&sp.warp_max), sizeof(int) * 3);
  const int more[4] = {sp.wide_max, sp.search_max, sp.bucket_max, sp.group_max};
  k.append(reinterpret_cast<const char*>(more), sizeof(more));
  k.append(reinterpret_cast<const char*>(&sp.margin), sizeof(float));
  const int hash_only = sp.flags & XGM_SCHED_HASH_ONLY;
  k.append(reinterpret_cast<const char*>(&hash_only), sizeof(int));
  if (sp.table) k.append(reinterpret_cast<const char*>(sp.table), sizeof(xgm_tune_table));
  return k;
}

xgm_status count_batched_impl(xgm_ctx* ctx, xgm_batch* b, const xgm_plan* const* plans, int P,
                              const xgm_sched& sp, uint64_t* out, xgm_stats& st) {
  cudaStream_t s = ctx->stream;
  XGM_CUDA_TRY(cudaSetDevice(ctx->device));
  Slots sl;
  xgm_status r = slots_of(plans, P, sl);
  if (r != XGM_OK) return r;
  r = batch_prepare(ctx, b, sl, P, sp);
  if (r != XGM_OK) return r;
  const bool use_graph = !(sp.flags & XGM_SCHED_NO_GRAPH);
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  if (use_graph) {
    const std::string key = sched_key(sl, sp);
    cudaGraphExec_t exec = nullptr;
    for (auto& c : b->cache)
      if (c.key == key) {
        exec = c.exec;
        st.launches = c.kernels;
      }
    if (!exec) {
      XGM_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      r = batch_sequence(ctx, b, sl, P, sp);
      cudaGraph_t graph = nullptr;
      const cudaError_t e = cudaStreamEndCapture(s, &graph);
      if (r != XGM_OK) {
        if (graph) cudaGraphDestroy(graph);
        return r;
      }
      XGM_CUDA_TRY(e);
      size_t nn = 0;
      int kern = 0;
      if (cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess && nn) {
        std::vector<cudaGraphNode_t> nodes(nn);
        if (cudaGraphGetNodes(graph, nodes.data(), &nn) == cudaSuccess)
          for (size_t i = 0; i < nn; ++i) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
              ++kern;
          }
      }
      const cudaError_t e2 = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      XGM_CUDA_TRY(e2);
      b->cache.push_back(CachedExec{key, exec, kern});
      st.launches = kern;
      XGM_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
    }
    XGM_CUDA_TRY(cudaGraphLaunch(exec, s));
  } else {
    r = batch_sequence(ctx, b, sl, P, sp);
    if (r != XGM_OK) return r;
  }
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  st.kernel_ms = ms;
  st.device_error = b->h_sc->err;
  st.tasks = b->graph.g.nv;
  if (sl.tri >= 0 || sl.k4 >= 0 || sl.dia >= 0 || sl.tail >= 0) {
    // vertex tasks per variant of the multi-pattern launch
    const int64_t* n = b->h_sc->n;
    st.variant_tasks[XGM_VAR_WARP] = n[2];
    st.variant_tasks[XGM_VAR_CTA] = n[1];
    st.variant_tasks[XGM_VAR_SPLIT] = n[0];
    st.variant_tasks[XGM_VAR_WIDE] = n[4];
    st.variant_tasks[XGM_VAR_SEARCH] = n[5];
    st.variant_tasks[XGM_VAR_BUCKET] = n[6];
    st.variant_tasks[XGM_VAR_GROUP] = n[7];
  }
  r = check_device_flag(ctx, b->h_sc->err);
  if (r != XGM_OK) return r;
  std::memcpy(out, b->h_out, sizeof(uint64_t) * (size_t)b->num_graphs * P);
  return XGM_OK;
}

}  // namespace

}  // namespace xgm

using namespace xgm;

extern "C" {

xgm_status xgm_batch_build_from_edges(xgm_ctx* ctx, int num_graphs, const int64_t* vtx_off,
                                      const int32_t* src, const int32_t* dst, int64_t m, int flags,
                                      xgm_batch** out) {
  if (!ctx || !out || m < 0 || (m > 0 && (!src || !dst))) return XGM_ERR_INVALID;
  *out = nullptr;
  xgm_status st = check_offsets(num_graphs, vtx_off);
  if (st != XGM_OK) {
    set_thread_error("vtx_off must start at 0 and increase strictly");
    return finish_status(ctx, st);
  }
  cudaStream_t s = ctx->stream;
  const int64_t nv = vtx_off[num_graphs];
  xgm_batch* b = new xgm_batch();
  b->ctx = ctx;
  b->num_graphs = num_graphs;
  b->graph.ctx = ctx;
  b->vtx_off.assign(vtx_off, vtx_off + num_graphs + 1);
  int32_t *ds = nullptr, *dd = nullptr;
  int64_t* d_off = nullptr;
  cudaError_t e = cudaMallocAsync(&ds, sizeof(int32_t) * (m > 0 ? m : 1), s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dd, sizeof(int32_t) * (m > 0 ? m : 1), s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_off, sizeof(int64_t) * (num_graphs + 1), s);
  if (e == cudaSuccess && m > 0) e = cudaMemcpyAsync(ds, src, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && m > 0) e = cudaMemcpyAsync(dd, dst, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_off, vtx_off, sizeof(int64_t) * (num_graphs + 1), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_sc, 0, sizeof(Scalars), s);
  if (e == cudaSuccess && m > 0) {
    k_check_samples_in_graph<<<grid_for(m), 256, 0, s>>>(d_off, num_graphs, ds, dd, m, &ctx->d_sc->err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = build_csr_from_samples(nv, ds, dd, m, flags & XGM_BUILD_CLEAN, b->graph.g, &ctx->d_sc->err, s);
  if (ds) cudaFreeAsync(ds, s);
  if (dd) cudaFreeAsync(dd, s);
  if (d_off) cudaFreeAsync(d_off, s);
  if (e != cudaSuccess) st = cuda_fail(e, "xgm_batch_build_from_edges", __FILE__, __LINE__);
  if (st == XGM_OK) st = ctx_sync_scalars(ctx);
  if (st == XGM_OK && ctx->h_sc->err) {
    set_thread_error("an edge sample leaves its graph's vertex range");
    st = XGM_ERR_GRAPH;
  }
  if (st == XGM_OK) st = batch_finish(ctx, b);
  if (st != XGM_OK) {
    batch_free(b);
    delete b;
    return finish_status(ctx, st);
  }
  *out = b;
  return XGM_OK;
}

xgm_status xgm_batch_upload(xgm_ctx* ctx, int num_graphs, const int64_t* vtx_off,
                            const xgm_csr_host* csr, int flags, xgm_batch** out) {
  if (!ctx || !out || !csr) return XGM_ERR_INVALID;
  *out = nullptr;
  xgm_status st = check_offsets(num_graphs, vtx_off);
  if (st != XGM_OK || csr->num_vertices != vtx_off[num_graphs]) {
    set_thread_error("vtx_off must start at 0, increase strictly and end at num_vertices");
    return finish_status(ctx, XGM_ERR_INVALID);
  }
  // entries must stay inside their row's graph
  for (int i = 0; i < num_graphs; ++i)
    for (int64_t v = vtx_off[i]; v < vtx_off[i + 1]; ++v)
      for (int64_t e = csr->rowptr[v]; e < csr->rowptr[v + 1]; ++e)
        if (csr->colidx[e] < vtx_off[i] || csr->colidx[e] >= vtx_off[i + 1]) {
          set_thread_error("a CSR entry leaves its graph's vertex range");
          return finish_status(ctx, XGM_ERR_GRAPH);
        }
  xgm_graph* tmp = nullptr;
  st = xgm_graph_upload(ctx, csr, flags, &tmp);
  if (st != XGM_OK) return st;
  xgm_batch* b = new xgm_batch();
  b->ctx = ctx;
  b->num_graphs = num_graphs;
  b->graph.ctx = ctx;
  b->vtx_off.assign(vtx_off, vtx_off + num_graphs + 1);
  // keep only the original-id CSR; ranks are recomputed with graph ids
  DevGraph& g = b->graph.g;
  g.nv = tmp->g.nv;
  g.ne = tmp->g.ne;
  g.rowptr_o = tmp->g.rowptr_o;
  g.col_o = tmp->g.col_o;
  tmp->g.rowptr_o = nullptr;
  tmp->g.col_o = nullptr;
  xgm_graph_destroy(tmp);
  st = batch_finish(ctx, b);
  if (st != XGM_OK) {
    batch_free(b);
    delete b;
    return finish_status(ctx, st);
  }
  *out = b;
  return XGM_OK;
}

int xgm_batch_num_graphs(const xgm_batch* b) { return b ? b->num_graphs : 0; }
const xgm_graph* xgm_batch_graph(const xgm_batch* b) { return b ? &b->graph : nullptr; }

xgm_status xgm_count_batched(xgm_ctx* ctx, xgm_batch* b, const xgm_plan* const* plans, int n_plans,
                             const xgm_sched* sched, uint64_t* out, xgm_stats* stats) {
  if (!ctx || !b || !plans || n_plans <= 0 || !out) return XGM_ERR_INVALID;
  xgm_sched def;
  std::memset(&def, 0, sizeof(def));
  xgm_stats local;
  xgm_stats& st = stats ? *stats : local;
  std::memset(&st, 0, sizeof(st));
  return finish_status(ctx, count_batched_impl(ctx, b, plans, n_plans, sched ? *sched : def, out, st));
}

void xgm_batch_destroy(xgm_batch* b) {
  if (!b) return;
  batch_free(b);
  delete b;
}

// ---------------------------------------------------------------- autotuner
xgm_status xgm_autotune(xgm_ctx* ctx, const xgm_graph* g, xgm_batch* b, const xgm_plan* const* plans,
                        int n_plans, int reps, xgm_tune_result* out) {
  if (!ctx || (!g && !b) || !plans || n_plans <= 0 || !out || reps <= 0) return XGM_ERR_INVALID;
  if (g && n_plans != 1) {
    set_thread_error("single-graph tuning takes one plan");
    return finish_status(ctx, XGM_ERR_INVALID);
  }
  const int64_t ng = b ? b->num_graphs : 1;
  std::vector<uint64_t> ref((size_t)ng * n_plans), cur((size_t)ng * n_plans);
  // one timed trial: median of reps per-call device times
  auto trial = [&](const xgm_sched& sp, std::vector<uint64_t>& res, double* ms) -> xgm_status {
    std::vector<double> t;
    for (int i = 0; i < reps + 1; ++i) {
      xgm_stats st;
      std::memset(&st, 0, sizeof(st));
      xgm_status r = b ? count_batched_impl(ctx, b, plans, n_plans, sp, res.data(), st)
                       : count_dispatch(ctx, g->g, plans[0]->pattern, sp, res.data(), st);
      if (r != XGM_OK) return r;
      if (i > 0) t.push_back(st.kernel_ms + st.prep_ms);  // first run warms up
    }
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return XGM_OK;
  };
  xgm_sched heur;
  std::memset(&heur, 0, sizeof(heur));
  heur.flags = XGM_SCHED_NO_GRAPH;
  double base_ms = 0;
  xgm_status r = trial(heur, ref, &base_ms);
  if (r != XGM_OK) return finish_status(ctx, r);
  xgm_tune_table tab;
  for (int k = 0; k < XGM_TUNE_BUCKETS; ++k) {
    const int64_t smax = k == 0 ? 0 : (int64_t(1) << k) - 1;
    tab.variant[k] = smax <= kWarpCap   ? XGM_VAR_WARP
                     : smax <= kWideCap ? XGM_VAR_WIDE
                     : smax <= kCtaCap  ? XGM_VAR_CTA
                                        : XGM_VAR_SPLIT;
  }
  xgm_sched ts = heur;
  ts.policy = XGM_SCHED_TUNED;
  ts.table = &tab;
  double best = 0;
  int trials = 1;
  r = trial(ts, cur, &best);
  if (r != XGM_OK) return finish_status(ctx, r);
  if (cur != ref) {
    set_thread_error("autotuner: schedules disagree on a count");
    return finish_status(ctx, XGM_ERR_DEVICE);
  }
  for (int pass = 0; pass < 2; ++pass) {
    for (int k = 1; k < XGM_TUNE_BUCKETS; ++k) {
      const int64_t smin = int64_t(1) << (k - 1);
      const uint8_t keep = tab.variant[k];
      uint8_t bestv = keep;
      for (uint8_t v = 0; v < XGM_NUM_VARIANTS; ++v) {
        if (v == keep) continue;
        if ((v == XGM_VAR_WARP || v == XGM_VAR_SEARCH || v == XGM_VAR_BUCKET) && smin > kWarpCap)
          continue;
        if (v == XGM_VAR_GROUP && smin > kGroupCap) continue;
        if (v == XGM_VAR_WIDE && smin > kWideCap) continue;
        if (v == XGM_VAR_CTA && smin > kCtaCap) continue;
        tab.variant[k] = v;
        double ms = 0;
        r = trial(ts, cur, &ms);
        ++trials;
        if (r != XGM_OK) return finish_status(ctx, r);
        if (cur != ref) {
          set_thread_error("autotuner: schedules disagree on a count");
          return finish_status(ctx, XGM_ERR_DEVICE);
        }
        if (ms < best * 0.98) {
          best = ms;
          bestv = v;
        }
      }
      tab.variant[k] = bestv;
    }
  }
  out->table = tab;
  out->best_ms = best;
  out->heuristic_ms = base_ms;
  out->trials = trials;
  return XGM_OK;
}

}  // extern "C"

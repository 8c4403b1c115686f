// Count dispatch behind xgm_count: schedule -> persistent counting launch -> uint64.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"
#include "learned.cuh"
#include "measure.cuh"
#include "motif.cuh"
#include "prim.cuh"

namespace xgm {

namespace {

template <class T>
cudaError_t grow(T** p, int64_t* cap, int64_t n, cudaStream_t s) {
  if (*cap >= n && *p) return cudaSuccess;
  if (*p) cudaFreeAsync(*p, s);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMallocAsync((void**)p, sizeof(T) * (size_t)(n > 0 ? n : 1), s);
  if (e == cudaSuccess) *cap = n;
  return e;
}

int clique_kind(int pattern) {
  switch (pattern) {
    case XGM_PATTERN_TRIANGLE: return 3;
    case XGM_PATTERN_CLIQUE4: return 4;
    case XGM_PATTERN_CLIQUE5: return 5;
    case XGM_PATTERN_CLIQUE6: return 6;
    case XGM_PATTERN_CLIQUE7: return 7;
    default: return 0;
  }
}

}  // namespace

int ensure_clique_grid(xgm_ctx* ctx) {
  if (ctx->clique_grid == 0) {
    int per_sm = 0;
    if (clique_occupancy(&per_sm) != cudaSuccess || per_sm <= 0) per_sm = 1;
    ctx->clique_grid = per_sm * ctx->num_sms;
  }
  return ctx->clique_grid;
}

bool sched_may_bucket(const xgm_sched& sp) {
  if (sp.policy == XGM_SCHED_LEARNED) return true;
  if (sp.policy == XGM_SCHED_FIXED) return sp.variant == XGM_VAR_BUCKET;
  if (sp.policy == XGM_SCHED_TUNED && sp.table) {
    for (int b = 0; b < XGM_TUNE_BUCKETS; ++b)
      if (sp.table->variant[b] == XGM_VAR_BUCKET) return true;
    return false;
  }
  return sp.bucket_max > 0;
}

// Fills tb from the schedule policy for a k-clique style launch (k = 3 for the
// participation and multi-pattern launches).  Builds the graph's bucket index first
// when the policy can pick BUCKET (outside stream capture: callers that capture call
// ensure_bucket_index before they begin).
xgm_status schedule_into(TaskBuf& tb, const DevGraph& g, int k, const xgm_sched& sp,
                         cudaStream_t s, int k_feat, bool hub) {
  bool order = false;
  if (sp.policy == XGM_SCHED_LEARNED) {
    if (!sp.model) {
      set_thread_error("XGM_SCHED_LEARNED needs a trained model (xgm_sched.model)");
      return XGM_ERR_INVALID;
    }
    order = sp.order_by_cost != 0;
    XGM_CUDA_TRY(ensure_bucket_index(g, s));  // the model may pick BUCKET
    XGM_CUDA_TRY(ensure_task_stats(g, s));
    XGM_CUDA_TRY(classify_learned(g, k, *sp.model, tb, order, sp.margin, s, k_feat));
  } else if (sp.policy == XGM_SCHED_TUNED) {
    if (!sp.table) {
      set_thread_error("XGM_SCHED_TUNED needs a variant table (xgm_sched.table)");
      return XGM_ERR_INVALID;
    }
    for (int b = 0; b < XGM_TUNE_BUCKETS; ++b)
      if (sp.table->variant[b] == XGM_VAR_BUCKET) {
        XGM_CUDA_TRY(ensure_bucket_index(g, s));
        break;
      }
    XGM_CUDA_TRY(classify_table(g, k - 1, *sp.table, tb, s));
  } else {
    int gmax = sp.group_max > 0 ? sp.group_max : 0;
    int bmax = sp.bucket_max > 0 ? sp.bucket_max : 0;
    int smax = sp.search_max > 0 ? sp.search_max : 0;
    int wmax = sp.warp_max > 0 ? sp.warp_max : kWarpCap;
    int dmax = sp.wide_max > 0 ? sp.wide_max : (sp.wide_max < 0 ? 0 : kWideCap);
    int cmax = sp.cta_max > 0 ? sp.cta_max : kCtaCap;
    if (sp.policy == XGM_SCHED_FIXED) {
      switch (sp.variant) {
        case XGM_VAR_WARP: wmax = kWarpCap; dmax = kWideCap; cmax = kCtaCap; break;
        case XGM_VAR_SEARCH: smax = kWarpCap; wmax = 0; dmax = kWideCap; cmax = kCtaCap; break;
        case XGM_VAR_WIDE: wmax = 0; dmax = kWideCap; cmax = kCtaCap; break;
        case XGM_VAR_CTA: wmax = 0; dmax = 0; cmax = kCtaCap; break;
        case XGM_VAR_SPLIT: wmax = 0; dmax = 0; cmax = 0; break;
        case XGM_VAR_BUCKET: bmax = kWarpCap; wmax = 0; dmax = kWideCap; cmax = kCtaCap; break;
        case XGM_VAR_GROUP: gmax = kGroupCap; wmax = kWarpCap; dmax = kWideCap; cmax = kCtaCap; break;
        default:
          set_thread_error("unknown variant for XGM_SCHED_FIXED");
          return XGM_ERR_INVALID;
      }
    } else if (sp.policy != XGM_SCHED_HEURISTIC) {
      set_thread_error("unknown schedule policy");
      return XGM_ERR_INVALID;
    }
    if (bmax > 0) XGM_CUDA_TRY(ensure_bucket_index(g, s));
    XGM_CUDA_TRY(classify_heuristic(g, k, wmax, dmax, cmax, tb, s, smax, bmax, gmax));
  }
  // The hub kernel counts up to 5-cliques, by default up to 4-cliques: at 5 the split
  // sub-tasks win (each works on the compressed rows of N+(v0) & N+(v1); R-MAT scale 23:
  // split 6.47 s, whole hubs 7.37 s; 4-cliques 1.08 s -> 0.25 s with whole hubs).
  const int hub_max = (!hub || k > 5 || sp.hub_max < 0 || (sp.hub_max == 0 && k > 4))
                          ? 0
                          : (sp.hub_max == 0 ? kHubCap : sp.hub_max);
  XGM_CUDA_TRY(build_lists(g, tb, order, s, hub_max));
  tb.hash_only = (sp.flags & XGM_SCHED_HASH_ONLY) ? 1 : 0;
  return XGM_OK;
}

namespace {

xgm_status schedule_tasks(xgm_ctx* ctx, const DevGraph& g, int k, const xgm_sched& sp,
                          bool hub = false) {
  return schedule_into(ctx->tb, g, k, sp, ctx->stream, 0, hub);
}

xgm_status ensure_c4(xgm_ctx* ctx, const DevGraph& g) {
  cudaStream_t s = ctx->stream;
  if (ctx->c4_vcap < g.nv || !ctx->wedges) {
    void* ps[] = {ctx->wedges, ctx->c4_flag_large, ctx->c4_flag_small, ctx->c4_pos,
                  ctx->c4_large, ctx->c4_small, ctx->c4_n};
    for (void* p : ps)
      if (p) cudaFreeAsync(p, s);
    const int64_t c = g.nv > 0 ? g.nv : 1;
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->wedges, sizeof(long long) * c, s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_flag_large, c, s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_flag_small, c, s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_pos, sizeof(int64_t) * c, s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_large, sizeof(int32_t) * c, s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_small, sizeof(int32_t) * c, s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_n, sizeof(int64_t) * 2, s));
    ctx->c4_vcap = c;
  }
  const int64_t need = (int64_t)cycle4_grid(ctx->num_sms) * (g.nv > 0 ? g.nv : 1);
  if (ctx->c4_scratch_cap < need) {
    XGM_CUDA_TRY(grow(&ctx->c4_scratch, &ctx->c4_scratch_cap, need, s));
    XGM_CUDA_TRY(cudaMemsetAsync(ctx->c4_scratch, 0, sizeof(uint32_t) * need, s));
  }
  return XGM_OK;
}

}  // namespace

namespace {

// Large 4-cycle tasks with at least 1/16 wedge per id of their range (v2 < v0) and
// numerous wedges are counted a group at a time with L2-resident counters
// (launch_c4_dense_walk); the others stay in the persistent kernel's list, whose large
// tasks pay two DRAM atomics per wedge.  A group's counters are reset by a memset of
// its ranges when they hold fewer than 8 counters per wedge, else by a second walk.
// Reads the large list back, rewrites it without the grouped tasks, and launches them.
constexpr int64_t kC4DenseMinWedges = int64_t(1) << 16;
constexpr int64_t kC4DenseRangePerWedge = 16;

xgm_status cycle4_dense_groups(xgm_ctx* ctx, const DevGraph& g, int* launches) {
  cudaStream_t s = ctx->stream;
  int64_t nls[2] = {0, 0};
  XGM_CUDA_TRY(cudaMemcpyAsync(nls, ctx->c4_n, sizeof(nls), cudaMemcpyDeviceToHost, s));
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  const int64_t nl = nls[0];
  if (nl == 0) return XGM_OK;
  XGM_CUDA_TRY(grow(&ctx->c4_info, &ctx->c4_info_cap, 2 * nl, s));
  XGM_CUDA_TRY(launch_c4_task_info(g.view(), ctx->c4_large, nl, ctx->wedges, ctx->c4_info, s));
  std::vector<int32_t> list(nl);
  std::vector<int64_t> info(2 * nl);
  XGM_CUDA_TRY(cudaMemcpyAsync(list.data(), ctx->c4_large, sizeof(int32_t) * nl,
                               cudaMemcpyDeviceToHost, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(info.data(), ctx->c4_info, sizeof(int64_t) * 2 * nl,
                               cudaMemcpyDeviceToHost, s));
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<int32_t> sparse, dense;
  for (int64_t t = 0; t < nl; ++t) {
    const int64_t w = info[2 * t], v0 = list[t];
    if (w >= kC4DenseMinWedges && kC4DenseRangePerWedge * w >= v0 && v0 <= kC4GroupCounters)
      dense.push_back((int32_t)t);
    else sparse.push_back(list[t]);
  }
  if (dense.empty()) return XGM_OK;
  std::sort(dense.begin(), dense.end(), [&](int32_t a, int32_t b) { return list[a] > list[b]; });
  // groups: consecutive dense tasks whose ranges fit the counter array
  std::vector<int32_t> tv0;
  std::vector<int64_t> ttab;
  struct Group { int64_t t0, m, tab, nseg, ncnt, wedges; };
  // groups: consecutive tasks whose ranges fit the counter array.  Segments (one per
  // task and lower neighbour) are numbered across all groups, so one segment launch and
  // one scan serve every group; a group is a segment range.
  std::vector<Group> groups;
  std::vector<int64_t> tseg{0}, tcnt;
  for (size_t i = 0; i < dense.size();) {
    Group gr{(int64_t)tv0.size(), 0, tseg.back(), 0, 0, 0};
    while (i < dense.size() && (gr.m == 0 || gr.ncnt + list[dense[i]] <= kC4GroupCounters)) {
      const int32_t t = dense[i++];
      tv0.push_back(list[t]);
      tcnt.push_back(gr.ncnt);
      gr.ncnt += list[t];
      gr.wedges += info[2 * t];
      tseg.push_back(tseg.back() + info[2 * t + 1]);
      ++gr.m;
    }
    gr.nseg = tseg.back() - gr.tab;  // tab: first segment of the group
    groups.push_back(gr);
  }
  const int64_t nseg_all = tseg.back();
  const int64_t m_all = (int64_t)tv0.size();
  ttab = tseg;
  ttab.insert(ttab.end(), tcnt.begin(), tcnt.end());
  if (!ctx->c4_counters) {
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_counters, sizeof(uint32_t) * kC4GroupCounters, s));
    XGM_CUDA_TRY(cudaMemsetAsync(ctx->c4_counters, 0, sizeof(uint32_t) * kC4GroupCounters, s));
  }
  if (ctx->c4_seg_cap < nseg_all) {
    void* ps[] = {ctx->c4_seg_base, ctx->c4_seg_pre, ctx->c4_seg_cnt};
    for (void* p : ps)
      if (p) cudaFreeAsync(p, s);
    ctx->c4_seg_cap = 0;
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_seg_base, sizeof(int64_t) * nseg_all, s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_seg_pre, sizeof(int64_t) * (nseg_all + 1), s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_seg_cnt, sizeof(int32_t) * nseg_all, s));
    ctx->c4_seg_cap = nseg_all;
  }
  const int64_t need = std::max<int64_t>(m_all, (int64_t)ttab.size());
  if (ctx->c4_task_cap < need) {
    if (ctx->c4_tv0) cudaFreeAsync(ctx->c4_tv0, s);
    if (ctx->c4_ttab) cudaFreeAsync(ctx->c4_ttab, s);
    ctx->c4_task_cap = 0;
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_tv0, sizeof(int32_t) * need, s));
    XGM_CUDA_TRY(cudaMallocAsync(&ctx->c4_ttab, sizeof(int64_t) * need, s));
    ctx->c4_task_cap = need;
  }
  // the sparse large tasks stay with the persistent kernel; all tables go up at once
  const int64_t ns = (int64_t)sparse.size();
  if (ns) XGM_CUDA_TRY(cudaMemcpyAsync(ctx->c4_large, sparse.data(), sizeof(int32_t) * ns,
                                      cudaMemcpyHostToDevice, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(ctx->c4_n, &ns, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(ctx->c4_tv0, tv0.data(), sizeof(int32_t) * m_all,
                               cudaMemcpyHostToDevice, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(ctx->c4_ttab, ttab.data(), sizeof(int64_t) * ttab.size(),
                               cudaMemcpyHostToDevice, s));
  XGM_CUDA_TRY(cudaStreamSynchronize(s));  // host tables are freed on return
  const GView view = g.view();
  const int grid = 4 * ctx->num_sms;
  XGM_CUDA_TRY(launch_c4_segments(view, ctx->c4_tv0, ctx->c4_ttab, ctx->c4_ttab + m_all + 1,
                                  (int)m_all, nseg_all, ctx->c4_seg_base, ctx->c4_seg_pre,
                                  ctx->c4_seg_cnt, s));
  XGM_CUDA_TRY(scan_excl(ctx->c4_seg_pre, ctx->c4_seg_pre, nseg_all, ctx->c4_seg_pre + nseg_all,
                         s));
  *launches += 2;
  for (const Group& gr : groups) {
    const int64_t e0 = gr.tab;
    XGM_CUDA_TRY(launch_c4_dense_walk(g.col, ctx->c4_seg_pre + e0, ctx->c4_seg_base + e0,
                                      ctx->c4_seg_cnt + e0, gr.nseg, ctx->c4_counters,
                                      &ctx->d_sc->count, grid, s));
    if (gr.ncnt <= 8 * gr.wedges)
      XGM_CUDA_TRY(cudaMemsetAsync(ctx->c4_counters, 0, sizeof(uint32_t) * gr.ncnt, s));
    else
      XGM_CUDA_TRY(launch_c4_dense_walk(g.col, ctx->c4_seg_pre + e0, ctx->c4_seg_base + e0,
                                        ctx->c4_seg_cnt + e0, gr.nseg, ctx->c4_counters, nullptr,
                                        grid, s, true));
    *launches += 2;
  }
  return XGM_OK;
}

}  // namespace

void motif_buffers_free(xgm_ctx* ctx) {
  cudaStream_t s = ctx->stream;
  void* ps[] = {ctx->vpart, ctx->epart, ctx->c4_scratch, ctx->wedges, ctx->c4_flag_large,
                ctx->c4_flag_small, ctx->c4_pos, ctx->c4_large, ctx->c4_small, ctx->c4_n,
                ctx->c4_counters, ctx->c4_info, ctx->c4_seg_base, ctx->c4_seg_pre,
                ctx->c4_seg_cnt, ctx->c4_tv0, ctx->c4_ttab};
  for (void* p : ps)
    if (p) cudaFreeAsync(p, s);
}

xgm_status count_dispatch(xgm_ctx* ctx, const DevGraph& g, int pattern, const xgm_sched& sp,
                          uint64_t* out, xgm_stats& st) {
  cudaStream_t s = ctx->stream;
  XGM_CUDA_TRY(cudaSetDevice(ctx->device));
  XGM_CUDA_TRY(taskbuf_reserve(ctx->tb, g.nv, s));
  XGM_CUDA_TRY(cudaMemsetAsync(ctx->d_sc, 0, sizeof(Scalars), s));
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  const int k = clique_kind(pattern);
  const GView view = g.view();
  int launches = 0;
  if (k) {
    xgm_status r = schedule_tasks(ctx, g, k, sp, true);
    if (r != XGM_OK) return r;
    XGM_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    XGM_CUDA_TRY(launch_clique(k, view, ctx->tb.lists(false), &ctx->d_sc->q, &ctx->d_sc->count,
                               &ctx->d_sc->err, ensure_clique_grid(ctx), s));
    launches = ctx->tb.hub_max > kCtaCap ? 2 : 1;  // + the hub kernel
  } else if (pattern == XGM_PATTERN_DIAMOND || pattern == XGM_PATTERN_TAILED_TRIANGLE) {
    xgm_sched tri = sp;
    if (tri.policy == XGM_SCHED_LEARNED && !tri.model) tri.policy = XGM_SCHED_HEURISTIC;
    xgm_status r = schedule_tasks(ctx, g, 3, tri);
    if (r != XGM_OK) return r;
    XGM_CUDA_TRY(grow(&ctx->vpart, &ctx->vpart_cap, g.nv, s));
    XGM_CUDA_TRY(grow(&ctx->epart, &ctx->epart_cap, g.ne, s));
    XGM_CUDA_TRY(cudaMemsetAsync(ctx->vpart, 0, sizeof(unsigned long long) * (g.nv > 0 ? g.nv : 1), s));
    XGM_CUDA_TRY(cudaMemsetAsync(ctx->epart, 0, sizeof(unsigned) * (g.ne > 0 ? g.ne : 1), s));
    XGM_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    XGM_CUDA_TRY(launch_triangle_participation(view, ctx->tb.lists(false), &ctx->d_sc->q,
                                               ctx->vpart, ctx->epart, &ctx->d_sc->err,
                                               ensure_clique_grid(ctx), s));
    if (pattern == XGM_PATTERN_DIAMOND)
      XGM_CUDA_TRY(launch_diamond_reduce(ctx->epart, g.ne, &ctx->d_sc->count, s));
    else
      XGM_CUDA_TRY(launch_tailed_reduce(ctx->vpart, g.rowptr, g.nv, &ctx->d_sc->count, s));
    launches = 2;
  } else if (pattern == XGM_PATTERN_CYCLE4) {
    xgm_status r = ensure_c4(ctx, g);
    if (r != XGM_OK) return r;
    XGM_CUDA_TRY(launch_wedge_count(view, ctx->wedges, ctx->c4_flag_large, ctx->c4_flag_small, s));
    XGM_CUDA_TRY(scan_excl(ctx->c4_flag_large, ctx->c4_pos, g.nv, ctx->c4_n + 0, s));
    XGM_CUDA_TRY(launch_scatter_flags(ctx->c4_flag_large, ctx->c4_pos, g.nv, ctx->c4_large, s));
    XGM_CUDA_TRY(scan_excl(ctx->c4_flag_small, ctx->c4_pos, g.nv, ctx->c4_n + 1, s));
    XGM_CUDA_TRY(launch_scatter_flags(ctx->c4_flag_small, ctx->c4_pos, g.nv, ctx->c4_small, s));
    XGM_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    launches = 1;
    r = cycle4_dense_groups(ctx, g, &launches);
    if (r != XGM_OK) return r;
    XGM_CUDA_TRY(launch_cycle4(view, ctx->c4_large, ctx->c4_small, ctx->c4_n, ctx->d_sc->c4heads,
                               ctx->c4_scratch, &ctx->d_sc->count, &ctx->d_sc->err,
                               cycle4_grid(ctx->num_sms), s));
  } else {
    set_thread_error("unknown pattern");
    return XGM_ERR_INVALID;
  }
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  if (k || pattern == XGM_PATTERN_DIAMOND || pattern == XGM_PATTERN_TAILED_TRIANGLE)
    XGM_CUDA_TRY(cudaMemcpyAsync(ctx->d_sc->n, ctx->tb.n, sizeof(int64_t) * 8,
                                 cudaMemcpyDeviceToDevice, s));
  xgm_status r = ctx_sync_scalars(ctx);
  if (r != XGM_OK) return r;
  float prep = 0, kern = 0;
  cudaEventElapsedTime(&prep, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&kern, ctx->ev[1], ctx->ev[2]);
  st.prep_ms = prep;
  st.kernel_ms = kern;
  st.device_error = ctx->h_sc->err;
  st.launches = launches;
  st.variant_tasks[XGM_VAR_WARP] = ctx->h_sc->n[2];
  st.variant_tasks[XGM_VAR_CTA] = ctx->h_sc->n[1];
  st.variant_tasks[XGM_VAR_SPLIT] = ctx->h_sc->n[0];
  st.variant_tasks[XGM_VAR_WIDE] = ctx->h_sc->n[4];
  st.variant_tasks[XGM_VAR_SEARCH] = ctx->h_sc->n[5];
  st.variant_tasks[XGM_VAR_BUCKET] = ctx->h_sc->n[6];
  st.variant_tasks[XGM_VAR_GROUP] = ctx->h_sc->n[7];
  st.tasks = ctx->h_sc->n[1] + ctx->h_sc->n[2] + ctx->h_sc->n[3] + ctx->h_sc->n[4] +
             ctx->h_sc->n[5] + ctx->h_sc->n[6] + ctx->h_sc->n[7];
  r = check_device_flag(ctx, ctx->h_sc->err);
  if (r != XGM_OK) return r;
  *out = ctx->h_sc->count;
  return XGM_OK;
}

// Captures the device work of one count (schedule + counting kernels) on the context
// stream into a CUDA graph and counts its kernel nodes.
xgm_status count_kernels(xgm_ctx* ctx, const DevGraph& g, int pattern, const xgm_sched& sp,
                         int* n_kernels) {
  cudaStream_t s = ctx->stream;
  XGM_CUDA_TRY(cudaSetDevice(ctx->device));
  XGM_CUDA_TRY(taskbuf_reserve(ctx->tb, g.nv, s));
  const int k = clique_kind(pattern);
  if (!k) {
    set_thread_error("kernel counting covers the triangle / clique plans");
    return XGM_ERR_UNSUPPORTED;
  }
  ensure_clique_grid(ctx);
  if (sched_may_bucket(sp)) XGM_CUDA_TRY(ensure_bucket_index(g, s));
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  XGM_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  xgm_status r = schedule_tasks(ctx, g, k, sp, true);
  cudaError_t e = cudaSuccess;
  if (r == XGM_OK)
    e = launch_clique(k, g.view(), ctx->tb.lists(false), &ctx->d_sc->q, &ctx->d_sc->count,
                      &ctx->d_sc->err, ensure_clique_grid(ctx), s);
  cudaGraph_t graph = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s, &graph);
  if (r != XGM_OK) {
    if (graph) cudaGraphDestroy(graph);
    return r;
  }
  XGM_CUDA_TRY(e);
  XGM_CUDA_TRY(e2);
  size_t n = 0;
  e = cudaGraphGetNodes(graph, nullptr, &n);
  std::vector<cudaGraphNode_t> nodes(n);
  if (e == cudaSuccess && n) e = cudaGraphGetNodes(graph, nodes.data(), &n);
  int kern = 0;
  for (size_t i = 0; e == cudaSuccess && i < n; ++i) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kern;
  }
  cudaGraphDestroy(graph);
  XGM_CUDA_TRY(e);
  *n_kernels = kern;
  return XGM_OK;
}

xgm_status algo_bytes_dispatch(xgm_ctx* ctx, const DevGraph& g, int pattern, uint64_t* out) {
  cudaStream_t s = ctx->stream;
  XGM_CUDA_TRY(cudaSetDevice(ctx->device));
  XGM_CUDA_TRY(taskbuf_reserve(ctx->tb, g.nv, s));
  XGM_CUDA_TRY(cudaMemsetAsync(ctx->d_sc, 0, sizeof(Scalars), s));
  const GView view = g.view();
  unsigned long long* acc = &ctx->d_sc->count;
  const int k = clique_kind(pattern);
  if (k > 5) {
    set_thread_error("algorithmic bytes cover the triangle, 4/5-clique and edge-induced "
                     "motif plans");
    return XGM_ERR_UNSUPPORTED;
  }
  xgm_sched heur;
  std::memset(&heur, 0, sizeof(heur));
  if (k) {
    XGM_CUDA_TRY(launch_bytes_basic(view, 0, acc, s));
    // W terms: 4 * sum over kk-cliques of d+(top member), kk = 3 .. k-1
    for (int kk = 3; kk <= k - 1; ++kk) {
      xgm_status r = schedule_tasks(ctx, g, kk, heur);
      if (r != XGM_OK) return r;
      XGM_CUDA_TRY(cudaMemsetAsync(&ctx->d_sc->q, 0, sizeof(QueueHeads), s));
      XGM_CUDA_TRY(launch_clique_weighted(kk, view, ctx->tb.lists(false), &ctx->d_sc->q,
                                          &ctx->d_sc->aux, &ctx->d_sc->err,
                                          ensure_clique_grid(ctx), s));
    }
    xgm_status r = ctx_sync_scalars(ctx);
    if (r != XGM_OK) return r;
    *out = ctx->h_sc->count + 4ull * ctx->h_sc->aux;
    return check_device_flag(ctx, ctx->h_sc->err);
  } else if (pattern == XGM_PATTERN_DIAMOND) {
    XGM_CUDA_TRY(launch_bytes_basic(view, 1, acc, s));
  } else if (pattern == XGM_PATTERN_TAILED_TRIANGLE) {
    XGM_CUDA_TRY(launch_bytes_basic(view, 2, acc, s));
  } else if (pattern == XGM_PATTERN_CYCLE4) {
    xgm_status r = ensure_c4(ctx, g);
    if (r != XGM_OK) return r;
    XGM_CUDA_TRY(launch_bytes_basic(view, 3, acc, s));
    XGM_CUDA_TRY(launch_wedge_count(view, ctx->wedges, ctx->c4_flag_large, ctx->c4_flag_small, s));
    XGM_CUDA_TRY(launch_sum_ll(ctx->wedges, g.nv, &ctx->d_sc->aux, s));
    xgm_status r2 = ctx_sync_scalars(ctx);
    if (r2 != XGM_OK) return r2;
    *out = ctx->h_sc->count + 4ull * ctx->h_sc->aux;
    return check_device_flag(ctx, ctx->h_sc->err);
  } else {
    return XGM_ERR_INVALID;
  }
  xgm_status r = ctx_sync_scalars(ctx);
  if (r != XGM_OK) return r;
  *out = ctx->h_sc->count;
  return check_device_flag(ctx, ctx->h_sc->err);
}

namespace {

// The sums of launch_motif_terms, after one triangle-participation pass when `part`.
xgm_status motif_terms(xgm_ctx* ctx, const DevGraph& g, const xgm_sched& sp, bool part,
                       uint64_t terms[6], xgm_stats& st) {
  cudaStream_t s = ctx->stream;
  XGM_CUDA_TRY(cudaSetDevice(ctx->device));
  XGM_CUDA_TRY(taskbuf_reserve(ctx->tb, g.nv, s));
  XGM_CUDA_TRY(cudaMemsetAsync(ctx->d_sc, 0, sizeof(Scalars), s));
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  const GView view = g.view();
  if (part) {
    xgm_sched tri = sp;
    if (tri.policy == XGM_SCHED_LEARNED && !tri.model) tri.policy = XGM_SCHED_HEURISTIC;
    xgm_status r = schedule_tasks(ctx, g, 3, tri);
    if (r != XGM_OK) return r;
    XGM_CUDA_TRY(grow(&ctx->vpart, &ctx->vpart_cap, g.nv, s));
    XGM_CUDA_TRY(grow(&ctx->epart, &ctx->epart_cap, g.ne, s));
    XGM_CUDA_TRY(cudaMemsetAsync(ctx->vpart, 0, sizeof(unsigned long long) * (g.nv > 0 ? g.nv : 1), s));
    XGM_CUDA_TRY(cudaMemsetAsync(ctx->epart, 0, sizeof(unsigned) * (g.ne > 0 ? g.ne : 1), s));
    XGM_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    XGM_CUDA_TRY(launch_triangle_participation(view, ctx->tb.lists(false), &ctx->d_sc->q,
                                               ctx->vpart, ctx->epart, &ctx->d_sc->err,
                                               ensure_clique_grid(ctx), s));
  } else {
    XGM_CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  }
  XGM_CUDA_TRY(launch_motif_terms(view, part ? ctx->vpart : nullptr, part ? ctx->epart : nullptr,
                                  ctx->d_sc->terms, s));
  XGM_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  if (part)
    XGM_CUDA_TRY(cudaMemcpyAsync(ctx->d_sc->n, ctx->tb.n, sizeof(int64_t) * 8,
                                 cudaMemcpyDeviceToDevice, s));
  xgm_status r = ctx_sync_scalars(ctx);
  if (r != XGM_OK) return r;
  float prep = 0, kern = 0;
  cudaEventElapsedTime(&prep, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&kern, ctx->ev[1], ctx->ev[2]);
  std::memset(&st, 0, sizeof(st));
  st.prep_ms = prep;
  st.kernel_ms = kern;
  st.device_error = ctx->h_sc->err;
  st.launches = part ? 2 : 1;
  if (part) {
    st.variant_tasks[XGM_VAR_WARP] = ctx->h_sc->n[2];
    st.variant_tasks[XGM_VAR_CTA] = ctx->h_sc->n[1];
    st.variant_tasks[XGM_VAR_SPLIT] = ctx->h_sc->n[0];
    st.variant_tasks[XGM_VAR_WIDE] = ctx->h_sc->n[4];
    st.variant_tasks[XGM_VAR_SEARCH] = ctx->h_sc->n[5];
    st.variant_tasks[XGM_VAR_BUCKET] = ctx->h_sc->n[6];
    st.variant_tasks[XGM_VAR_GROUP] = ctx->h_sc->n[7];
    st.tasks = ctx->h_sc->n[1] + ctx->h_sc->n[2] + ctx->h_sc->n[3] + ctx->h_sc->n[4] +
               ctx->h_sc->n[5] + ctx->h_sc->n[6] + ctx->h_sc->n[7];
  }
  r = check_device_flag(ctx, ctx->h_sc->err);
  if (r != XGM_OK) return r;
  for (int i = 0; i < 6; ++i) terms[i] = ctx->h_sc->terms[i];
  return XGM_OK;
}

void add_stats(xgm_stats& acc, const xgm_stats& x) {
  acc.kernel_ms += x.kernel_ms;
  acc.prep_ms += x.prep_ms;
  acc.tasks += x.tasks;
  for (int i = 0; i < XGM_NUM_VARIANTS; ++i) acc.variant_tasks[i] += x.variant_tasks[i];
  acc.algo_bytes += x.algo_bytes;
  acc.device_error |= x.device_error;
  acc.launches += x.launches;
}

// The pieces of the 4-vertex identities (all wrapping uint64).
struct Motif4Parts {
  uint64_t k4 = 0, c4e = 0;
  uint64_t t[6] = {0, 0, 0, 0, 0, 0};  // motif_terms with participation
};

xgm_status motif4_parts(xgm_ctx* ctx, const DevGraph& g, const xgm_sched& sp, bool need_c4,
                        Motif4Parts& m, xgm_stats& st) {
  xgm_stats x;
  xgm_status r = motif_terms(ctx, g, sp, true, m.t, x);
  if (r != XGM_OK) return r;
  add_stats(st, x);
  std::memset(&x, 0, sizeof(x));
  r = count_dispatch(ctx, g, XGM_PATTERN_CLIQUE4, sp, &m.k4, x);
  if (r != XGM_OK) return r;
  add_stats(st, x);
  if (need_c4) {
    std::memset(&x, 0, sizeof(x));
    r = count_dispatch(ctx, g, XGM_PATTERN_CYCLE4, sp, &m.c4e, x);
    if (r != XGM_OK) return r;
    add_stats(st, x);
  }
  return XGM_OK;
}

// Vertex-induced 4-vertex motifs from the edge-induced counts.  Every edge-induced
// embedding sits in exactly one induced connected 4-vertex subgraph; per 4-set:
//                3-star 4-path tailed 4-cycle diamond K4
//   3-stars        1      0      1      0       2     4      (sum_v C(d_v, 3))
//   4-paths        0      1      2      4       6    12      (3-walks - 3 x triangles)
//   tailed         .      .      1      0       4    12
//   4-cycles       .      .      0      1       1     3
//   diamonds       .      .      0      0       1     6
// The triangular system is solved from the bottom up.  The reference's formula motif
// counter (codes/GraphMiner/src/motif/omp_formula.cc:38-48 with
// cpu_kernels/automine_formula.h:20-57) derives the same six numbers from
// per-edge local counts plus enumerated 4-cycles and 4-cliques; its output order is
// [3-star, 4-path, tailed triangle, 4-cycle, diamond, 4-clique].
void motif4_solve(const Motif4Parts& m, uint64_t out[6]) {
  const uint64_t k4 = m.k4, dia_e = m.t[4], tail_e = m.t[3];
  const uint64_t star_e = m.t[1], path_e = m.t[2] - m.t[5];
  const uint64_t dia = dia_e - 6 * k4;
  const uint64_t c4 = m.c4e + 3 * k4 - dia_e;
  const uint64_t tail = tail_e - 4 * dia - 12 * k4;
  out[0] = star_e - tail - 2 * dia - 4 * k4;
  out[1] = path_e - 2 * tail - 4 * c4 - 6 * dia - 12 * k4;
  out[2] = tail;
  out[3] = c4;
  out[4] = dia;
  out[5] = k4;
}

}  // namespace

// Reference interface: MotifSolver(Graph&, int k, std::vector<uint64_t>& total, ...)
// (codes/GraphMiner/src/motif/omp_formula.cc:8, main.cc:8-31): k = 3 gives
// [wedges, triangles], k = 4 the six counts of motif4_solve, all vertex-induced.
xgm_status count_motifs(xgm_ctx* ctx, const DevGraph& g, int k, const xgm_sched& sp,
                        uint64_t* out, xgm_stats& st) {
  std::memset(&st, 0, sizeof(st));
  if (k == 3) {
    uint64_t t[6], tri = 0;
    xgm_stats x;
    xgm_status r = motif_terms(ctx, g, sp, false, t, x);
    if (r != XGM_OK) return r;
    add_stats(st, x);
    std::memset(&x, 0, sizeof(x));
    r = count_dispatch(ctx, g, XGM_PATTERN_TRIANGLE, sp, &tri, x);
    if (r != XGM_OK) return r;
    add_stats(st, x);
    out[0] = t[0] - 3 * tri;
    out[1] = tri;
    return XGM_OK;
  }
  if (k != 4) {
    set_thread_error("motif counting covers k = 3 and k = 4");
    return XGM_ERR_UNSUPPORTED;
  }
  Motif4Parts m;
  xgm_status r = motif4_parts(ctx, g, sp, true, m, st);
  if (r != XGM_OK) return r;
  motif4_solve(m, out);
  return XGM_OK;
}

// One plan: the clique and edge-induced motif kernels directly; wedges, 3-stars,
// 4-paths and every vertex-induced motif through the motif sums and identities.
xgm_status count_plan(xgm_ctx* ctx, const DevGraph& g, int pattern, int induced,
                      const xgm_sched& sp, uint64_t* out, xgm_stats& st) {
  const bool clique = pattern == XGM_PATTERN_TRIANGLE || pattern == XGM_PATTERN_CLIQUE4 ||
                      pattern == XGM_PATTERN_CLIQUE5 || pattern == XGM_PATTERN_CLIQUE6 ||
                      pattern == XGM_PATTERN_CLIQUE7;
  const bool kernel = pattern == XGM_PATTERN_DIAMOND || pattern == XGM_PATTERN_CYCLE4 ||
                      pattern == XGM_PATTERN_TAILED_TRIANGLE;
  if (clique || (kernel && !induced)) return count_dispatch(ctx, g, pattern, sp, out, st);
  std::memset(&st, 0, sizeof(st));
  if (pattern == XGM_PATTERN_WEDGE) {
    if (induced) {
      uint64_t m3[2];
      xgm_status r = count_motifs(ctx, g, 3, sp, m3, st);
      if (r == XGM_OK) *out = m3[0];
      return r;
    }
    uint64_t t[6];
    xgm_status r = motif_terms(ctx, g, sp, false, t, st);
    if (r == XGM_OK) *out = t[0];
    return r;
  }
  if (pattern == XGM_PATTERN_STAR3 && !induced) {
    uint64_t t[6];
    xgm_status r = motif_terms(ctx, g, sp, false, t, st);
    if (r == XGM_OK) *out = t[1];
    return r;
  }
  if (pattern == XGM_PATTERN_PATH4 && !induced) {
    uint64_t t[6];
    xgm_status r = motif_terms(ctx, g, sp, true, t, st);
    if (r == XGM_OK) *out = t[2] - t[5];
    return r;
  }
  // vertex-induced 4-vertex motifs; the 4-cycle kernel only where the identity needs it
  const bool need_c4 = pattern == XGM_PATTERN_CYCLE4 || pattern == XGM_PATTERN_PATH4;
  Motif4Parts m;
  xgm_status r = motif4_parts(ctx, g, sp, need_c4, m, st);
  if (r != XGM_OK) return r;
  uint64_t v[6];
  motif4_solve(m, v);
  switch (pattern) {
    case XGM_PATTERN_STAR3: *out = v[0]; break;
    case XGM_PATTERN_PATH4: *out = v[1]; break;
    case XGM_PATTERN_TAILED_TRIANGLE: *out = v[2]; break;
    case XGM_PATTERN_CYCLE4: *out = v[3]; break;
    case XGM_PATTERN_DIAMOND: *out = v[4]; break;
    default: set_thread_error("unknown pattern"); return XGM_ERR_INVALID;
  }
  return XGM_OK;
}

// Pattern matching of a small adjacency matrix against the builtins (edge-induced).
int match_pattern(const xgm_plan_desc* d) {
  const int n = d->num_vertices;
  if (n < 3 || n > 8) return -1;
  int deg[8] = {0}, m = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const bool a = d->adj[i][j] != 0, b = d->adj[j][i] != 0;
      if (a != b || (i == j && a)) return -1;
      if (a && i < j) ++m, ++deg[i], ++deg[j];
    }
  int sorted[8];
  for (int i = 0; i < n; ++i) sorted[i] = deg[i];
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j)
      if (sorted[j] < sorted[i]) { int t = sorted[i]; sorted[i] = sorted[j]; sorted[j] = t; }
  if (n == 3 && m == 3) return XGM_PATTERN_TRIANGLE;
  if (n == 4 && m == 6) return XGM_PATTERN_CLIQUE4;
  if (n == 5 && m == 10) return XGM_PATTERN_CLIQUE5;
  if (n == 6 && m == 15) return XGM_PATTERN_CLIQUE6;
  if (n == 7 && m == 21) return XGM_PATTERN_CLIQUE7;
  if (n == 4 && m == 5) return XGM_PATTERN_DIAMOND;  // K4 minus one edge
  if (n == 4 && m == 4 && sorted[0] == 2 && sorted[3] == 2) return XGM_PATTERN_CYCLE4;
  if (n == 4 && m == 4 && sorted[0] == 1 && sorted[1] == 2 && sorted[2] == 2 && sorted[3] == 3)
    return XGM_PATTERN_TAILED_TRIANGLE;
  if (n == 3 && m == 2 && sorted[0] == 1) return XGM_PATTERN_WEDGE;
  if (n == 4 && m == 3 && sorted[0] == 1 && sorted[2] == 1 && sorted[3] == 3) return XGM_PATTERN_STAR3;
  if (n == 4 && m == 3 && sorted[0] == 1 && sorted[1] == 1 && sorted[2] == 2 && sorted[3] == 2)
    return XGM_PATTERN_PATH4;
  return 0;
}

int pattern_from_name(const char* name, int* induced, uint64_t* scale) {
  const std::string s(name);
  if (induced) *induced = 0;
  if (scale) *scale = 1;
  if (s == "triangle" || s == "3-clique" || s == "clique3" || s == "tc" || s == "3-triangle")
    return XGM_PATTERN_TRIANGLE;
  if (s == "4-clique" || s == "clique4" || s == "k4") return XGM_PATTERN_CLIQUE4;
  if (s == "5-clique" || s == "clique5" || s == "k5") return XGM_PATTERN_CLIQUE5;
  if (s == "6-clique" || s == "clique6" || s == "k6") return XGM_PATTERN_CLIQUE6;
  if (s == "7-clique" || s == "clique7" || s == "k7") return XGM_PATTERN_CLIQUE7;
  if (s == "diamond" || s == "4-diamond") return XGM_PATTERN_DIAMOND;
  if (s == "rectangle" || s == "4-cycle" || s == "cycle4") return XGM_PATTERN_CYCLE4;
  if (s == "tailedtriangle" || s == "tailed-triangle" || s == "tailed_triangle" ||
      s == "4-tailed-triangle")
    return XGM_PATTERN_TAILED_TRIANGLE;
  if (s == "wedge" || s == "3-path") return XGM_PATTERN_WEDGE;
  if (s == "4-star" || s == "3-star") return XGM_PATTERN_STAR3;
  if (s == "4-path") return XGM_PATTERN_PATH4;
  // GLUMIN pattern ids (G2Miner/main.cc:13-60): vertex-induced.  P1 counts each star
  // once (GM_kernels/P1-GM.yml.cuh: leaves ordered v3 < v2 < v1); P2 walks every
  // directed edge as the diamond's shared edge (init_edgelist without symmetry
  // breaking, gpu_GM_LUT.cu:89 / common/graph.cc:296-330; P2-GM.yml.cuh), so each diamond
  // counts twice; P3 counts each tailed triangle once (v2 < v1 around the anchor v0).
  int p = 0;
  uint64_t k = 1;
  if (s == "P1") p = XGM_PATTERN_STAR3;
  else if (s == "P2") p = XGM_PATTERN_DIAMOND, k = 2;
  else if (s == "P3") p = XGM_PATTERN_TAILED_TRIANGLE;
  else if (s == "P4") p = XGM_PATTERN_CLIQUE4;
  else if (s == "P5") p = XGM_PATTERN_CLIQUE5;
  else if (s == "P23") p = XGM_PATTERN_CLIQUE6;
  else if (s == "P24") p = XGM_PATTERN_CLIQUE7;
  if (p) {
    if (induced) *induced = 1;
    if (scale) *scale = k;
  }
  return p;
}

}  // namespace xgm

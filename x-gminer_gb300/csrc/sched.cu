// Task generation for the clique kernels: variant per vertex -> ordered task lists.
//
// The reference sizes one grid per launch and grid-strides over the COO edge list
// (clique4_warp_edge.cuh:14) or splits vertices by degree thresholds into warp / block
// / per-hub launches (xgminer/src/glumin/glumin_GM_solver.cu:324-346, 490-503).  Here
// one persistent launch consumes seven device-built queues (clique.cu), and the
// schedule is only the content and order of those queues; it never changes a count.
#include "prim.cuh"
#include "sched.cuh"

namespace xgm {

namespace {

constexpr int kThreads = 256;
constexpr int kBins = 64;  // cost bins of the learned ordering

inline unsigned grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  if (b > (int64_t(1) << 20)) b = int64_t(1) << 20;
  return (unsigned)b;
}

#define GRID_STRIDE(i, n)                                                   \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); \
       i += (int64_t)gridDim.x * blockDim.x)

__global__ void k_classify_heur(const longlong2* dptr, int64_t nv, int kmin, int group_max,
                                int bucket_max, int search_max, int warp_max, int wide_max,
                                int cta_max, uint8_t* var) {
  GRID_STRIDE(r, nv) {
    const longlong2 d = dptr[r];
    const int64_t s = d.y - d.x;
    uint8_t v;
    if (s < kmin) v = VAR_SKIP;
    else if (s <= group_max) v = VAR_GROUP;
    else if (s <= bucket_max) v = VAR_BUCKET;
    else if (s <= search_max) v = VAR_SEARCH;
    else if (s <= warp_max) v = VAR_WARP;
    else if (s <= wide_max) v = VAR_WIDE;
    else if (s <= cta_max) v = VAR_CTA;
    else v = VAR_SPLIT;
    var[r] = v;
  }
}

// Bucket b of out-degree s: 0 for s == 0, else floor(log2(s)) + 1, capped.
__device__ __forceinline__ int degree_bucket(int64_t s) {
  if (s <= 0) return 0;
  const int b = 64 - __clzll((unsigned long long)s);
  return b < XGM_TUNE_BUCKETS ? b : XGM_TUNE_BUCKETS - 1;
}

__global__ void k_classify_table(const longlong2* dptr, int64_t nv, int kmin, xgm_tune_table tab,
                                 uint8_t* var) {
  GRID_STRIDE(r, nv) {
    const longlong2 d = dptr[r];
    const int64_t s = d.y - d.x;
    uint8_t v = VAR_SKIP;
    if (s >= kmin) {
      v = tab.variant[degree_bucket(s)];
      if (v > VAR_GROUP) v = VAR_SPLIT;
      if (v == VAR_GROUP && s > kGroupCap) v = VAR_WARP;
      if ((v == VAR_SEARCH || v == VAR_BUCKET) && s > kWarpCap) v = VAR_WIDE;
      if (v == VAR_WARP && s > kWarpCap) v = VAR_WIDE;
      if (v == VAR_WIDE && s > kWideCap) v = VAR_CTA;
      if (v == VAR_CTA && s > kCtaCap) v = VAR_SPLIT;
    }
    var[r] = v;
  }
}

__global__ void k_hub_tail(const int64_t* n, int64_t* split_off) {
  split_off[n[3]] = n[0];
}

// ---- learned ordering: counting sort of each list by descending predicted cost
__device__ __forceinline__ int cost_bin(float c) {
  // predicted log2-cycles in [0, 32) -> 64 bins, bin 0 = most expensive
  int b = (int)((32.0f - c) * 2.0f);
  return b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
}

__global__ void k_bin_hist(const uint8_t* var, const float* cost, int64_t nv,
                           unsigned long long* hist /*[kNumVar][kBins]*/) {
  __shared__ unsigned int h[kNumVar * kBins];
  for (int i = threadIdx.x; i < kNumVar * kBins; i += blockDim.x) h[i] = 0;
  __syncthreads();
  GRID_STRIDE(r, nv) {
    const uint8_t v = var[r];
    if (v < kNumVar) atomicAdd(&h[v * kBins + cost_bin(cost[r])], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kNumVar * kBins; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], (unsigned long long)h[i]);
}

// One block: exclusive scan of each list's bins into cursors; list sizes into n[].
__global__ void k_bin_scan(unsigned long long* hist, int64_t* n) {
  if (threadIdx.x < kNumVar) {
    const int v = threadIdx.x;
    unsigned long long run = 0;
    for (int b = 0; b < kBins; ++b) {
      unsigned long long c = hist[v * kBins + b];
      hist[v * kBins + b] = run;
      run += c;
    }
    // var code -> n[] slot: WARP 2, CTA 1, SPLIT 3, WIDE 4, SEARCH 5, BUCKET 6, GROUP 7
    n[v == VAR_WARP ? 2 : v == VAR_CTA ? 1 : v == VAR_SPLIT ? 3 : v == VAR_WIDE ? 4
      : v == VAR_SEARCH ? 5 : v == VAR_BUCKET ? 6 : 7] = (int64_t)run;
  }
}

__global__ void k_bin_scatter(const uint8_t* var, const float* cost, int64_t nv,
                              unsigned long long* cursor, int32_t* warp_l, int32_t* cta_l,
                              int32_t* hub_l, int32_t* wide_l, int32_t* search_l,
                              int32_t* bucket_l, int32_t* group_l) {
  GRID_STRIDE(r, nv) {
    const uint8_t v = var[r];
    if (v < kNumVar) {
      const unsigned long long p = atomicAdd(&cursor[v * kBins + cost_bin(cost[r])], 1ull);
      int32_t* out = v == VAR_WARP    ? warp_l
                     : v == VAR_CTA   ? cta_l
                     : v == VAR_SPLIT ? hub_l
                     : v == VAR_WIDE  ? wide_l
                     : v == VAR_SEARCH ? search_l
                     : v == VAR_BUCKET ? bucket_l
                                      : group_l;
      out[p] = (int32_t)r;
    }
  }
}

// ---- natural-order lists in one pass: per-tile code counts, one scan, stable scatter
constexpr int kCompactThreads = 256;
constexpr int kCompactItems = 16;
constexpr int kCompactTile = kCompactThreads * kCompactItems;

__global__ void __launch_bounds__(kCompactThreads) k_compact_count(const uint8_t* var, int64_t nv,
                                                                   int64_t tiles, int64_t* cnt) {
  __shared__ int c_sm[kNumVar];
  if (threadIdx.x < kNumVar) c_sm[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kCompactTile;
#pragma unroll 4
  for (int j = 0; j < kCompactItems; ++j) {
    const int64_t i = base + j * kCompactThreads + threadIdx.x;
    const int v = i < nv ? var[i] : kNumVar;
    const unsigned peers = __match_any_sync(0xffffffffu, v);
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    if (v < kNumVar && (peers & lt) == 0u) atomicAdd(&c_sm[v], __popc(peers));
  }
  __syncthreads();
  if (threadIdx.x < kNumVar) cnt[threadIdx.x * tiles + blockIdx.x] = c_sm[threadIdx.x];
}

struct ListOuts {
  int32_t* p[kNumVar];  // output list per variant code
};

// cnt holds the exclusive scan of [code][tile] counts (cnt[kNumVar * tiles] = total):
// an element's slot in its code's list = cnt[c][tile] - cnt[c][0] + rank in the tile.
__global__ void __launch_bounds__(kCompactThreads) k_compact_scatter(
    const uint8_t* var, int64_t nv, int64_t tiles, const int64_t* cnt, ListOuts outs) {
  __shared__ int64_t run[kNumVar];
  __shared__ int wcnt[kCompactThreads / 32][kNumVar];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < kNumVar)
    run[threadIdx.x] = cnt[threadIdx.x * tiles + blockIdx.x] - cnt[threadIdx.x * tiles];
  const int64_t base = (int64_t)blockIdx.x * kCompactTile;
  for (int j = 0; j < kCompactItems; ++j) {
    if (lane < kNumVar) wcnt[warp][lane] = 0;
    __syncthreads();
    const int64_t i = base + j * kCompactThreads + threadIdx.x;
    const int v = i < nv ? var[i] : kNumVar;
    const unsigned peers = __match_any_sync(0xffffffffu, v);
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    const int rank = __popc(peers & lt);
    if (v < kNumVar && rank == 0) wcnt[warp][v] = __popc(peers);
    __syncthreads();
    if (v < kNumVar) {
      int64_t pos = run[v] + rank;
      for (int w = 0; w < warp; ++w) pos += wcnt[w][v];
      outs.p[v][pos] = (int32_t)i;
    }
    __syncthreads();
    if (threadIdx.x < kNumVar) {
      int t = 0;
      for (int w = 0; w < kCompactThreads / 32; ++w) t += wcnt[w][threadIdx.x];
      run[threadIdx.x] += t;
    }
    __syncthreads();
  }
}

// List sizes into n[] (code -> slot as in k_bin_scan).
__global__ void k_compact_sizes(const int64_t* cnt, int64_t tiles, int64_t* n) {
  if (threadIdx.x < kNumVar) {
    const int v = threadIdx.x;
    const int64_t sz = cnt[(v + 1) * tiles] - cnt[v * tiles];
    n[v == VAR_WARP ? 2 : v == VAR_CTA ? 1 : v == VAR_SPLIT ? 3 : v == VAR_WIDE ? 4
      : v == VAR_SEARCH ? 5 : v == VAR_BUCKET ? 6 : 7] = sz;
  }
}

// Hubs the hub kernel could run whole (kCtaCap < out-degree <= hub_max) into n[8].
__global__ void k_hub_eligible(const int32_t* hubs, int64_t* n, const longlong2* dptr,
                               int hub_max) {
  const int64_t nh = n[3];
  unsigned long long c = 0;
  GRID_STRIDE(h, nh) {
    const longlong2 d = dptr[hubs[h]];
    const int64_t s = d.y - d.x;
    c += (s > kCtaCap && s <= hub_max) ? 1ull : 0ull;
  }
  if (c) atomicAdd((unsigned long long*)&n[8], c);
}

// Hub sub-task offsets in hub-list order.  Eligible hubs run whole (no sub-tasks) when
// there are at least kHubMinWhole of them: the hub kernel runs after the main launch, so
// a handful of whole hubs would be a tail of one CTA each (R-MAT scale 22: 4 hubs of
// ~1030, +0.7 ms whole), while their sub-tasks run first inside the main launch.
constexpr int64_t kHubMinWhole = 32;
__global__ void k_hub_weights_list(const int32_t* hubs, const int64_t* n, const longlong2* dptr,
                                   int hub_max, int64_t* w) {
  const int64_t nh = n[3];
  const bool whole = n[8] >= kHubMinWhole;
  GRID_STRIDE(h, nh) {
    const longlong2 d = dptr[hubs[h]];
    const int64_t s = d.y - d.x;
    w[h] = (whole && s > kCtaCap && s <= hub_max) ? 0 : s;
  }
}

template <class T>
cudaError_t dalloc(T** p, int64_t n, cudaStream_t s) {
  return cudaMallocAsync((void**)p, sizeof(T) * (size_t)(n > 0 ? n : 1), s);
}

#define TRY(x)                        \
  do {                                \
    cudaError_t _e = (x);             \
    if (_e != cudaSuccess) return _e; \
  } while (0)

}  // namespace

TaskLists TaskBuf::lists(bool with_log) const {
  TaskLists t;
  t.cta = cta;
  t.warp = warp;
  t.wide = wide;
  t.search = search;
  t.bucket = bucket;
  t.group = group;
  t.split_v = split_v;
  t.split_off = split_off;
  t.n = n;
  t.hub_max = hub_max;
  t.hash_only = hash_only;
  if (with_log && log) {
    t.log_cta = log;
    t.log_warp = log + cap_v;
    t.log_wide = log + 2 * cap_v;
    t.log_search = log + 3 * cap_v;
    t.log_bucket = log + 4 * cap_v;
    t.log_group = log + 5 * cap_v;
    t.log_split = log + 6 * cap_v;
  }
  return t;
}

cudaError_t taskbuf_reserve(TaskBuf& tb, int64_t nv, cudaStream_t s) {
  if (tb.cap_v >= nv && tb.cta) return cudaSuccess;
  taskbuf_free(tb, s);
  const int64_t c = nv > 0 ? nv : 1;
  TRY(dalloc(&tb.cta, c, s));
  TRY(dalloc(&tb.warp, c, s));
  TRY(dalloc(&tb.wide, c, s));
  TRY(dalloc(&tb.search, c, s));
  TRY(dalloc(&tb.bucket, c, s));
  TRY(dalloc(&tb.group, c, s));
  TRY(dalloc(&tb.split_v, c, s));
  TRY(dalloc(&tb.split_off, c + 1, s));
  TRY(dalloc(&tb.n, 9, s));
  TRY(dalloc(&tb.var, c, s));
  TRY(dalloc(&tb.w, c, s));
  TRY(dalloc(&tb.cost, c, s));
  tb.cap_v = c;
  return cudaSuccess;
}

void taskbuf_free(TaskBuf& tb, cudaStream_t s) {
  void* ps[] = {tb.cta, tb.warp, tb.wide, tb.search, tb.bucket, tb.group, tb.split_v, tb.split_off, tb.n, tb.var,
                tb.w, tb.cost, tb.log};
  for (void* p : ps)
    if (p) cudaFreeAsync(p, s);
  tb = TaskBuf{};
}

cudaError_t classify_heuristic(const DevGraph& g, int k, int warp_max, int wide_max, int cta_max,
                               TaskBuf& tb, cudaStream_t s, int search_max, int bucket_max,
                               int group_max) {
  if (search_max > kWarpCap) search_max = kWarpCap;
  if (bucket_max > kWarpCap) bucket_max = kWarpCap;
  if (group_max > kGroupCap) group_max = kGroupCap;
  if (warp_max > kWarpCap) warp_max = kWarpCap;
  if (wide_max > kWideCap) wide_max = kWideCap;
  if (k < 2) k = 2;
  if (cta_max > kCtaCap) cta_max = kCtaCap;
  if (g.nv == 0) return cudaSuccess;
  k_classify_heur<<<grid_for(g.nv), kThreads, 0, s>>>(g.dptr, g.nv, k - 1, group_max, bucket_max,
                                                      search_max, warp_max, wide_max, cta_max,
                                                      tb.var);
  return cudaGetLastError();
}

cudaError_t classify_table(const DevGraph& g, int kmin, const xgm_tune_table& tab, TaskBuf& tb,
                           cudaStream_t s) {
  if (g.nv == 0) return cudaSuccess;
  k_classify_table<<<grid_for(g.nv), kThreads, 0, s>>>(g.dptr, g.nv, kmin, tab, tb.var);
  return cudaGetLastError();
}

cudaError_t build_lists(const DevGraph& g, TaskBuf& tb, bool order, cudaStream_t s,
                        int hub_max) {
  const int64_t nv = g.nv;
  tb.hub_max = hub_max > kHubCap ? kHubCap : (hub_max > kCtaCap ? hub_max : 0);
  tb.hash_only = 0;
  hub_max = tb.hub_max;
  TRY(cudaMemsetAsync(tb.n, 0, 9 * sizeof(int64_t), s));
  if (nv == 0) return cudaMemsetAsync(tb.split_off, 0, sizeof(int64_t), s);
  if (!order) {
    const int64_t tiles = (nv + kCompactTile - 1) / kCompactTile;
    int64_t* cnt = nullptr;
    TRY(dalloc(&cnt, kNumVar * tiles + 1, s));
    ListOuts outs;
    outs.p[VAR_WARP] = tb.warp;
    outs.p[VAR_CTA] = tb.cta;
    outs.p[VAR_SPLIT] = tb.split_v;
    outs.p[VAR_WIDE] = tb.wide;
    outs.p[VAR_SEARCH] = tb.search;
    outs.p[VAR_BUCKET] = tb.bucket;
    outs.p[VAR_GROUP] = tb.group;
    k_compact_count<<<(unsigned)tiles, kCompactThreads, 0, s>>>(tb.var, nv, tiles, cnt);
    TRY(scan_excl(cnt, cnt, kNumVar * tiles, cnt + kNumVar * tiles, s));
    k_compact_scatter<<<(unsigned)tiles, kCompactThreads, 0, s>>>(tb.var, nv, tiles, cnt, outs);
    k_compact_sizes<<<1, 32, 0, s>>>(cnt, tiles, tb.n);
    cudaFreeAsync(cnt, s);
    // hub offsets in hub-list order (at most nv hubs; the rest of w stays zero)
    TRY(cudaMemsetAsync(tb.w, 0, sizeof(int64_t) * nv, s));
    if (hub_max > 0)
      k_hub_eligible<<<grid_for(nv), kThreads, 0, s>>>(tb.split_v, tb.n, g.dptr, hub_max);
    k_hub_weights_list<<<grid_for(nv), kThreads, 0, s>>>(tb.split_v, tb.n, g.dptr, hub_max,
                                                         tb.w);
    TRY(cudaGetLastError());
    TRY(scan_excl(tb.w, tb.split_off, nv, tb.n + 0, s));
  } else {
    unsigned long long* hist = nullptr;
    TRY(dalloc(&hist, kNumVar * kBins, s));
    TRY(cudaMemsetAsync(hist, 0, kNumVar * kBins * sizeof(unsigned long long), s));
    k_bin_hist<<<grid_for(nv), kThreads, 0, s>>>(tb.var, tb.cost, nv, hist);
    k_bin_scan<<<1, 32, 0, s>>>(hist, tb.n);
    k_bin_scatter<<<grid_for(nv), kThreads, 0, s>>>(tb.var, tb.cost, nv, hist, tb.warp, tb.cta,
                                                    tb.split_v, tb.wide, tb.search, tb.bucket,
                                                    tb.group);
    cudaFreeAsync(hist, s);
    // hub offsets follow the ordered hub list (at most nv hubs; the unused tail of w
    // is zero so the scan total is the number of hub sub-tasks)
    TRY(cudaMemsetAsync(tb.w, 0, sizeof(int64_t) * nv, s));
    if (hub_max > 0)
      k_hub_eligible<<<grid_for(nv), kThreads, 0, s>>>(tb.split_v, tb.n, g.dptr, hub_max);
    k_hub_weights_list<<<grid_for(nv), kThreads, 0, s>>>(tb.split_v, tb.n, g.dptr, hub_max,
                                                         tb.w);
    TRY(cudaGetLastError());
    TRY(scan_excl(tb.w, tb.split_off, nv, tb.n + 0, s));
  }
  k_hub_tail<<<1, 1, 0, s>>>(tb.n, tb.split_off);
  return cudaGetLastError();
}

}  // namespace xgm

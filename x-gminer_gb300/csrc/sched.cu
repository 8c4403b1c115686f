// Task generation for the clique kernels: variant per vertex -> ordered task lists.
//
// The reference sizes one grid per launch and grid-strides over the COO edge list
// (clique4_warp_edge.cuh:14) or splits vertices by degree thresholds into warp / block
// / per-hub launches (xgminer/src/glumin/glumin_GM_solver.cu:324-346, 490-503).  Here
// one persistent launch consumes three device-built queues (clique.cu), and the
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

__global__ void k_classify_heur(const longlong2* dptr, int64_t nv, int kmin, int bucket_max,
                                int search_max, int warp_max, int wide_max, int cta_max,
                                uint8_t* var) {
  GRID_STRIDE(r, nv) {
    const longlong2 d = dptr[r];
    const int64_t s = d.y - d.x;
    uint8_t v;
    if (s < kmin) v = VAR_SKIP;
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
      if (v > VAR_BUCKET) v = VAR_SPLIT;
      if ((v == VAR_SEARCH || v == VAR_BUCKET) && s > kWarpCap) v = VAR_WIDE;
      if (v == VAR_WARP && s > kWarpCap) v = VAR_WIDE;
      if (v == VAR_WIDE && s > kWideCap) v = VAR_CTA;
      if (v == VAR_CTA && s > kCtaCap) v = VAR_SPLIT;
    }
    var[r] = v;
  }
}

__global__ void k_flag_eq(const uint8_t* var, int64_t nv, uint8_t x, uint8_t* flag) {
  GRID_STRIDE(r, nv) flag[r] = var[r] == x;
}

__global__ void k_scatter(const uint8_t* flag, const int64_t* pos, int64_t nv, int32_t* out) {
  GRID_STRIDE(r, nv) if (flag[r]) out[pos[r]] = (int32_t)r;
}

__global__ void k_hub_weights(const uint8_t* var, const longlong2* dptr, int64_t nv, int64_t* w) {
  GRID_STRIDE(r, nv) {
    const longlong2 d = dptr[r];
    w[r] = var[r] == VAR_SPLIT ? (d.y - d.x) : 0;
  }
}

__global__ void k_hub_offsets(const uint8_t* var, const int64_t* pos, const int64_t* w, int64_t nv,
                              int64_t* split_off) {
  GRID_STRIDE(r, nv) if (var[r] == VAR_SPLIT) split_off[pos[r]] = w[r];
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
    // var code -> n[] slot: WARP 2, CTA 1, SPLIT 3, WIDE 4, SEARCH 5, BUCKET 6
    n[v == VAR_WARP ? 2 : v == VAR_CTA ? 1 : v == VAR_SPLIT ? 3 : v == VAR_WIDE ? 4
      : v == VAR_SEARCH ? 5 : 6] = (int64_t)run;
  }
}

__global__ void k_bin_scatter(const uint8_t* var, const float* cost, int64_t nv,
                              unsigned long long* cursor, int32_t* warp_l, int32_t* cta_l,
                              int32_t* hub_l, int32_t* wide_l, int32_t* search_l,
                              int32_t* bucket_l) {
  GRID_STRIDE(r, nv) {
    const uint8_t v = var[r];
    if (v < kNumVar) {
      const unsigned long long p = atomicAdd(&cursor[v * kBins + cost_bin(cost[r])], 1ull);
      int32_t* out = v == VAR_WARP    ? warp_l
                     : v == VAR_CTA   ? cta_l
                     : v == VAR_SPLIT ? hub_l
                     : v == VAR_WIDE  ? wide_l
                     : v == VAR_SEARCH ? search_l
                                      : bucket_l;
      out[p] = (int32_t)r;
    }
  }
}

// Hub sub-task offsets in hub-list order.
__global__ void k_hub_weights_list(const int32_t* hubs, const int64_t* n, const longlong2* dptr,
                                   int64_t* w) {
  const int64_t nh = n[3];
  GRID_STRIDE(h, nh) {
    const longlong2 d = dptr[hubs[h]];
    w[h] = d.y - d.x;
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
  t.split_v = split_v;
  t.split_off = split_off;
  t.n = n;
  if (with_log && log) {
    t.log_cta = log;
    t.log_warp = log + cap_v;
    t.log_wide = log + 2 * cap_v;
    t.log_search = log + 3 * cap_v;
    t.log_bucket = log + 4 * cap_v;
    t.log_split = log + 5 * cap_v;
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
  TRY(dalloc(&tb.split_v, c, s));
  TRY(dalloc(&tb.split_off, c + 1, s));
  TRY(dalloc(&tb.n, 8, s));
  TRY(dalloc(&tb.var, c, s));
  TRY(dalloc(&tb.flag, c, s));
  TRY(dalloc(&tb.pos, c, s));
  TRY(dalloc(&tb.w, c, s));
  TRY(dalloc(&tb.cost, c, s));
  TRY(dalloc(&tb.tmp, c, s));
  tb.cap_v = c;
  return cudaSuccess;
}

void taskbuf_free(TaskBuf& tb, cudaStream_t s) {
  void* ps[] = {tb.cta, tb.warp, tb.wide, tb.search, tb.bucket, tb.split_v, tb.split_off, tb.n, tb.var,
                tb.flag, tb.pos, tb.w, tb.cost, tb.tmp, tb.log};
  for (void* p : ps)
    if (p) cudaFreeAsync(p, s);
  tb = TaskBuf{};
}

cudaError_t classify_heuristic(const DevGraph& g, int k, int warp_max, int wide_max, int cta_max,
                               TaskBuf& tb, cudaStream_t s, int search_max, int bucket_max) {
  if (search_max > kWarpCap) search_max = kWarpCap;
  if (bucket_max > kWarpCap) bucket_max = kWarpCap;
  if (warp_max > kWarpCap) warp_max = kWarpCap;
  if (wide_max > kWideCap) wide_max = kWideCap;
  if (k < 2) k = 2;
  if (cta_max > kCtaCap) cta_max = kCtaCap;
  if (g.nv == 0) return cudaSuccess;
  k_classify_heur<<<grid_for(g.nv), kThreads, 0, s>>>(g.dptr, g.nv, k - 1, bucket_max, search_max,
                                                      warp_max, wide_max, cta_max, tb.var);
  return cudaGetLastError();
}

cudaError_t classify_table(const DevGraph& g, int kmin, const xgm_tune_table& tab, TaskBuf& tb,
                           cudaStream_t s) {
  if (g.nv == 0) return cudaSuccess;
  k_classify_table<<<grid_for(g.nv), kThreads, 0, s>>>(g.dptr, g.nv, kmin, tab, tb.var);
  return cudaGetLastError();
}

cudaError_t build_lists(const DevGraph& g, TaskBuf& tb, bool order, cudaStream_t s) {
  const int64_t nv = g.nv;
  TRY(cudaMemsetAsync(tb.n, 0, 8 * sizeof(int64_t), s));
  if (nv == 0) return cudaMemsetAsync(tb.split_off, 0, sizeof(int64_t), s);
  if (!order) {
    // the hub pass goes last: its positions are reused for the hub offsets below
    const uint8_t codes[6] = {VAR_CTA, VAR_WARP, VAR_WIDE, VAR_SEARCH, VAR_BUCKET, VAR_SPLIT};
    int32_t* outs[6] = {tb.cta, tb.warp, tb.wide, tb.search, tb.bucket, tb.split_v};
    int64_t* cnts[6] = {tb.n + 1, tb.n + 2, tb.n + 4, tb.n + 5, tb.n + 6, tb.n + 3};
    for (int x = 0; x < 6; ++x) {
      k_flag_eq<<<grid_for(nv), kThreads, 0, s>>>(tb.var, nv, codes[x], tb.flag);
      TRY(scan_excl(tb.flag, tb.pos, nv, cnts[x], s));
      k_scatter<<<grid_for(nv), kThreads, 0, s>>>(tb.flag, tb.pos, nv, outs[x]);
    }
    // tb.pos still holds the hub positions (last pass)
    k_hub_weights<<<grid_for(nv), kThreads, 0, s>>>(tb.var, g.dptr, nv, tb.w);
    TRY(scan_excl(tb.w, tb.w, nv, tb.n + 0, s));
    k_hub_offsets<<<grid_for(nv), kThreads, 0, s>>>(tb.var, tb.pos, tb.w, nv, tb.split_off);
  } else {
    unsigned long long* hist = nullptr;
    TRY(dalloc(&hist, kNumVar * kBins, s));
    TRY(cudaMemsetAsync(hist, 0, kNumVar * kBins * sizeof(unsigned long long), s));
    k_bin_hist<<<grid_for(nv), kThreads, 0, s>>>(tb.var, tb.cost, nv, hist);
    k_bin_scan<<<1, 32, 0, s>>>(hist, tb.n);
    k_bin_scatter<<<grid_for(nv), kThreads, 0, s>>>(tb.var, tb.cost, nv, hist, tb.warp, tb.cta,
                                                    tb.split_v, tb.wide, tb.search, tb.bucket);
    cudaFreeAsync(hist, s);
    // hub offsets follow the ordered hub list (at most nv hubs; the unused tail of w
    // is zero so the scan total is the number of hub sub-tasks)
    TRY(cudaMemsetAsync(tb.w, 0, sizeof(int64_t) * nv, s));
    k_hub_weights_list<<<grid_for(nv), kThreads, 0, s>>>(tb.split_v, tb.n, g.dptr, tb.w);
    TRY(cudaGetLastError());
    TRY(scan_excl(tb.w, tb.split_off, nv, tb.n + 0, s));
  }
  k_hub_tail<<<1, 1, 0, s>>>(tb.n, tb.split_off);
  return cudaGetLastError();
}

}  // namespace xgm

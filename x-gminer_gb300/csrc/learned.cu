// Learned scheduler: task features, a 12 -> 32 -> 1 MLP (fp16 weights, fp32
// accumulation) with hand-written forward / backward / Adam kernels, the fused
// classify kernel used by XGM_SCHED_LEARNED, and per-task timing collection.
//
// No counterpart in the reference: its schedule is the fixed degree-threshold split
// (xgminer/include/glumin/common.h:114-116, glumin_GM_solver.cu:324-346); its only
// per-task instrumentation counts binary-search probes (search.cuh:39,
// glumin_GM_solver.cu:1015-1033).  Here the engine logs per-task clock64 durations and
// learns log2(warp-cycles) per (task, variant).  The model decides the variant a task
// runs with and the queue order; counts are identical under every schedule.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "api_internal.h"
#include "learned.cuh"

namespace xgm {

namespace {

constexpr int kThreads = 256;

// By default a task leaves the heuristic's variant only for a predicted saving of at
// least 0.2 in log2 warp-cycles (~15%): near-ties are where the model is least
// reliable.  xgm_sched.margin overrides it (the trainer picks it on held-out graphs).
constexpr float kLearnedMargin = 0.2f;

inline unsigned grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  if (b > 65536) b = 65536;
  return (unsigned)b;
}

// Warps a task of each variant occupies while it runs (resource-time weight).
__host__ __device__ inline float variant_warps(int v) {
  return (v == XGM_VAR_CTA || v == XGM_VAR_SPLIT) ? (float)kCtaWarps
         : v == XGM_VAR_GROUP                      ? 1.0f / kGroupsPerWarp
                                                   : 1.0f;
}

// Features of vertex task r (variant one-hot left zero for the caller).
__device__ void task_features(const GView& g, int32_t r, int k, float* f) {
  const longlong2 d0 = g.dptr[r];
  const long long s = d0.y - d0.x;
  long long sum = 0, maxd = 0;
  if (g.tsum) {  // precomputed (ensure_task_stats)
    sum = g.tsum[r];
    maxd = g.tmax[r];
  } else {
    for (long long e = d0.x; e < d0.y; ++e) {
      const longlong2 d = g.dptr[g.col[e]];
      const long long l = d.y - d.x;
      sum += l;
      maxd = l > maxd ? l : maxd;
    }
  }
  // 0-3 task shape, 4 clique depth, 5-11 variant one-hot (caller)
  f[0] = log2f(1.0f + (float)s) / 11.0f;
  f[1] = log2f(1.0f + (float)sum) / 24.0f;
  f[2] = log2f(1.0f + (float)maxd) / 11.0f;
  f[3] = (float)sum / ((float)s * (float)maxd + 1.0f);
  f[4] = k == kFeatMulti ? 0.75f : (float)(k - 3) * 0.5f;
  for (int v = 0; v < XGM_NUM_VARIANTS; ++v) f[kShapeFeat + v] = 0.0f;
}

__device__ __forceinline__ float mlp_forward(const float* P, const float* f) {
  float y = P[kOffB2];
#pragma unroll 4
  for (int h = 0; h < kHidden; ++h) {
    float a = P[kOffB1 + h];
#pragma unroll
    for (int j = 0; j < kFeat; ++j) a = fmaf(P[h * kFeat + j], f[j], a);
    y = fmaf(P[kOffW2 + h], fmaxf(a, 0.0f), y);
  }
  return y;
}

__device__ __forceinline__ void load_params(const __half* wh, float* P) {
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) P[i] = __half2float(wh[i]);
  __syncthreads();
}

// The model over the variants of one task: the first layer's task-shape part
// (features 0-5) is shared, each variant adds its one-hot column.
__device__ __forceinline__ void mlp_variants(const float* P, const float* f, const bool* cand,
                                             float* pred) {
#pragma unroll
  for (int v = 0; v < XGM_NUM_VARIANTS; ++v) pred[v] = P[kOffB2];
#pragma unroll 4
  for (int h = 0; h < kHidden; ++h) {
    float a = P[kOffB1 + h];
#pragma unroll
    for (int j = 0; j < kShapeFeat; ++j) a = fmaf(P[h * kFeat + j], f[j], a);
    const float w2 = P[kOffW2 + h];
#pragma unroll
    for (int v = 0; v < XGM_NUM_VARIANTS; ++v)
      if (cand[v]) pred[v] = fmaf(w2, fmaxf(a + P[h * kFeat + kShapeFeat + v], 0.0f), pred[v]);
  }
}

__global__ void k_classify_learned(GView g, int k, int k_feat, const __half* wh, uint8_t* var,
                                   float* cost, int need_cost, float margin) {
  __shared__ float P[kParams];
  load_params(wh, P);
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < g.nv;
       r += (int64_t)gridDim.x * blockDim.x) {
    const longlong2 d0 = g.dptr[r];
    const long long s = d0.y - d0.x;
    if (s < k - 1) {
      var[r] = VAR_SKIP;
      cost[r] = 0.0f;
      continue;
    }
    // the plain heuristic's variant stays unless the model predicts a clear saving
    const uint8_t hv = s <= kWarpCap ? VAR_WARP : s <= kWideCap ? VAR_WIDE
                       : s <= kCtaCap ? VAR_CTA : VAR_SPLIT;
    bool cand[XGM_NUM_VARIANTS];
    int ncand = 0;
    for (int v = 0; v < XGM_NUM_VARIANTS; ++v) {
      // edge-splitting stays the capacity fallback: splitting a task a CTA can hold
      // multiplies its set-up work and never paid off in any measured configuration
      cand[v] = !(((v == XGM_VAR_WARP || v == XGM_VAR_SEARCH || v == XGM_VAR_BUCKET) &&
                   s > kWarpCap) ||
                  (v == XGM_VAR_GROUP && s > kGroupCap) ||
                  (v == XGM_VAR_WIDE && (s > kWideCap || s <= kWarpCap)) ||
                  (v == XGM_VAR_CTA && s > kCtaCap) ||
                  (v == XGM_VAR_SPLIT && s <= kCtaCap));
      ncand += cand[v];
    }
    if (ncand == 1 && !need_cost) {  // nothing to decide and no order to give
      var[r] = hv;
      cost[r] = 0.0f;
      continue;
    }
    float f[kFeat];
    task_features(g, (int32_t)r, k_feat, f);
    float pred[XGM_NUM_VARIANTS];
    mlp_variants(P, f, cand, pred);
    for (int v = 0; v < XGM_NUM_VARIANTS; ++v)
      if (!cand[v]) pred[v] = 3.0e38f;
    uint8_t bv = hv;
    float best = pred[hv];
    for (int v = 0; v < XGM_NUM_VARIANTS; ++v)
      if (pred[v] < best - (v == hv ? 0.0f : margin)) {
        best = pred[v] + margin;  // later candidates must beat the incumbent too
        bv = (uint8_t)v;
      }
    var[r] = bv;
    cost[r] = pred[bv];
  }
}

__global__ void k_predict(const __half* wh, const float* X, int64_t n, float* y) {
  __shared__ float P[kParams];
  load_params(wh, P);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = mlp_forward(P, X + i * kFeat);
}

// Mean squared error over samples idx[0..n) (or 0..n when idx is null) and, when grad
// is non-null, its gradient with respect to the fp16-rounded parameters.
__global__ void k_loss_grad(const __half* wh, const float* X, const float* Y, const int32_t* idx,
                            int64_t n, float inv_n, float* grad, float* loss) {
  __shared__ float P[kParams];
  __shared__ float G[kParams];
  __shared__ float L;
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) G[i] = 0.0f;
  if (threadIdx.x == 0) L = 0.0f;
  load_params(wh, P);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx ? idx[t] : t;
    const float* f = X + i * kFeat;
    float a[kHidden];
    float yhat = P[kOffB2];
#pragma unroll
    for (int h = 0; h < kHidden; ++h) {
      float z = P[kOffB1 + h];
#pragma unroll
      for (int j = 0; j < kFeat; ++j) z = fmaf(P[h * kFeat + j], f[j], z);
      a[h] = z;
      yhat = fmaf(P[kOffW2 + h], fmaxf(z, 0.0f), yhat);
    }
    const float r = yhat - Y[i];
    atomicAdd(&L, r * r * inv_n);
    if (grad) {
      const float dy = 2.0f * r * inv_n;
      atomicAdd(&G[kOffB2], dy);
#pragma unroll
      for (int h = 0; h < kHidden; ++h) {
        if (a[h] > 0.0f) {
          atomicAdd(&G[kOffW2 + h], dy * a[h]);
          const float dz = dy * P[kOffW2 + h];
          atomicAdd(&G[kOffB1 + h], dz);
#pragma unroll
          for (int j = 0; j < kFeat; ++j) atomicAdd(&G[h * kFeat + j], dz * f[j]);
        }
      }
    }
  }
  __syncthreads();
  if (grad)
    for (int i = threadIdx.x; i < kParams; i += blockDim.x)
      if (G[i] != 0.0f) atomicAdd(&grad[i], G[i]);
  if (threadIdx.x == 0 && L != 0.0f) atomicAdd(loss, L);
}

__global__ void k_adam(float* master, float* m, float* v, const float* grad, __half* wh, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float gi = grad[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float w = master[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  master[i] = w;
  wh[i] = __float2half_rn(w);
}

__global__ void k_to_half(const float* p, __half* wh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kParams) wh[i] = __float2half_rn(p[i]);
}

// Samples from a timed run: list positions 0, stride, 2*stride, ... of one variant.
__global__ void k_assemble(GView g, int k, int variant, const int32_t* list, const int64_t* n,
                           int nidx, const long long* log, const int64_t* split_off, int stride,
                           float* X, float* Y, int64_t max_rows, unsigned long long* rows) {
  const int64_t nt = n[nidx];
  for (int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * stride; t < nt;
       t += (int64_t)gridDim.x * blockDim.x * stride) {
    const int32_t r = list[t];
    double cyc = 0;
    if (variant == XGM_VAR_SPLIT) {
      for (int64_t u = split_off[t]; u < split_off[t + 1]; ++u) cyc += (double)log[u];
    } else {
      cyc = (double)log[t];
    }
    const unsigned long long o = atomicAdd(rows, 1ull);
    if ((int64_t)o >= max_rows) continue;
    float* f = X + o * kFeat;
    task_features(g, r, k, f);
    f[kShapeFeat + variant] = 1.0f;
    Y[o] = log2f((float)fmax(cyc, 1.0) * variant_warps(variant));
  }
}

uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

int clique_k(int pattern) {
  switch (pattern) {
    case XGM_PATTERN_TRIANGLE: return 3;
    case XGM_PATTERN_CLIQUE4: return 4;
    case XGM_PATTERN_CLIQUE5: return 5;
    case XGM_PATTERN_CLIQUE6: return 6;
    case XGM_PATTERN_CLIQUE7: return 7;
    case XGM_PATTERN_DIAMOND:
    case XGM_PATTERN_TAILED_TRIANGLE: return 3;  // same task structure (k = 3 kernel)
    default: return 0;
  }
}

}  // namespace

// Out-neighbour degree sum and maximum of every vertex, a warp per vertex (coalesced over
// its out-list): the features task_features would otherwise gather serially per task.
__global__ void k_task_stats(GView g, int64_t* tsum, int32_t* tmax) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < g.nv; r += warps) {
    const longlong2 d0 = g.dptr[r];
    long long sum = 0, maxd = 0;
    for (long long e = d0.x + lane; e < d0.y; e += 32) {
      const longlong2 d = g.dptr[g.col[e]];
      const long long l = d.y - d.x;
      sum += l;
      maxd = l > maxd ? l : maxd;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sum += __shfl_xor_sync(kFull, sum, o);
      const long long y = __shfl_xor_sync(kFull, maxd, o);
      maxd = y > maxd ? y : maxd;
    }
    if (lane == 0) {
      tsum[r] = sum;
      tmax[r] = (int32_t)maxd;
    }
  }
}

cudaError_t ensure_task_stats(const DevGraph& g, cudaStream_t s) {
  if (g.tsum || g.nv == 0) return cudaSuccess;
  int64_t* tsum = nullptr;
  int32_t* tmax = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&tsum, sizeof(int64_t) * (size_t)g.nv, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&tmax, sizeof(int32_t) * (size_t)g.nv, s);
  if (e != cudaSuccess) {
    if (tsum) cudaFreeAsync(tsum, s);
    return e;
  }
  int64_t blocks = (g.nv + kThreads / 32 - 1) / (kThreads / 32);
  if (blocks > 65536) blocks = 65536;
  k_task_stats<<<(unsigned)blocks, kThreads, 0, s>>>(g.view(), tsum, tmax);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFreeAsync(tsum, s);
    cudaFreeAsync(tmax, s);
    return e;
  }
  g.tsum = tsum;
  g.tmax = tmax;
  return cudaSuccess;
}

cudaError_t classify_learned(const DevGraph& g, int k, const xgm_model& m, TaskBuf& tb,
                             bool need_cost, float margin, cudaStream_t s, int k_feat) {
  if (g.nv == 0) return cudaSuccess;
  k_classify_learned<<<grid_for(g.nv), kThreads, 0, s>>>(g.view(), k, k_feat > 0 ? k_feat : k,
                                                         m.wh, tb.var, tb.cost,
                                                         need_cost ? 1 : 0,
                                                         margin > 0.0f ? margin : kLearnedMargin);
  return cudaGetLastError();
}

}  // namespace xgm

using namespace xgm;

extern "C" {

xgm_status xgm_model_create(xgm_ctx* ctx, uint64_t seed, xgm_model** out) {
  if (!ctx || !out) return XGM_ERR_INVALID;
  *out = nullptr;
  std::vector<float> p(kParams, 0.0f);
  uint64_t st = seed;
  auto uni = [&](float a) {
    st = mix64(st);
    return (float)((double)(st >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0) * a;
  };
  for (int i = 0; i < kHidden * kFeat; ++i) p[i] = uni(1.0f / std::sqrt((float)kFeat) * 1.7f);
  for (int h = 0; h < kHidden; ++h) p[kOffB1 + h] = 0.1f;
  for (int h = 0; h < kHidden; ++h) p[kOffW2 + h] = uni(1.0f / std::sqrt((float)kHidden) * 1.7f);
  p[kOffB2] = 12.0f;  // log2 cycles of a typical small task
  xgm_model* m = new xgm_model();
  m->ctx = ctx;
  cudaError_t e = cudaMalloc(&m->wh, sizeof(__half) * kParams);
  if (e == cudaSuccess) e = cudaMalloc(&m->master, sizeof(float) * kParams);
  if (e == cudaSuccess) e = cudaMalloc(&m->m, sizeof(float) * kParams);
  if (e == cudaSuccess) e = cudaMalloc(&m->v, sizeof(float) * kParams);
  if (e == cudaSuccess) e = cudaMemset(m->m, 0, sizeof(float) * kParams);
  if (e == cudaSuccess) e = cudaMemset(m->v, 0, sizeof(float) * kParams);
  if (e != cudaSuccess) {
    xgm_model_destroy(m);
    return finish_status(ctx, cuda_fail(e, "xgm_model_create", __FILE__, __LINE__));
  }
  xgm_status r = xgm_model_set_params(m, p.data());
  if (r != XGM_OK) {
    xgm_model_destroy(m);
    return r;
  }
  *out = m;
  return XGM_OK;
}

void xgm_model_destroy(xgm_model* m) {
  if (!m) return;
  if (m->wh) cudaFree(m->wh);
  if (m->master) cudaFree(m->master);
  if (m->m) cudaFree(m->m);
  if (m->v) cudaFree(m->v);
  delete m;
}

xgm_status xgm_model_set_params(xgm_model* m, const float* params) {
  if (!m || !params) return XGM_ERR_INVALID;
  XGM_CUDA_TRY(cudaMemcpy(m->master, params, sizeof(float) * kParams, cudaMemcpyHostToDevice));
  k_to_half<<<(kParams + 255) / 256, 256>>>(m->master, m->wh);
  XGM_CUDA_TRY(cudaGetLastError());
  XGM_CUDA_TRY(cudaDeviceSynchronize());
  return XGM_OK;
}

xgm_status xgm_model_get_params(const xgm_model* m, float* params) {
  if (!m || !params) return XGM_ERR_INVALID;
  XGM_CUDA_TRY(cudaMemcpy(params, m->master, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
  return XGM_OK;
}

xgm_status xgm_model_predict(xgm_ctx* ctx, const xgm_model* m, const float* X, int64_t n, float* y) {
  if (!ctx || !m || (n > 0 && (!X || !y)) || n < 0) return XGM_ERR_INVALID;
  if (n == 0) return XGM_OK;
  cudaStream_t s = ctx->stream;
  float *dx = nullptr, *dy = nullptr;
  XGM_CUDA_TRY(cudaMallocAsync(&dx, sizeof(float) * n * kFeat, s));
  XGM_CUDA_TRY(cudaMallocAsync(&dy, sizeof(float) * n, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(dx, X, sizeof(float) * n * kFeat, cudaMemcpyHostToDevice, s));
  k_predict<<<grid_for(n), kThreads, 0, s>>>(m->wh, dx, n, dy);
  XGM_CUDA_TRY(cudaGetLastError());
  XGM_CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(dx, s);
  cudaFreeAsync(dy, s);
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  return XGM_OK;
}

xgm_status xgm_model_loss_grad(xgm_ctx* ctx, const xgm_model* m, const float* X, const float* y,
                               int64_t n, float* loss, float* grad) {
  if (!ctx || !m || n <= 0 || !X || !y || !loss) return XGM_ERR_INVALID;
  cudaStream_t s = ctx->stream;
  float *dx = nullptr, *dy = nullptr, *dg = nullptr;
  XGM_CUDA_TRY(cudaMallocAsync(&dx, sizeof(float) * n * kFeat, s));
  XGM_CUDA_TRY(cudaMallocAsync(&dy, sizeof(float) * n, s));
  XGM_CUDA_TRY(cudaMallocAsync(&dg, sizeof(float) * (kParams + 1), s));
  XGM_CUDA_TRY(cudaMemcpyAsync(dx, X, sizeof(float) * n * kFeat, cudaMemcpyHostToDevice, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  XGM_CUDA_TRY(cudaMemsetAsync(dg, 0, sizeof(float) * (kParams + 1), s));
  k_loss_grad<<<grid_for(n), kThreads, 0, s>>>(m->wh, dx, dy, nullptr, n, 1.0f / (float)n,
                                               grad ? dg : nullptr, dg + kParams);
  XGM_CUDA_TRY(cudaGetLastError());
  std::vector<float> h(kParams + 1);
  XGM_CUDA_TRY(cudaMemcpyAsync(h.data(), dg, sizeof(float) * (kParams + 1), cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(dx, s);
  cudaFreeAsync(dy, s);
  cudaFreeAsync(dg, s);
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  *loss = h[kParams];
  if (grad) std::memcpy(grad, h.data(), sizeof(float) * kParams);
  return XGM_OK;
}

xgm_status xgm_model_train(xgm_ctx* ctx, xgm_model* m, const float* X, const float* y, int64_t n,
                           int epochs, int batch, float lr, uint64_t seed, float* final_loss) {
  if (!ctx || !m || n <= 0 || !X || !y || epochs < 0 || batch <= 0 || !(lr > 0))
    return XGM_ERR_INVALID;
  cudaStream_t s = ctx->stream;
  float *dx = nullptr, *dy = nullptr, *dg = nullptr;
  int32_t* didx = nullptr;
  XGM_CUDA_TRY(cudaMallocAsync(&dx, sizeof(float) * n * kFeat, s));
  XGM_CUDA_TRY(cudaMallocAsync(&dy, sizeof(float) * n, s));
  XGM_CUDA_TRY(cudaMallocAsync(&dg, sizeof(float) * (kParams + 1), s));
  XGM_CUDA_TRY(cudaMallocAsync(&didx, sizeof(int32_t) * n, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(dx, X, sizeof(float) * n * kFeat, cudaMemcpyHostToDevice, s));
  XGM_CUDA_TRY(cudaMemcpyAsync(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  std::vector<int32_t> idx(n);
  for (int64_t i = 0; i < n; ++i) idx[i] = (int32_t)i;
  std::mt19937_64 rng(seed);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(idx.begin(), idx.end(), rng);
    XGM_CUDA_TRY(cudaMemcpyAsync(didx, idx.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    XGM_CUDA_TRY(cudaStreamSynchronize(s));  // idx is reused next epoch
    for (int64_t b0 = 0; b0 < n; b0 += batch) {
      const int64_t nb = std::min<int64_t>(batch, n - b0);
      XGM_CUDA_TRY(cudaMemsetAsync(dg, 0, sizeof(float) * (kParams + 1), s));
      k_loss_grad<<<grid_for(nb), kThreads, 0, s>>>(m->wh, dx, dy, didx + b0, nb,
                                                    1.0f / (float)nb, dg, dg + kParams);
      m->step += 1;
      const float c1 = 1.0f - std::pow(b1, (float)m->step);
      const float c2 = 1.0f - std::pow(b2, (float)m->step);
      k_adam<<<(kParams + 255) / 256, 256, 0, s>>>(m->master, m->m, m->v, dg, m->wh, lr, b1, b2,
                                                   eps, c1, c2);
    }
    XGM_CUDA_TRY(cudaGetLastError());
  }
  XGM_CUDA_TRY(cudaMemsetAsync(dg, 0, sizeof(float) * (kParams + 1), s));
  k_loss_grad<<<grid_for(n), kThreads, 0, s>>>(m->wh, dx, dy, nullptr, n, 1.0f / (float)n, nullptr,
                                               dg + kParams);
  float l = 0;
  XGM_CUDA_TRY(cudaMemcpyAsync(&l, dg + kParams, sizeof(float), cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(dx, s);
  cudaFreeAsync(dy, s);
  cudaFreeAsync(dg, s);
  cudaFreeAsync(didx, s);
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  if (final_loss) *final_loss = l;
  return XGM_OK;
}

xgm_status xgm_model_collect(xgm_ctx* ctx, const xgm_graph* g, const xgm_plan* plan, int variant,
                             int stride, float* X, float* y, int64_t max_rows, int64_t* n_rows,
                             uint64_t* count_out) {
  const bool multi = (variant & XGM_COLLECT_MULTI) != 0;
  variant &= ~XGM_COLLECT_MULTI;
  if (!ctx || !g || !plan || !X || !y || !n_rows || max_rows < 0 || stride <= 0 ||
      variant < 0 || variant >= XGM_NUM_VARIANTS)
    return XGM_ERR_INVALID;
  const int k = clique_k(plan->pattern);
  if (!k || (multi && k != 3)) {
    set_thread_error(multi ? "the multi-pattern timing runs with the triangle plan"
                           : "timing collection covers the triangle / clique / participation plans");
    return finish_status(ctx, XGM_ERR_UNSUPPORTED);
  }
  cudaStream_t s = ctx->stream;
  const DevGraph& G = g->g;
  TaskBuf& tb = ctx->tb;
  XGM_CUDA_TRY(cudaSetDevice(ctx->device));
  XGM_CUDA_TRY(taskbuf_reserve(tb, G.nv, s));
  const int64_t need = 6 * tb.cap_v + (G.ne_dag > 0 ? G.ne_dag : 1);
  if (tb.log_cap < need) {
    if (tb.log) cudaFreeAsync(tb.log, s);
    tb.log = nullptr;
    XGM_CUDA_TRY(cudaMallocAsync(&tb.log, sizeof(long long) * need, s));
    tb.log_cap = need;
  }
  int gmax = 0, bmax = 0, smax = 0, wmax = kWarpCap, dmax = kWideCap, cmax = kCtaCap;
  if (variant == XGM_VAR_GROUP) gmax = kGroupCap;
  if (variant == XGM_VAR_BUCKET) {
    bmax = kWarpCap;
    XGM_CUDA_TRY(ensure_bucket_index(G, s));
  }
  if (variant == XGM_VAR_SEARCH) smax = kWarpCap;
  if (variant == XGM_VAR_WIDE) wmax = 0;
  if (variant == XGM_VAR_CTA) wmax = dmax = 0;
  if (variant == XGM_VAR_SPLIT) wmax = dmax = cmax = 0;
  XGM_CUDA_TRY(classify_heuristic(G, k, wmax, dmax, cmax, tb, s, smax, bmax, gmax));
  XGM_CUDA_TRY(build_lists(G, tb, false, s));
  XGM_CUDA_TRY(cudaMemsetAsync(ctx->d_sc, 0, sizeof(Scalars), s));
  const int grid = ctx->clique_grid > 0 ? ctx->clique_grid : 2 * ctx->num_sms;
  unsigned long long* vpart = nullptr;
  unsigned* epart = nullptr;
  if (multi) {  // per-task triangles + 4-cliques + participation, as in the batched launch
    XGM_CUDA_TRY(cudaMallocAsync(&vpart, sizeof(unsigned long long) * (G.nv > 0 ? G.nv : 1), s));
    XGM_CUDA_TRY(cudaMallocAsync(&epart, sizeof(unsigned) * (G.ne > 0 ? G.ne : 1), s));
    XGM_CUDA_TRY(cudaMemsetAsync(vpart, 0, sizeof(unsigned long long) * (G.nv > 0 ? G.nv : 1), s));
    XGM_CUDA_TRY(cudaMemsetAsync(epart, 0, sizeof(unsigned) * (G.ne > 0 ? G.ne : 1), s));
    XGM_CUDA_TRY(launch_multi(G.view(), tb.lists(true), &ctx->d_sc->q, vpart, epart,
                              &ctx->d_sc->err, grid, s, GOut{}));
  } else {
    XGM_CUDA_TRY(launch_clique(k, G.view(), tb.lists(true), &ctx->d_sc->q, &ctx->d_sc->count,
                               &ctx->d_sc->err, grid, s));
  }
  float *dx = nullptr, *dy = nullptr;
  const int64_t cap = max_rows > 0 ? max_rows : 1;
  XGM_CUDA_TRY(cudaMallocAsync(&dx, sizeof(float) * cap * kFeat, s));
  XGM_CUDA_TRY(cudaMallocAsync(&dy, sizeof(float) * cap, s));
  const TaskLists tl = tb.lists(true);
  const int32_t* list = variant == XGM_VAR_WARP     ? tb.warp
                        : variant == XGM_VAR_CTA    ? tb.cta
                        : variant == XGM_VAR_WIDE   ? tb.wide
                        : variant == XGM_VAR_SEARCH ? tb.search
                        : variant == XGM_VAR_BUCKET ? tb.bucket
                        : variant == XGM_VAR_GROUP  ? tb.group
                                                    : tb.split_v;
  const int nidx = variant == XGM_VAR_WARP     ? 2
                   : variant == XGM_VAR_CTA    ? 1
                   : variant == XGM_VAR_WIDE   ? 4
                   : variant == XGM_VAR_SEARCH ? 5
                   : variant == XGM_VAR_BUCKET ? 6
                   : variant == XGM_VAR_GROUP  ? 7
                                               : 3;
  const long long* lg = variant == XGM_VAR_WARP     ? tl.log_warp
                        : variant == XGM_VAR_CTA    ? tl.log_cta
                        : variant == XGM_VAR_WIDE   ? tl.log_wide
                        : variant == XGM_VAR_SEARCH ? tl.log_search
                        : variant == XGM_VAR_BUCKET ? tl.log_bucket
                        : variant == XGM_VAR_GROUP  ? tl.log_group
                                                    : tl.log_split;
  k_assemble<<<grid_for(G.nv), kThreads, 0, s>>>(G.view(), multi ? kFeatMulti : k, variant, list, tb.n, nidx, lg,
                                                 tb.split_off, stride, dx, dy, max_rows,
                                                 &ctx->d_sc->aux);
  XGM_CUDA_TRY(cudaGetLastError());
  xgm_status r = ctx_sync_scalars(ctx);
  if (r == XGM_OK) r = check_device_flag(ctx, ctx->h_sc->err);
  if (r == XGM_OK) {
    const int64_t rows = std::min<int64_t>((int64_t)ctx->h_sc->aux, max_rows);
    if (rows > 0) {
      XGM_CUDA_TRY(cudaMemcpyAsync(X, dx, sizeof(float) * rows * kFeat, cudaMemcpyDeviceToHost, s));
      XGM_CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(float) * rows, cudaMemcpyDeviceToHost, s));
    }
    *n_rows = rows;
    if (count_out) *count_out = ctx->h_sc->count;
  }
  cudaFreeAsync(dx, s);
  cudaFreeAsync(dy, s);
  if (vpart) cudaFreeAsync(vpart, s);
  if (epart) cudaFreeAsync(epart, s);
  XGM_CUDA_TRY(cudaStreamSynchronize(s));
  return finish_status(ctx, r);
}

}  // extern "C"

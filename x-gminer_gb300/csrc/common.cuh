// Shared device-side definitions of the GB300 counting engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/xgm.h"

namespace xgm {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xFFFFFFFFu;

// Device error flag bits (OR-ed into Counters::err).
enum : uint32_t {
  ERR_CAPACITY = 1u,   // a task exceeded the capacity of the variant it was given
  ERR_BOUNDS = 2u,     // an index check failed
  ERR_TIMEOUT = 4u,    // a bounded wait ran out
};

// Graph view the counting kernels read.  Vertex ids are degree ranks, so that the
// degree orientation u -> v (deg v > deg u, ties by id; graph.cc:233-275) is simply
// rank(v) > rank(u), and the out-neighbours N+(r) of r are the upper part of its
// sorted undirected row: col[dptr[r].x .. dptr[r].y).  Lower part (ids < r):
// col[rowptr[r] .. dptr[r].x).
// Bucket index of the out-lists (the BUCKET variant; null until a schedule needs it):
// out-list N+(u) = col[dptr[u].x, dptr[u].y) regrouped by bucket b = id & 15 into
// bcol[dptr[u].x, ...), ascending inside a bucket; bucket b starts boff[16u + b]
// entries into the row; bit b of bmask[u] is set iff bucket b is not empty.
constexpr int kBuckets = 16;

struct GView {
  const int32_t* col;        // undirected adjacency, rank ids, sorted rows
  const int64_t* rowptr;     // [V+1] undirected row starts
  const longlong2* dptr;     // [V] {first out-neighbour, row end}
  int64_t nv;
  const int32_t* bcol = nullptr;    // [E] bucket-grouped out-lists (same row positions)
  const uint32_t* boff = nullptr;   // [16 V] bucket starts within each out-list
  const uint16_t* bmask = nullptr;  // [V] non-empty buckets
  const int64_t* tsum = nullptr;    // [V] sum of the out-neighbours' out-degrees
  const int32_t* tmax = nullptr;    // [V] largest out-neighbour out-degree
};

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
  return v;
}

// Row load that bypasses L1 allocation for streaming adjacency reads.
__device__ __forceinline__ int32_t ldg_i32(const int32_t* p) { return __ldg(p); }
__device__ __forceinline__ longlong2 ldg_ll2(const longlong2* p) { return __ldg(p); }

// Number of 32-bit words in the triangular bitmap of an s-vertex local DAG whose
// row i keeps words floor(i/32) .. W-1 (bits j > i only), W = ceil(s/32).
__host__ __device__ __forceinline__ int tri_row_off(int i, int W) {
  int q = i >> 5, r = i & 31;
  return i * W - (16 * q * (q - 1) + r * q);
}
__host__ __device__ __forceinline__ int tri_words(int s) {
  int W = (s + 31) >> 5;
  return tri_row_off(s, W);
}

}  // namespace xgm

// Host-side error helpers.
#define XGM_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return ::xgm::cuda_fail(_e, #expr, __FILE__, __LINE__); \
  } while (0)

namespace xgm {
xgm_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);
void set_thread_error(const std::string& msg);
}  // namespace xgm

// Bucket index of the out-lists for the BUCKET task variant.
//
// X-GMiner's pre-filter (xgminer/include/xgminer_bitmap.cuh:661-813,
// bigset_bitmap_processing) splits every adjacency list into 2^k buckets by the low
// bits of the neighbour id (k = BMAP_BUCKET_NUM, 4 by default), keeps a 2^k-bit
// bitmap of the non-empty buckets per vertex and the bucket offsets, and intersects
// two lists by ANDing their bitmaps and searching only inside common buckets
// (:161-278).  The reference builds this on the host, one vertex at a time.  Here one
// warp per vertex builds it on the device for the DAG out-lists: shared-memory bucket
// counters, a 16-entry scan, then a stable scatter in list order (__match_any_sync
// ranks equal buckets inside a 32-element chunk), so every bucket stays sorted.
#include "graph.cuh"

namespace xgm {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

__global__ void __launch_bounds__(kThreads) k_bucket_index(GView g, int32_t* bcol, uint32_t* boff,
                                                           uint16_t* bmask) {
  __shared__ uint32_t cnt[kWarps][kBuckets];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t nwarps = (int64_t)gridDim.x * kWarps;
  for (int64_t r = (int64_t)blockIdx.x * kWarps + wib; r < g.nv; r += nwarps) {
    const longlong2 d = g.dptr[r];
    if (lane < kBuckets) cnt[wib][lane] = 0u;
    __syncwarp();
    for (long long e = d.x + lane; e < d.y; e += 32) atomicAdd(&cnt[wib][g.col[e] & (kBuckets - 1)], 1u);
    __syncwarp();
    const uint32_t c = lane < kBuckets ? cnt[wib][lane] : 0u;
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < kBuckets; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const unsigned nonempty = __ballot_sync(0xffffffffu, lane < kBuckets && c > 0u);
    __syncwarp();
    if (lane < kBuckets) {
      boff[r * kBuckets + lane] = incl - c;
      cnt[wib][lane] = incl - c;  // scatter cursors
    }
    if (lane == 0) bmask[r] = (uint16_t)(nonempty & 0xFFFFu);
    __syncwarp();
    for (long long base = d.x; base < d.y; base += 32) {
      const long long e = base + lane;
      const bool valid = e < d.y;
      const int32_t x = valid ? g.col[e] : 0;
      const int b = x & (kBuckets - 1);
      const unsigned peers = __match_any_sync(0xffffffffu, valid ? b : kBuckets + lane);
      unsigned lt;
      asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
      const uint32_t rank = (uint32_t)__popc(peers & lt);
      uint32_t pos = 0;
      if (valid) pos = cnt[wib][b] + rank;
      __syncwarp();
      if (valid) {
        bcol[d.x + pos] = x;
        if (rank == 0) cnt[wib][b] += (uint32_t)__popc(peers);
      }
      __syncwarp();
    }
  }
}

}  // namespace

cudaError_t ensure_bucket_index(const DevGraph& g, cudaStream_t s) {
  if (g.bcol || g.nv == 0) return cudaSuccess;
  int32_t* bcol = nullptr;
  uint32_t* boff = nullptr;
  uint16_t* bmask = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&bcol, sizeof(int32_t) * (size_t)(g.ne > 0 ? g.ne : 1), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&boff, sizeof(uint32_t) * kBuckets * (size_t)g.nv, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&bmask, sizeof(uint16_t) * (size_t)g.nv, s);
  if (e != cudaSuccess) {
    if (bcol) cudaFreeAsync(bcol, s);
    if (boff) cudaFreeAsync(boff, s);
    return e;
  }
  int64_t blocks = (g.nv + kWarps - 1) / kWarps;
  if (blocks > 65536) blocks = 65536;
  k_bucket_index<<<(unsigned)blocks, kThreads, 0, s>>>(g.view(), bcol, boff, bmask);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFreeAsync(bcol, s);
    cudaFreeAsync(boff, s);
    cudaFreeAsync(bmask, s);
    return e;
  }
  g.bcol = bcol;
  g.boff = boff;
  g.bmask = bmask;
  return cudaSuccess;
}

}  // namespace xgm

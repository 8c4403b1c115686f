// Device-wide primitives used by the CSR build and the scheduler: exclusive scan and
// LSD radix sort of 64-bit keys.  Written for this engine; no library sort or scan is
// on the path.
#include "prim.cuh"

namespace xgm {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // 2048

template <class T>
__device__ __forceinline__ int64_t as_i64(T v) { return (int64_t)v; }

// Block-wide exclusive scan of one int64 per thread; returns the block total too.
__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t* total) {
  __shared__ int64_t warp_tot[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int64_t w = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
    int64_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(kFull, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = wi - w;  // exclusive
    if (lane == kScanThreads / 32 - 1) *total = wi;
  }
  __syncthreads();
  int64_t r = warp_tot[warp] + inc - v;
  __syncthreads();
  return r;
}

template <class T>
__global__ void __launch_bounds__(kScanThreads) k_tile_reduce(const T* in, int64_t n,
                                                              int64_t* partial) {
  __shared__ int64_t red[kScanThreads / 32];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int64_t s = 0;
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    int64_t i = base + t * kScanThreads + threadIdx.x;
    if (i < n) s += as_i64(in[i]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(kFull, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
    partial[blockIdx.x] = t;
  }
}

// out[i] = offset(tile) + exclusive prefix within the tile.  in and out may alias.
template <class T>
__global__ void __launch_bounds__(kScanThreads) k_tile_scan(const T* in, int64_t* out, int64_t n,
                                                            const int64_t* tile_off,
                                                            int64_t* total) {
  __shared__ int64_t buf[kScanTile];
  __shared__ int64_t btotal;
  int64_t base = (int64_t)blockIdx.x * kScanTile;
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    int64_t i = base + t * kScanThreads + threadIdx.x;
    buf[t * kScanThreads + threadIdx.x] = i < n ? as_i64(in[i]) : 0;
  }
  __syncthreads();
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    v[t] = buf[threadIdx.x * kScanItems + t];
    s += v[t];
  }
  int64_t off = block_excl_scan(s, &btotal) + (tile_off ? tile_off[blockIdx.x] : 0);
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    buf[threadIdx.x * kScanItems + t] = off;
    off += v[t];
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < kScanItems; ++t) {
    int64_t i = base + t * kScanThreads + threadIdx.x;
    if (i < n) out[i] = buf[t * kScanThreads + threadIdx.x];
  }
  if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
    *total = (tile_off ? tile_off[blockIdx.x] : 0) + btotal;
}

template <class T>
cudaError_t scan_impl(const T* in, int64_t* out, int64_t n, int64_t* total, cudaStream_t st) {
  if (n <= 0) {
    if (total) return cudaMemsetAsync(total, 0, sizeof(int64_t), st);
    return cudaSuccess;
  }
  int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    k_tile_scan<T><<<1, kScanThreads, 0, st>>>(in, out, n, nullptr, total);
    return cudaGetLastError();
  }
  int64_t* partial = nullptr;
  cudaError_t e = cudaMallocAsync(&partial, sizeof(int64_t) * tiles, st);
  if (e != cudaSuccess) return e;
  k_tile_reduce<T><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, partial);
  e = scan_impl<int64_t>(partial, partial, tiles, nullptr, st);
  if (e == cudaSuccess) {
    k_tile_scan<T><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, partial, total);
    e = cudaGetLastError();
  }
  cudaFreeAsync(partial, st);
  return e;
}

// ------------------------------------------------------------------ radix sort
constexpr int kSortWarps = 8;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortWarps * 32 * kSortItems;  // 2048 keys
constexpr int kRadix = 256;

__global__ void __launch_bounds__(kSortWarps * 32) k_radix_hist(const uint64_t* keys, int64_t n,
                                                               int shift, int64_t* counts,
                                                               int64_t tiles) {
  __shared__ uint32_t h[kRadix];
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) h[d] = 0;
  __syncthreads();
  int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int t = 0; t < kSortTile / (kSortWarps * 32); ++t) {
    int64_t i = base + (int64_t)t * kSortWarps * 32 + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) counts[(int64_t)d * tiles + blockIdx.x] = h[d];
}

// Stable scatter: warp w of the tile owns keys [w*256, (w+1)*256) of the tile and
// walks them in 8 rounds of 32; __match_any_sync groups equal digits inside a round
// so each key gets its rank among equal digits in tile order.  The keys are then
// placed in digit order in shared memory and written out in that order, so every
// digit's run reaches global memory as contiguous, coalesced stores.
__global__ void __launch_bounds__(kSortWarps * 32) k_radix_scatter(const uint64_t* in,
                                                                  uint64_t* out, int64_t n,
                                                                  int shift,
                                                                  const int64_t* offs,
                                                                  int64_t tiles) {
  __shared__ uint64_t sk[kSortTile];
  __shared__ uint32_t wcnt[kSortWarps][kRadix];
  __shared__ uint32_t dstart[kRadix];
  __shared__ uint32_t wsum[kSortWarps];
  __shared__ int64_t gbase[kRadix];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int d = tid; d < kRadix; d += blockDim.x) gbase[d] = offs[(int64_t)d * tiles + blockIdx.x];
  for (int i = tid; i < kSortWarps * kRadix; i += blockDim.x) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int64_t tile0 = (int64_t)blockIdx.x * kSortTile;
  const int tn = (int)min((int64_t)kSortTile, n - tile0);
  const int64_t base = tile0 + warp * (32 * kSortItems);
  uint64_t k[kSortItems];
  uint32_t rk[kSortItems];
#pragma unroll
  for (int t = 0; t < kSortItems; ++t) {
    const int64_t i = base + t * 32 + lane;
    const bool valid = i < n;
    k[t] = valid ? in[i] : 0ull;
    const int d = valid ? (int)((k[t] >> shift) & (kRadix - 1)) : kRadix;
    const unsigned peers = __match_any_sync(kFull, d);
    const uint32_t before = valid ? wcnt[warp][d] : 0u;
    rk[t] = before + __popc(peers & lanemask_lt());
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: exclusive prefix over the warps, then the tile-local start of each digit
  uint32_t tot = 0;
  if (tid < kRadix) {
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t c = wcnt[w][tid];
      wcnt[w][tid] = tot;
      tot += c;
    }
  }
  uint32_t incl = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (tid < kRadix) {
    uint32_t off = 0;
    for (int w = 0; w < warp; ++w) off += wsum[w];
    dstart[tid] = off + incl - tot;
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < kSortItems; ++t) {
    const int64_t i = base + t * 32 + lane;
    if (i < n) {
      const int d = (int)((k[t] >> shift) & (kRadix - 1));
      sk[dstart[d] + wcnt[warp][d] + rk[t]] = k[t];
    }
  }
  __syncthreads();
  for (int i = tid; i < tn; i += blockDim.x) {
    const uint64_t key = sk[i];
    const int d = (int)((key >> shift) & (kRadix - 1));
    out[gbase[d] + (i - (int)dstart[d])] = key;
  }
}

}  // namespace

cudaError_t scan_excl(const int64_t* in, int64_t* out, int64_t n, int64_t* total, cudaStream_t s) {
  return scan_impl<int64_t>(in, out, n, total, s);
}
cudaError_t scan_excl(const int32_t* in, int64_t* out, int64_t n, int64_t* total, cudaStream_t s) {
  return scan_impl<int32_t>(in, out, n, total, s);
}
cudaError_t scan_excl(const uint8_t* in, int64_t* out, int64_t n, int64_t* total, cudaStream_t s) {
  return scan_impl<uint8_t>(in, out, n, total, s);
}

cudaError_t radix_sort_u64(uint64_t* keys, uint64_t* tmp, int64_t n, int bits, cudaStream_t st,
                           int shift0, uint64_t** where) {
  if (where) *where = keys;
  if (n <= 1 || bits <= 0) return cudaSuccess;
  int64_t tiles = (n + kSortTile - 1) / kSortTile;
  int64_t* counts = nullptr;
  cudaError_t e = cudaMallocAsync(&counts, sizeof(int64_t) * kRadix * tiles, st);
  if (e != cudaSuccess) return e;
  uint64_t *a = keys, *b = tmp;
  for (int shift = shift0; shift < shift0 + bits && e == cudaSuccess; shift += 8) {
    k_radix_hist<<<(unsigned)tiles, kSortWarps * 32, 0, st>>>(a, n, shift, counts, tiles);
    e = scan_impl<int64_t>(counts, counts, kRadix * tiles, nullptr, st);
    if (e != cudaSuccess) break;
    k_radix_scatter<<<(unsigned)tiles, kSortWarps * 32, 0, st>>>(a, b, n, shift, counts, tiles);
    e = cudaGetLastError();
    uint64_t* t = a;
    a = b;
    b = t;
  }
  if (e == cudaSuccess && where) *where = a;
  else if (e == cudaSuccess && a != keys)
    e = cudaMemcpyAsync(keys, a, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, st);
  cudaFreeAsync(counts, st);
  return e;
}

}  // namespace xgm

// Algorithmic-bytes counters: the bytes of graph-resident adjacency data each plan
// reads (4 B per int32 list element + 8 B per task record), the numerator of the
// roofline figures.  The W-dependent terms come from the weighted mode of the clique
// kernel (clique.cu); the rest are single passes here.
#include "measure.cuh"

namespace xgm {

namespace {

// kind 0: DAG edges 8 + 4(d+u + d+v)          (triangle / clique plans)
// kind 1: undirected edges v<u 8 + 4(du + dv)  (diamond, diamond.h)
// kind 2: sum_{d(u)>2} sum_{v in N(u)} 4(du + dv)  (tailed triangle, tailedtriangle.h)
// kind 3: sum_u 4 du                           (4-cycle row reads, rectangle.h)
__global__ void k_bytes(GView g, int kind, unsigned long long* out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  unsigned long long acc = 0;
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < g.nv; u += warps) {
    const longlong2 du = g.dptr[u];
    const long long row0 = g.rowptr[u];
    const long long dp = du.y - du.x, d = du.y - row0;
    if (kind == 3) {
      if (lane == 0) acc += 4ull * (unsigned long long)d;
      continue;
    }
    if (kind == 2 && d <= 2) continue;
    const long long b = kind == 2 ? row0 : du.x;
    for (long long e = b + lane; e < du.y; e += 32) {
      const int32_t v = g.col[e];
      const longlong2 dv = g.dptr[v];
      if (kind == 0) acc += 8ull + 4ull * (unsigned long long)(dp + (dv.y - dv.x));
      else if (kind == 1) acc += 8ull + 4ull * (unsigned long long)(d + (dv.y - g.rowptr[v]));
      else acc += 4ull * (unsigned long long)(d + (dv.y - g.rowptr[v]));
    }
  }
  acc = warp_sum_u64(acc);
  if (lane == 0 && acc) atomicAdd(out, acc);
}

__global__ void k_sum_ll(const long long* x, int64_t n, unsigned long long* out) {
  unsigned long long acc = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    acc += (unsigned long long)x[i];
  acc = warp_sum_u64(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

}  // namespace

cudaError_t launch_bytes_basic(const GView& g, int kind, unsigned long long* out, cudaStream_t s) {
  if (g.nv == 0) return cudaSuccess;
  int64_t blocks = (g.nv * 32 + 255) / 256;
  if (blocks > 65536) blocks = 65536;
  k_bytes<<<(unsigned)blocks, 256, 0, s>>>(g, kind, out);
  return cudaGetLastError();
}

cudaError_t launch_sum_ll(const long long* x, int64_t n, unsigned long long* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 65536) blocks = 65536;
  k_sum_ll<<<(unsigned)blocks, 256, 0, s>>>(x, n, out);
  return cudaGetLastError();
}

}  // namespace xgm

// Edge-induced 4-vertex motif plans on the undirected graph (rank ids).
//
// Reference (CPU, the counting definitions): codes/GraphMiner/src/count/omp_base.cc:5-58
// with cpu_kernels/diamond.h:1-8, rectangle.h:1-46 and tailedtriangle.h:1-12; GPU
// analogues codes/GraphMiner/src/count/gpu_base.cu:1-104.
//
//  diamond        = sum over undirected edges e of C(n_e, 2), n_e = |N(u) & N(v)| =
//                   number of triangles containing e.
//  tailed triangle = sum over v with deg(v) > 2 of t(v) * (deg(v) - 2), t(v) = number
//                   of triangles containing v.
//  4-cycle        = for every v0, wedges v0-v1-v2 with v1 < v0 and v2 < v0 grouped by
//                   v2; a group of c wedges closes C(c, 2) cycles.
// n_e and t(v) come from one triangle-participation pass of the DAG kernels
// (clique.cu); the 4-cycle plan has its own kernel below.  Any total order of the
// vertices gives the same counts, so rank ids serve for the "v1 < v0" restrictions.
#include "clique.cuh"
#include "motif.cuh"

namespace xgm {

namespace {

constexpr int kThreads = 256;

__global__ void k_diamond_reduce(const unsigned* epart, int64_t ne, unsigned long long* out) {
  unsigned long long acc = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long n = epart[e];
    acc += n * (n - (n > 0)) / 2;
  }
  acc = warp_sum_u64(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

__global__ void k_tailed_reduce(const unsigned long long* vpart, const int64_t* rowptr, int64_t nv,
                                unsigned long long* out) {
  unsigned long long acc = 0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nv;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t d = rowptr[r + 1] - rowptr[r];
    if (d > 2) acc += vpart[r] * (unsigned long long)(d - 2);
  }
  acc = warp_sum_u64(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// C(d, 3) in wrapping uint64 arithmetic without an intermediate overflow for d < 2^32:
// 3 divides one of d, d-1, d-2; when it does not divide x = d(d-1)/2 it divides d-2.
__device__ __forceinline__ unsigned long long choose3(unsigned long long d) {
  if (d < 3) return 0;
  const unsigned long long x = d * (d - 1) / 2;
  return x % 3 == 0 ? (x / 3) * (d - 2) : x * ((d - 2) / 3);
}

// The sums behind the motif identities, one warp per vertex (lane 0: vertex terms;
// lanes stride the out-neighbours for the edge terms), wrapping uint64:
//   out[0] = sum_v C(d_v, 2)                 edge-induced wedges
//   out[1] = sum_v C(d_v, 3)                 edge-induced 3-stars
//   out[2] = sum_{uv in E} (d_u-1)(d_v-1)    3-edge walks x-u-v-y, x != v, y != u
//   out[3] = sum_v t_v (d_v - 2)             edge-induced tailed triangles
//   out[4] = sum_{uv in E} C(t_uv, 2)        edge-induced diamonds
//   out[5] = sum_v t_v                       3 x triangles
// t_v / t_uv are the triangle-participation counters (vpart / epart, null for the
// 3-vertex census: out[3..5] stay 0).
__global__ void __launch_bounds__(kThreads) k_motif_terms(GView g, const unsigned long long* vpart,
                                                          const unsigned* epart,
                                                          unsigned long long* out) {
  const int lane = threadIdx.x & 31;
  unsigned long long acc[6] = {0, 0, 0, 0, 0, 0};
  const int64_t nwarps = (int64_t)gridDim.x * (kThreads / 32);
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < g.nv; r += nwarps) {
    const unsigned long long d = (unsigned long long)(g.rowptr[r + 1] - g.rowptr[r]);
    if (lane == 0) {
      acc[0] += d * (d - (d > 0)) / 2;
      acc[1] += choose3(d);
      if (vpart) {
        const unsigned long long t = vpart[r];
        if (d > 2) acc[3] += t * (d - 2);
        acc[5] += t;
      }
    }
    const longlong2 p = g.dptr[r];
    for (long long j = p.x + lane; j < p.y; j += 32) {
      const int32_t v = ldg_i32(g.col + j);
      const unsigned long long dv = (unsigned long long)(g.rowptr[v + 1] - g.rowptr[v]);
      acc[2] += (d - 1) * (dv - 1);
      if (epart) {
        const unsigned long long n = epart[j];
        acc[4] += n * (n - (n > 0)) / 2;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const unsigned long long w = warp_sum_u64(acc[i]);
    if (lane == 0 && w) atomicAdd(out + i, w);
  }
}

// Entries of row v1 below v0: col[rowptr[v1] .. first index with col >= v0).
__device__ __forceinline__ long long lower_end(const GView& g, int32_t v1, int32_t v0) {
  long long lo = g.rowptr[v1], hi = g.dptr[v1].y;
  while (lo < hi) {
    long long mid = (lo + hi) >> 1;
    if (ldg_i32(g.col + mid) < v0) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// wedges[r] = number of wedges r-v1-v2 with v1, v2 < r.  Warp per vertex.
__global__ void k_wedge_count(GView g, long long* wedges, int hash_half, uint8_t* is_large,
                              uint8_t* is_small) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < g.nv; r += warps) {
    const long long a0 = g.rowptr[r], a1 = g.dptr[r].x;  // lower neighbours
    long long w = 0;
    for (long long e = a0 + lane; e < a1; e += 32) {
      const int32_t v1 = ldg_i32(g.col + e);
      w += lower_end(g, v1, (int32_t)r) - g.rowptr[v1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(kFull, w, o);
    if (lane == 0) {
      wedges[r] = w;
      is_large[r] = w > hash_half;
      is_small[r] = w > 1 && w <= hash_half;
    }
  }
}

__global__ void k_scatter_flags(const uint8_t* flag, const int64_t* pos, int64_t nv, int32_t* out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nv;
       r += (int64_t)gridDim.x * blockDim.x)
    if (flag[r]) out[pos[r]] = (int32_t)r;
}

// ------------------------------------------------------------ 4-cycle kernel
constexpr int kC4Threads = 256;
constexpr int kC4Chunk = 1024;           // lower neighbours handled per chunk
constexpr int kC4Hash = 4096;            // smem hash slots (small tasks)

struct C4Smem {
  long long lb[kC4Chunk];
  int32_t pre[kC4Chunk + 1];
  int32_t hkey[kC4Hash];
  uint32_t hcnt[kC4Hash];
  int32_t wtot[kC4Threads / 32];
  long long task;
};

__device__ __forceinline__ uint32_t c4_slot(int32_t x) {
  return ((uint32_t)x * 2654435761u) >> (32 - 12);
}

// Loads chunk [c0, c0+n) of v0's lower neighbours: lb/pre (prefix of wedge lengths).
__device__ int c4_load_chunk(const GView& g, C4Smem& sm, int32_t v0, long long c0, int n) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // kC4Chunk = 4 * kC4Threads: 4 items per thread
  int len[4];
  int s = 0;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = tid * 4 + t;
    len[t] = 0;
    if (i < n) {
      const int32_t v1 = ldg_i32(g.col + c0 + i);
      const long long b = g.rowptr[v1];
      sm.lb[i] = b;
      len[t] = (int)(lower_end(g, v1, v0) - b);
    }
    s += len[t];
  }
  int inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) sm.wtot[warp] = inc;
  __syncthreads();
  int off = 0, tot = 0;
  for (int w = 0; w < kC4Threads / 32; ++w) {
    if (w < warp) off += sm.wtot[w];
    tot += sm.wtot[w];
  }
  int ex = off + inc - s;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = tid * 4 + t;
    if (i < n) sm.pre[i] = ex;
    ex += len[t];
  }
  if (tid == 0) sm.pre[n] = tot;
  __syncthreads();
  return tot;
}

// Visits the v2 of every wedge of the loaded chunk (flattened, coalesced per row): each
// thread walks k = tid, tid + 256, ... keeping its segment (lower neighbour) in
// registers, with four loads in flight per step.
template <class F>
__device__ __forceinline__ void c4_walk(const GView& g, const C4Smem& sm, int n, int total, F f) {
  const int tid = threadIdx.x;
  if (tid >= total) return;
  int i;
  {
    int lo = 0, hi = n;  // largest i with pre[i] <= tid
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (sm.pre[mid] <= tid) lo = mid; else hi = mid;
    }
    i = lo;
  }
  int seg_end = sm.pre[i + 1];
  long long seg_base = sm.lb[i] - sm.pre[i];
  for (int kb = tid; kb < total; kb += 4 * kC4Threads) {
    int32_t xv[4];
    bool ok[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int k = kb + t * kC4Threads;
      ok[t] = k < total;
      xv[t] = 0;
      if (ok[t]) {
        while (k >= seg_end) {
          ++i;
          seg_end = sm.pre[i + 1];
          seg_base = sm.lb[i] - sm.pre[i];
        }
        xv[t] = ldg_i32(g.col + seg_base + k);
      }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (ok[t]) f(xv[t]);
  }
}

// Persistent CTA kernel.  Large tasks (more wedges than half the smem table) group
// wedges in a per-CTA dense counter array in global memory (`scratch`, nv entries per
// CTA, kept zeroed: each group is read back with atomicExch); small tasks use an
// open-addressing table in shared memory.
__global__ void __launch_bounds__(kC4Threads) k_cycle4(GView g, const int32_t* large,
                                                       const int32_t* small, const int64_t* n,
                                                       unsigned long long* heads,
                                                       uint32_t* scratch,
                                                       unsigned long long* out, uint32_t* err,
                                                       GOut o) {
  __shared__ C4Smem sm;
  const int tid = threadIdx.x;
  uint32_t* cnt = scratch + (size_t)blockIdx.x * (size_t)g.nv;
  unsigned long long acc = 0;
  const long long n_large = n[0], n_small = n[1];
  for (int phase = 0; phase < 2; ++phase) {
    const int32_t* list = phase ? small : large;
    const long long nt = phase ? n_small : n_large;
    for (;;) {
      if (tid == 0) sm.task = (long long)atomicAdd(&heads[phase], 1ull);
      __syncthreads();
      const long long ti = sm.task;
      __syncthreads();
      if (ti >= nt) break;
      const int32_t v0 = list[ti];
      const long long a0 = g.rowptr[v0], a1 = g.dptr[v0].x;
      unsigned long long tacc = 0;
      if (phase == 1)
        for (int h = tid; h < kC4Hash; h += kC4Threads) sm.hkey[h] = -1, sm.hcnt[h] = 0;
      __syncthreads();
      for (int pass = 0; pass < (phase ? 1 : 2); ++pass) {
        for (long long c0 = a0; c0 < a1; c0 += kC4Chunk) {
          const int nc = (int)min((long long)kC4Chunk, a1 - c0);
          const int total = c4_load_chunk(g, sm, v0, c0, nc);
          if (phase == 0 && pass == 0) {
            c4_walk(g, sm, nc, total, [&](int32_t v2) { atomicAdd(&cnt[v2], 1u); });
          } else if (phase == 0) {
            c4_walk(g, sm, nc, total, [&](int32_t v2) {
              unsigned long long c = atomicExch(&cnt[v2], 0u);
              tacc += c * (c - (c > 0)) / 2;
            });
          } else {
            c4_walk(g, sm, nc, total, [&](int32_t v2) {
              uint32_t slot = c4_slot(v2);
              for (int probe = 0; probe < kC4Hash; ++probe) {
                int32_t k = atomicCAS(&sm.hkey[slot], -1, v2);
                if (k == -1 || k == v2) {
                  atomicAdd(&sm.hcnt[slot], 1u);
                  return;
                }
                slot = (slot + 1) & (kC4Hash - 1);
              }
              atomicOr(err, ERR_CAPACITY);
            });
          }
          __syncthreads();
        }
        __syncthreads();
      }
      if (phase == 1) {
        for (int h = tid; h < kC4Hash; h += kC4Threads) {
          unsigned long long c = sm.hcnt[h];
          tacc += c * (c - (c > 0)) / 2;
        }
        __syncthreads();
      }
      if (o.gid) {
        const unsigned long long w = warp_sum_u64(tacc);
        if ((tid & 31) == 0 && w)
          atomicAdd(&o.out[(long long)o.gid[v0] * o.stride + o.slot], w);
      } else {
        acc += tacc;
      }
    }
  }
  acc = warp_sum_u64(acc);
  if ((tid & 31) == 0 && acc && out) atomicAdd(out, acc);
}

// ---------------------------------------------- 4-cycle, grouped dense tasks
// Tasks with many wedges relative to their id range (v2 < v0) are counted a group at a
// time by the whole GPU: each task of the group owns v0 counters of one L2-resident
// array (the group's ranges add up to at most kC4GroupCounters), every wedge adds one
// to counter v2 of its task, and the count grows by the counter's old value (the k-th
// wedge into a group closes k-1 new cycles, so the sum of old values is C(c, 2) per
// group) — one pass, no read-back; the host clears the array between groups.
// Segments: one per (task, lower neighbour v1), the part of N(v1) below v0.
__global__ void k_c4_segments(GView g, const int32_t* tv0, const int64_t* tseg,
                              const int64_t* tcnt, int m, int64_t nseg, int64_t* seg_base,
                              int64_t* seg_len, int32_t* seg_cnt) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nseg;
       e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = m;  // task t with tseg[t] <= e < tseg[t+1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (tseg[mid] <= e) lo = mid; else hi = mid;
    }
    const int32_t v0 = tv0[lo];
    const int32_t v1 = ldg_i32(g.col + g.rowptr[v0] + (e - tseg[lo]));
    const long long b = g.rowptr[v1];
    seg_base[e] = b;
    seg_len[e] = lower_end(g, v1, v0) - b;
    seg_cnt[e] = (int32_t)tcnt[lo];
  }
}

__global__ void k_c4_task_info(GView g, const int32_t* list, int64_t n, const long long* wedges,
                               int64_t* info) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = list[t];
    info[2 * t] = wedges[r];
    info[2 * t + 1] = g.dptr[r].x - g.rowptr[r];
  }
}

constexpr int kC4TileIters = 16;  // a warp walks 32 x 16 consecutive wedges per tile

__global__ void __launch_bounds__(kThreads) k_c4_dense_walk(const int32_t* col,
                                                            const int64_t* seg_pre,
                                                            const int64_t* seg_base,
                                                            const int32_t* seg_cnt, int64_t nseg,
                                                            uint32_t* counters,
                                                            unsigned long long* out, int clear) {
  const int lane = threadIdx.x & 31;
  // seg_pre holds a prefix over a larger segment set: wedges of this call are
  // [seg_pre[0], seg_pre[nseg]), indexed here from 0
  const int64_t base = seg_pre[0];
  const int64_t total = seg_pre[nseg] - base;
  const int64_t tile = 32 * kC4TileIters;
  const int64_t nwarps = (int64_t)gridDim.x * (kThreads / 32);
  unsigned long long acc = 0;
  for (int64_t t0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * tile; t0 < total;
       t0 += nwarps * tile) {
    // segment of the tile's first wedge (lane 0 searches, the warp shares it)
    int64_t e = 0;
    if (lane == 0) {
      int64_t lo = 0, hi = nseg;  // largest e with seg_pre[e] - base <= t0
      while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (seg_pre[mid] - base <= t0) lo = mid; else hi = mid;
      }
      e = lo;
    }
    e = __shfl_sync(kFull, e, 0);
    int64_t seg_end = seg_pre[e + 1] - base;
    for (int j = 0; j < kC4TileIters; ++j) {
      const int64_t k = t0 + j * 32 + lane;
      if (k >= total) break;
      while (k >= seg_end) {
        ++e;
        seg_end = seg_pre[e + 1] - base;
      }
      const int32_t v2 = ldg_i32(col + seg_base[e] + (k - (seg_pre[e] - base)));
      if (clear) counters[(int64_t)seg_cnt[e] + v2] = 0u;  // second walk: reset what it touched
      else acc += atomicAdd(&counters[(int64_t)seg_cnt[e] + v2], 1u);
    }
  }
  acc = warp_sum_u64(acc);
  if (lane == 0 && acc) atomicAdd(out, acc);
}

// Per-graph diamond / tailed-triangle totals from the participation counters: block
// of consecutive rank ids (graphs are contiguous in rank order), shared-memory
// aggregation by graph id, then one atomic per (block, graph).
__global__ void k_part_reduce_graphs(GView g, const int32_t* gid,
                                     const unsigned long long* vpart, const unsigned* epart,
                                     unsigned long long* out, int stride, int slot_d, int slot_t) {
  __shared__ unsigned long long sd[kThreads], st[kThreads];
  __shared__ int32_t gfirst;
  for (int64_t base = (int64_t)blockIdx.x * kThreads; base < g.nv;
       base += (int64_t)gridDim.x * kThreads) {
    sd[threadIdx.x] = 0;
    st[threadIdx.x] = 0;
    if (threadIdx.x == 0) gfirst = gid[base];
    __syncthreads();
    const int64_t r = base + threadIdx.x;
    if (r < g.nv) {
      const longlong2 d = g.dptr[r];
      const long long deg = d.y - g.rowptr[r];
      unsigned long long dia = 0;
      if (slot_d >= 0)
        for (long long e = d.x; e < d.y; ++e) {
          const unsigned long long c = epart[e];
          dia += c * (c - (c > 0)) / 2;
        }
      const unsigned long long tt = (slot_t >= 0 && deg > 2) ? vpart[r] * (unsigned long long)(deg - 2) : 0;
      const int k = gid[r] - gfirst;  // < kThreads: ids are non-decreasing in rank order
      if (dia) atomicAdd(&sd[k], dia);
      if (tt) atomicAdd(&st[k], tt);
    }
    __syncthreads();
    const long long gg = (long long)gfirst + threadIdx.x;
    if (slot_d >= 0 && sd[threadIdx.x]) atomicAdd(&out[gg * stride + slot_d], sd[threadIdx.x]);
    if (slot_t >= 0 && st[threadIdx.x]) atomicAdd(&out[gg * stride + slot_t], st[threadIdx.x]);
    __syncthreads();
  }
}

inline unsigned grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, int64_t(1) << 20));
}

}  // namespace

cudaError_t launch_diamond_reduce(const unsigned* epart, int64_t ne, unsigned long long* out,
                                  cudaStream_t s) {
  k_diamond_reduce<<<grid_for(ne), kThreads, 0, s>>>(epart, ne, out);
  return cudaGetLastError();
}

cudaError_t launch_tailed_reduce(const unsigned long long* vpart, const int64_t* rowptr, int64_t nv,
                                 unsigned long long* out, cudaStream_t s) {
  k_tailed_reduce<<<grid_for(nv), kThreads, 0, s>>>(vpart, rowptr, nv, out);
  return cudaGetLastError();
}

cudaError_t launch_motif_terms(const GView& g, const unsigned long long* vpart,
                               const unsigned* epart, unsigned long long* out, cudaStream_t s) {
  if (g.nv == 0) return cudaSuccess;
  k_motif_terms<<<grid_for(g.nv * 32), kThreads, 0, s>>>(g, vpart, epart, out);
  return cudaGetLastError();
}

int cycle4_grid(int num_sms) { return 4 * num_sms; }
int cycle4_hash_half() { return kC4Hash / 2; }

cudaError_t launch_wedge_count(const GView& g, long long* wedges, uint8_t* is_large,
                               uint8_t* is_small, cudaStream_t s) {
  if (g.nv == 0) return cudaSuccess;
  k_wedge_count<<<grid_for(g.nv * 32), kThreads, 0, s>>>(g, wedges, kC4Hash / 2, is_large,
                                                         is_small);
  return cudaGetLastError();
}

cudaError_t launch_scatter_flags(const uint8_t* flag, const int64_t* pos, int64_t nv, int32_t* out,
                                 cudaStream_t s) {
  if (nv == 0) return cudaSuccess;
  k_scatter_flags<<<grid_for(nv), kThreads, 0, s>>>(flag, pos, nv, out);
  return cudaGetLastError();
}

cudaError_t launch_cycle4(const GView& g, const int32_t* large, const int32_t* small,
                          const int64_t* n, unsigned long long* heads, uint32_t* scratch,
                          unsigned long long* out, uint32_t* err, int grid, cudaStream_t s,
                          const GOut& o) {
  k_cycle4<<<grid, kC4Threads, 0, s>>>(g, large, small, n, heads, scratch, out, err, o);
  return cudaGetLastError();
}

cudaError_t launch_c4_segments(const GView& g, const int32_t* tv0, const int64_t* tseg,
                               const int64_t* tcnt, int m, int64_t nseg, int64_t* seg_base,
                               int64_t* seg_len, int32_t* seg_cnt, cudaStream_t s) {
  if (nseg == 0) return cudaSuccess;
  k_c4_segments<<<grid_for(nseg), kThreads, 0, s>>>(g, tv0, tseg, tcnt, m, nseg, seg_base,
                                                    seg_len, seg_cnt);
  return cudaGetLastError();
}

cudaError_t launch_c4_task_info(const GView& g, const int32_t* list, int64_t n,
                                const long long* wedges, int64_t* info, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_c4_task_info<<<grid_for(n), kThreads, 0, s>>>(g, list, n, wedges, info);
  return cudaGetLastError();
}

cudaError_t launch_c4_dense_walk(const int32_t* col, const int64_t* seg_pre,
                                 const int64_t* seg_base, const int32_t* seg_cnt, int64_t nseg,
                                 uint32_t* counters, unsigned long long* out, int grid,
                                 cudaStream_t s, bool clear) {
  if (nseg == 0) return cudaSuccess;
  k_c4_dense_walk<<<grid, kThreads, 0, s>>>(col, seg_pre, seg_base, seg_cnt, nseg, counters, out,
                                            clear ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_part_reduce_graphs(const GView& g, const int32_t* gid,
                                      const unsigned long long* vpart, const unsigned* epart,
                                      unsigned long long* out, int stride, int slot_d, int slot_t,
                                      cudaStream_t s) {
  if (g.nv == 0) return cudaSuccess;
  k_part_reduce_graphs<<<grid_for(g.nv), kThreads, 0, s>>>(g, gid, vpart, epart, out, stride,
                                                           slot_d, slot_t);
  return cudaGetLastError();
}

}  // namespace xgm

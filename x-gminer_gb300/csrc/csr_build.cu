// GPU CSR build and degree orientation.
//
// Reference behaviour being replaced:
//  - scripts/graph_format_conversion.py:20-44 symmetrises and sorts edge lists offline
//    (no dedupe, no self-loop removal); here the same runs on the GPU with dedupe and
//    self-loop removal, as the benchmark graphs require.
//  - Graph_V2::orientation, xgminer/src/graph_v2.cpp:243-289 (= GraphMiner
//    src/common/graph.cc:233-275): keep u->v iff deg(v) > deg(u) or (equal and v > u).
//    Here vertices are ranked by (degree, id); the kept edges are exactly those with
//    rank(v) > rank(u), i.e. the upper part of each row once rows are sorted by rank.
//  - Graph::init_edgelist, graph.cc:295-330: the COO task list is not materialised;
//    tasks are generated from the rank-space rows by the scheduler.
#include <algorithm>
#include <vector>

#include "graph.cuh"
#include "prim.cuh"

namespace xgm {

int bits_for(int64_t n) {
  int b = 1;
  while ((int64_t(1) << b) < n) ++b;
  return b;
}

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int threads = kThreads) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > (int64_t(1) << 20)) g = int64_t(1) << 20;
  return (unsigned)g;
}

__global__ void k_make_keys(const int32_t* src, const int32_t* dst, int64_t m, int64_t nv, int vb,
                            int flags, uint64_t* keys, uint32_t* err) {
  const bool sym = flags & XGM_BUILD_SYMMETRIZE;
  const bool noself = flags & XGM_BUILD_DROP_SELF;
  const uint64_t inv = (1ull << (2 * vb)) - 1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    int32_t u = src[i], v = dst[i];
    uint64_t k1, k2;
    if (u < 0 || u >= nv || v < 0 || v >= nv) {
      atomicOr(err, ERR_BOUNDS);
      k1 = k2 = inv;
    } else if (noself && u == v) {
      k1 = k2 = inv;
    } else {
      k1 = ((uint64_t)u << vb) | (uint64_t)v;
      k2 = ((uint64_t)v << vb) | (uint64_t)u;
    }
    if (sym) {
      keys[2 * i] = k1;
      keys[2 * i + 1] = k2;
    } else {
      keys[i] = k1;
    }
  }
}

__global__ void k_keep_flags(const uint64_t* keys, int64_t n, uint64_t inv, bool noself,
                             bool dedup, uint8_t* keep) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t k = keys[i];
    bool ok = !(noself && k == inv);
    if (ok && dedup && i > 0 && keys[i - 1] == k) ok = false;
    keep[i] = ok ? 1 : 0;
  }
}

__global__ void k_compact(const uint64_t* keys, const uint8_t* keep, const int64_t* pos, int64_t n,
                          int vb, int32_t* col, int32_t* rows) {
  const uint64_t vmask = (1ull << vb) - 1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (keep[i]) {
      uint64_t k = keys[i];
      col[pos[i]] = (int32_t)(k & vmask);
      rows[pos[i]] = (int32_t)(k >> vb);
    }
  }
}

// rowptr[r] = first position whose row id is >= r (rows sorted ascending).
__global__ void k_row_bounds(const int32_t* rows, int64_t ne, int64_t nv, int64_t* rowptr) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < ne;
       p += (int64_t)gridDim.x * blockDim.x) {
    int64_t u = rows[p];
    int64_t prev = p ? rows[p - 1] : -1;
    for (int64_t r = prev + 1; r <= u; ++r) rowptr[r] = p;
    if (p == ne - 1)
      for (int64_t r = u + 1; r <= nv; ++r) rowptr[r] = ne;
  }
}

__global__ void k_degrees(const int64_t* rowptr, int64_t nv, int32_t* deg,
                          unsigned long long* maxdeg) {
  int64_t local = 0;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x) {
    int64_t d = rowptr[v + 1] - rowptr[v];
    deg[v] = (int32_t)d;
    local = d > local ? d : local;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    int64_t y = __shfl_down_sync(kFull, local, o);
    local = y > local ? y : local;
  }
  if ((threadIdx.x & 31) == 0 && local > 0) atomicMax(maxdeg, (unsigned long long)local);
}

__global__ void k_rank_keys(const int32_t* deg, const int32_t* group, int64_t nv, int vb, int db,
                            uint64_t* keys) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x) {
    uint64_t k = ((uint64_t)deg[v] << vb) | (uint64_t)v;
    if (group) k |= (uint64_t)group[v] << (vb + db);
    keys[v] = k;
  }
}

__global__ void k_rank_from_sorted(const uint64_t* keys, const int32_t* deg, int64_t nv, int vb,
                                   int db, bool grouped, int32_t* perm, int32_t* rank,
                                   int32_t* degp, int32_t* gid) {
  const uint64_t vmask = (1ull << vb) - 1;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nv;
       r += (int64_t)gridDim.x * blockDim.x) {
    uint64_t k = keys[r];
    int32_t v = (int32_t)(k & vmask);
    perm[r] = v;
    rank[v] = (int32_t)r;
    degp[r] = deg[v];
    if (grouped) gid[r] = (int32_t)(k >> (vb + db));
  }
}

// Warp per rank-space row r (original row x = perm[r]): the entries y of x as keys
// (rank[y] << vb) | r, written at row r of the rank-space layout (sequential writes
// across the grid), so the key sequence is ordered by r.  By symmetry these are all the
// rank-space entries with row and column swapped; a stable sort on the row bits alone
// (bits [vb, 2 vb)) then leaves every row's columns sorted — half the radix passes of
// sorting (row, column) keys from scratch.
// A warp takes 32 consecutive new rows at once: lane i fetches row i's source and
// destination, then the lanes walk the 32 rows' entries as one flat range (each entry
// finds its row by a 5-step search over the lanes' prefix of lengths), so short rows
// keep every lane busy and the rows' loads overlap.  Rows longer than kLongRow (the
// hubs, which rank order puts together at the end) are listed in `longs` (count in
// nlong) for k_rank_entry_keys_long.
constexpr int64_t kLongRow = 1024;
constexpr int kLongSplit = 16;  // blocks per long row

__global__ void k_rank_entry_keys(const int64_t* rowptr_o, const int32_t* col_o,
                                  const int32_t* rank, const int32_t* perm,
                                  const int64_t* rowptr_r, int64_t nv, int vb, uint64_t* keys,
                                  int32_t* longs, unsigned long long* nlong) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * 32; r0 < nv;
       r0 += warps * 32) {
    const int64_t r = r0 + lane;
    int64_t src = 0, dst = 0, len = 0;
    if (r < nv) {
      dst = rowptr_r[r];
      len = rowptr_r[r + 1] - dst;
      if (len > kLongRow) {
        longs[atomicAdd(nlong, 1ull)] = (int32_t)r;
        len = 0;
      } else {
        src = rowptr_o[perm[r]];
      }
    }
    int64_t incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int64_t total = __shfl_sync(0xffffffffu, incl, 31);
    const int64_t excl = incl - len;
    for (int64_t b = 0; b < total; b += 32) {
      const int64_t t = b + lane;
      int k = 0;  // last row whose first flat index is <= t
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int64_t ex = __shfl_sync(0xffffffffu, excl, k + step);
        if (ex <= t) k += step;
      }
      const int64_t ks = __shfl_sync(0xffffffffu, src, k);
      const int64_t kd = __shfl_sync(0xffffffffu, dst, k);
      const int64_t kx = __shfl_sync(0xffffffffu, excl, k);
      if (t < total) {
        const int64_t j = t - kx;
        keys[kd + j] = ((uint64_t)rank[col_o[ks + j]] << vb) | (uint64_t)(r0 + k);
      }
    }
  }
}

// The listed long rows: kLongSplit blocks per row (blockIdx.y), each one slice of the
// row's entries, its threads striding the slice.
__global__ void k_rank_entry_keys_long(const int64_t* rowptr_o, const int32_t* col_o,
                                       const int32_t* rank, const int32_t* perm,
                                       const int64_t* rowptr_r, const int32_t* longs,
                                       const unsigned long long* nlong, int vb,
                                       uint64_t* keys) {
  const int64_t n = (int64_t)*nlong;
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    const int64_t r = longs[i];
    const int64_t dst = rowptr_r[r], len = rowptr_r[r + 1] - dst;
    const int64_t src = rowptr_o[perm[r]];
    const int64_t lo = len * blockIdx.y / gridDim.y, hi = len * (blockIdx.y + 1) / gridDim.y;
    for (int64_t j = lo + threadIdx.x; j < hi; j += blockDim.x)
      keys[dst + j] = ((uint64_t)rank[col_o[src + j]] << vb) | (uint64_t)r;
  }
}

__global__ void k_extract_col(const uint64_t* keys, int64_t ne, int vb, int32_t* col) {
  const uint64_t vmask = (1ull << vb) - 1;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne;
       e += (int64_t)gridDim.x * blockDim.x)
    col[e] = (int32_t)(keys[e] & vmask);
}

// dptr[r] = {first entry of row r with id > r, row end}; stats of the DAG.
__global__ void k_dptr(const int64_t* rowptr, const int32_t* col, int64_t nv, longlong2* dptr,
                       unsigned long long* max_out, unsigned long long* ne_dag) {
  int64_t mo = 0;
  unsigned long long sum = 0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nv;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = rowptr[r], hi = rowptr[r + 1];
    int64_t a = lo, b = hi;  // first index with col > r
    while (a < b) {
      int64_t mid = (a + b) >> 1;
      if (col[mid] > r) b = mid; else a = mid + 1;
    }
    dptr[r] = make_longlong2(a, hi);
    int64_t d = hi - a;
    mo = d > mo ? d : mo;
    sum += (unsigned long long)d;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    int64_t y = __shfl_down_sync(kFull, mo, o);
    mo = y > mo ? y : mo;
    sum += __shfl_down_sync(kFull, sum, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (mo > 0) atomicMax(max_out, (unsigned long long)mo);
    if (sum) atomicAdd(ne_dag, sum);
  }
}

__global__ void k_dag_count(const int64_t* rowptr_o, const int32_t* col_o, const int32_t* rank,
                            int64_t nv, int32_t* cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < nv; u += warps) {
    const int32_t ru = rank[u];
    int c = 0;
    for (int64_t e = rowptr_o[u] + lane; e < rowptr_o[u + 1]; e += 32) c += rank[col_o[e]] > ru;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(kFull, c, o);
    if (lane == 0) cnt[u] = c;
  }
}

__global__ void k_dag_write(const int64_t* rowptr_o, const int32_t* col_o, const int32_t* rank,
                            int64_t nv, const int64_t* drow, int32_t* dcol) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < nv; u += warps) {
    const int32_t ru = rank[u];
    int64_t out = drow[u];
    const int64_t lo = rowptr_o[u], hi = rowptr_o[u + 1];
    for (int64_t base = lo; base < hi; base += 32) {
      int64_t e = base + lane;
      int32_t v = e < hi ? col_o[e] : 0;
      bool keep = e < hi && rank[v] > ru;
      unsigned b = __ballot_sync(kFull, keep);
      if (keep) dcol[out + __popc(b & lanemask_lt())] = v;
      out += __popc(b);
    }
  }
}

__global__ void k_validate(const int64_t* rowptr, const int32_t* col, int64_t nv, int64_t ne,
                           uint32_t* err) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < nv; u += warps) {
    const int64_t lo = rowptr[u], hi = rowptr[u + 1];
    bool bad = lo > hi || lo < 0 || hi > ne;
    if (!bad) {
      for (int64_t e = lo + lane; e < hi; e += 32) {
        int32_t v = col[e];
        if (v < 0 || v >= nv || v == u || (e > lo && col[e - 1] >= v)) { bad = true; break; }
        // symmetric: u must appear in N(v)
        int64_t a = rowptr[v], b = rowptr[v + 1];
        if (a < 0 || b > ne || a > b) { bad = true; break; }
        while (a < b) {
          int64_t mid = (a + b) >> 1;
          if (col[mid] < u) a = mid + 1; else b = mid;
        }
        if (a >= rowptr[v + 1] || col[a] != u) { bad = true; break; }
      }
    }
    if (__any_sync(kFull, bad) && lane == 0) atomicOr(err, ERR_BOUNDS);
  }
}

template <class T>
cudaError_t dalloc(T** p, int64_t n, cudaStream_t s) {
  return cudaMallocAsync((void**)p, sizeof(T) * (size_t)(n > 0 ? n : 1), s);
}

#define TRY(x)                          \
  do {                                  \
    cudaError_t _e = (x);               \
    if (_e != cudaSuccess) return _e;   \
  } while (0)

}  // namespace

void free_graph(DevGraph& g, cudaStream_t s) {
  void* ps[] = {g.rowptr_o, g.col_o, g.rank, g.perm, g.rowptr, g.col, g.dptr, g.gid,
                g.bcol, g.boff, g.bmask, g.lut_rows, g.lut_off, g.tsum, g.tmax};
  for (void* p : ps)
    if (p) cudaFreeAsync(p, s);
  g = DevGraph{};
}

cudaError_t build_csr_from_samples(int64_t nv, const int32_t* src, const int32_t* dst, int64_t m,
                                   int flags, DevGraph& g, uint32_t* err, cudaStream_t s) {
  const int vb = bits_for(nv);
  const bool sym = flags & XGM_BUILD_SYMMETRIZE;
  const int64_t n = sym ? 2 * m : m;
  uint64_t *keys = nullptr, *tmp = nullptr;
  uint8_t* keep = nullptr;
  int64_t *pos = nullptr, *d_ne = nullptr;
  int32_t* rows = nullptr;
  TRY(dalloc(&keys, n, s));
  TRY(dalloc(&tmp, n, s));
  TRY(dalloc(&keep, n, s));
  TRY(dalloc(&pos, n, s));
  TRY(dalloc(&d_ne, 1, s));
  if (m > 0) {
    k_make_keys<<<grid_for(m), kThreads, 0, s>>>(src, dst, m, nv, vb, flags, keys, err);
    TRY(cudaGetLastError());
  }
  TRY(radix_sort_u64(keys, tmp, n, 2 * vb, s));
  const uint64_t inv = (1ull << (2 * vb)) - 1;
  if (n > 0) {
    k_keep_flags<<<grid_for(n), kThreads, 0, s>>>(keys, n, inv, flags & XGM_BUILD_DROP_SELF,
                                                  flags & XGM_BUILD_DEDUP, keep);
    TRY(cudaGetLastError());
  }
  TRY(scan_excl(keep, pos, n, d_ne, s));
  int64_t ne = 0;
  TRY(cudaMemcpyAsync(&ne, d_ne, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  TRY(cudaStreamSynchronize(s));
  g.nv = nv;
  g.ne = ne;
  TRY(dalloc(&g.rowptr_o, nv + 1, s));
  TRY(dalloc(&g.col_o, ne, s));
  TRY(dalloc(&rows, ne, s));
  if (n > 0) {
    k_compact<<<grid_for(n), kThreads, 0, s>>>(keys, keep, pos, n, vb, g.col_o, rows);
    TRY(cudaGetLastError());
  }
  if (ne > 0) {
    k_row_bounds<<<grid_for(ne), kThreads, 0, s>>>(rows, ne, nv, g.rowptr_o);
    TRY(cudaGetLastError());
  } else {
    TRY(cudaMemsetAsync(g.rowptr_o, 0, sizeof(int64_t) * (nv + 1), s));
  }
  cudaFreeAsync(keys, s);
  cudaFreeAsync(tmp, s);
  cudaFreeAsync(keep, s);
  cudaFreeAsync(pos, s);
  cudaFreeAsync(d_ne, s);
  cudaFreeAsync(rows, s);
  return cudaSuccess;
}

cudaError_t validate_csr(const DevGraph& g, uint32_t* err, cudaStream_t s) {
  if (g.nv == 0) return cudaSuccess;
  k_validate<<<grid_for(g.nv * 32), kThreads, 0, s>>>(g.rowptr_o, g.col_o, g.nv, g.ne, err);
  return cudaGetLastError();
}

cudaError_t finish_graph(DevGraph& g, const int32_t* group, int num_groups, cudaStream_t s) {
  const int64_t nv = g.nv, ne = g.ne;
  const int vb = bits_for(nv);
  int32_t *deg = nullptr, *degp = nullptr;
  unsigned long long* stats = nullptr;  // [0] max deg, [1] max out, [2] ne_dag, [3] long rows
  TRY(dalloc(&deg, nv, s));
  TRY(dalloc(&degp, nv, s));
  TRY(dalloc(&stats, 4, s));
  TRY(cudaMemsetAsync(stats, 0, 4 * sizeof(unsigned long long), s));
  if (nv > 0) {
    k_degrees<<<grid_for(nv), kThreads, 0, s>>>(g.rowptr_o, nv, deg, stats);
    TRY(cudaGetLastError());
  }
  unsigned long long h[3] = {0, 0, 0};
  TRY(cudaMemcpyAsync(h, stats, sizeof(h), cudaMemcpyDeviceToHost, s));
  TRY(cudaStreamSynchronize(s));
  g.max_deg = (int64_t)h[0];
  const int db = bits_for(g.max_deg + 1);
  const int gb = group ? bits_for(num_groups) : 0;
  if (vb + db + gb > 64) return cudaErrorInvalidValue;
  // the counting kernels pack a list position into 40 bits (clique.cu, count modes)
  if (ne >= (int64_t(1) << 40)) return cudaErrorInvalidValue;

  uint64_t *keys = nullptr, *tmp = nullptr;
  const int64_t nk = std::max(nv, ne);
  TRY(dalloc(&keys, nk, s));
  TRY(dalloc(&tmp, nk, s));
  TRY(dalloc(&g.rank, nv, s));
  TRY(dalloc(&g.perm, nv, s));
  TRY(dalloc(&g.rowptr, nv + 1, s));
  TRY(dalloc(&g.col, ne + 4, s));  // 16 bytes of slack: bulk copies round a list up to 16 B
  TRY(dalloc(&g.dptr, nv, s));
  if (group) TRY(dalloc(&g.gid, nv, s));
  if (nv > 0) {
    k_rank_keys<<<grid_for(nv), kThreads, 0, s>>>(deg, group, nv, vb, db, keys);
    TRY(cudaGetLastError());
  }
  // keys start in id order, so a stable sort on the (group, degree) bits alone gives
  // (group, degree, id) order
  TRY(radix_sort_u64(keys, tmp, nv, db + gb, s, vb));
  if (nv > 0) {
    k_rank_from_sorted<<<grid_for(nv), kThreads, 0, s>>>(keys, deg, nv, vb, db, group != nullptr,
                                                         g.perm, g.rank, degp, g.gid);
    TRY(cudaGetLastError());
  }
  TRY(scan_excl(degp, g.rowptr, nv, g.rowptr + nv, s));
  if (nv > 0) {
    // at most ne / kLongRow rows are long
    const int64_t cap = ne / kLongRow + 1;
    int32_t* longs = nullptr;
    TRY(dalloc(&longs, cap, s));
    TRY(cudaMemsetAsync(stats + 3, 0, sizeof(unsigned long long), s));
    k_rank_entry_keys<<<grid_for(nv), kThreads, 0, s>>>(g.rowptr_o, g.col_o, g.rank, g.perm,
                                                        g.rowptr, nv, vb, keys, longs, stats + 3);
    TRY(cudaGetLastError());
    const dim3 lg((unsigned)std::min<int64_t>(cap, 2048), kLongSplit);
    k_rank_entry_keys_long<<<lg, kThreads, 0, s>>>(g.rowptr_o, g.col_o, g.rank, g.perm, g.rowptr,
                                                   longs, stats + 3, vb, keys);
    TRY(cudaGetLastError());
    cudaFreeAsync(longs, s);
  }
  uint64_t* sorted = keys;
  TRY(radix_sort_u64(keys, tmp, ne, vb, s, vb, &sorted));
  if (ne > 0) {
    k_extract_col<<<grid_for(ne), kThreads, 0, s>>>(sorted, ne, vb, g.col);
    TRY(cudaGetLastError());
  }
  if (nv > 0) {
    k_dptr<<<grid_for(nv), kThreads, 0, s>>>(g.rowptr, g.col, nv, g.dptr, stats + 1, stats + 2);
    TRY(cudaGetLastError());
  }
  TRY(cudaMemcpyAsync(h, stats, sizeof(h), cudaMemcpyDeviceToHost, s));
  TRY(cudaStreamSynchronize(s));
  g.max_out = (int64_t)h[1];
  g.ne_dag = (int64_t)h[2];
  cudaFreeAsync(keys, s);
  cudaFreeAsync(tmp, s);
  cudaFreeAsync(deg, s);
  cudaFreeAsync(degp, s);
  cudaFreeAsync(stats, s);
  return cudaSuccess;
}

cudaError_t dag_original(const DevGraph& g, int64_t** rowptr, int32_t** col, cudaStream_t s) {
  int32_t* cnt = nullptr;
  TRY(dalloc(&cnt, g.nv, s));
  TRY(dalloc(rowptr, g.nv + 1, s));
  TRY(dalloc(col, g.ne_dag, s));
  if (g.nv > 0) {
    k_dag_count<<<grid_for(g.nv * 32), kThreads, 0, s>>>(g.rowptr_o, g.col_o, g.rank, g.nv, cnt);
    TRY(cudaGetLastError());
  }
  TRY(scan_excl(cnt, *rowptr, g.nv, *rowptr + g.nv, s));
  if (g.nv > 0) {
    k_dag_write<<<grid_for(g.nv * 32), kThreads, 0, s>>>(g.rowptr_o, g.col_o, g.rank, g.nv,
                                                         *rowptr, *col);
    TRY(cudaGetLastError());
  }
  cudaFreeAsync(cnt, s);
  return cudaSuccess;
}

}  // namespace xgm

// Device graph storage and the GPU CSR build (csr_build.cu).
#pragma once
#include "common.cuh"

namespace xgm {

// Device-resident graph.  Two id spaces:
//  - original ids: the undirected CSR exactly as loaded / built (rowptr_o, col_o);
//  - rank ids: vertices renumbered by (degree, id), so the reference's orientation
//    rule (graph.cc:247-249) reads rank(v) > rank(u).  Rows are re-sorted in rank ids;
//    the counting kernels only read this space.
struct DevGraph {
  int64_t nv = 0;
  int64_t ne = 0;          // undirected CSR entries
  int64_t ne_dag = 0;      // entries kept by the orientation (= ne / 2)
  int64_t max_deg = 0;
  int64_t max_out = 0;     // max out-degree of the oriented DAG
  int64_t* rowptr_o = nullptr;
  int32_t* col_o = nullptr;
  int32_t* rank = nullptr;   // [nv] original -> rank
  int32_t* perm = nullptr;   // [nv] rank -> original
  int64_t* rowptr = nullptr; // [nv+1] rank space
  int32_t* col = nullptr;    // [ne] rank space, sorted rows
  longlong2* dptr = nullptr; // [nv] {first out-neighbour, row end}
  int32_t* gid = nullptr;    // [nv] rank -> graph id (batched graphs only)
  // bucket index (GView), built on first use by a schedule that can pick BUCKET
  mutable int32_t* bcol = nullptr;
  mutable uint32_t* boff = nullptr;
  mutable uint16_t* bmask = nullptr;
  // adjacency rows among N(v) for v of degree 33..1024 (setprog.cu), built on first use
  // by a set-operation program: lut_off[v] words into lut_rows; lut_state 1 built,
  // -1 not built (too large)
  mutable uint32_t* lut_rows = nullptr;
  mutable int64_t* lut_off = nullptr;
  mutable int lut_state = 0;
  // out-neighbour degree sums / maxima (the learned schedule's task features), built on
  // first use by the learned schedule
  mutable int64_t* tsum = nullptr;
  mutable int32_t* tmax = nullptr;

  GView view() const { return GView{col, rowptr, dptr, nv, bcol, boff, bmask, tsum, tmax}; }
};

void free_graph(DevGraph& g, cudaStream_t s);

// Builds g's out-neighbour degree sums and maxima once (learned.cu); later calls return
// at once.
cudaError_t ensure_task_stats(const DevGraph& g, cudaStream_t s);

// Builds g's bucket index once (bucket.cu); later calls return at once.
cudaError_t ensure_bucket_index(const DevGraph& g, cudaStream_t s);

// Raw samples on the device -> undirected CSR in original ids (g.rowptr_o/col_o).
// flags: XGM_BUILD_* bits.  err (device) gets ERR_BOUNDS for ids outside [0, nv).
cudaError_t build_csr_from_samples(int64_t nv, const int32_t* src, const int32_t* dst,
                                   int64_t m, int flags, DevGraph& g, uint32_t* err,
                                   cudaStream_t s);

// Checks an uploaded undirected CSR: ids in range, rows strictly increasing (sorted,
// no duplicates), no self-loops, symmetric.  Sets ERR_BOUNDS in err on failure.
cudaError_t validate_csr(const DevGraph& g, uint32_t* err, cudaStream_t s);

// From g.rowptr_o/col_o: degrees, ranks, the rank-space CSR, out-neighbour pointers
// and the size statistics.  `group` (optional, [nv] original ids, values below
// num_groups) keeps vertices of one group contiguous in rank order (batched graphs)
// and fills g.gid.
cudaError_t finish_graph(DevGraph& g, const int32_t* group, int num_groups, cudaStream_t s);

// The oriented DAG in original ids (graph.cc:233-275 output), device arrays
// allocated here; caller frees.
cudaError_t dag_original(const DevGraph& g, int64_t** rowptr, int32_t** col, cudaStream_t s);

int bits_for(int64_t n);  // smallest b with 2^b >= n (>= 1)

}  // namespace xgm

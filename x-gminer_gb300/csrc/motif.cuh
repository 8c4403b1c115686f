// Edge-induced motif plans (motif.cu).
#pragma once
#include <algorithm>

#include "clique.cuh"
#include "common.cuh"

namespace xgm {

cudaError_t launch_diamond_reduce(const unsigned* epart, int64_t ne, unsigned long long* out,
                                  cudaStream_t s);
cudaError_t launch_tailed_reduce(const unsigned long long* vpart, const int64_t* rowptr, int64_t nv,
                                 unsigned long long* out, cudaStream_t s);

// out[0..5] += wedge / 3-star / 3-walk / tailed-triangle / diamond / 3 x triangle sums
// (edge-induced; vpart/epart null for the 3-vertex census).
cudaError_t launch_motif_terms(const GView& g, const unsigned long long* vpart,
                               const unsigned* epart, unsigned long long* out, cudaStream_t s);

// 4-cycle: wedge counts per vertex, then the persistent grouping kernel.
int cycle4_grid(int num_sms);
int cycle4_hash_half();
cudaError_t launch_wedge_count(const GView& g, long long* wedges, uint8_t* is_large,
                               uint8_t* is_small, cudaStream_t s);
cudaError_t launch_scatter_flags(const uint8_t* flag, const int64_t* pos, int64_t nv, int32_t* out,
                                 cudaStream_t s);
// n[0] = large tasks, n[1] = small tasks; heads[0..1] zeroed; scratch = grid * nv
// zeroed uint32 counters (left zeroed on return).
cudaError_t launch_cycle4(const GView& g, const int32_t* large, const int32_t* small,
                          const int64_t* n, unsigned long long* heads, uint32_t* scratch,
                          unsigned long long* out, uint32_t* err, int grid, cudaStream_t s,
                          const GOut& o = GOut{});
// 4-cycle tasks counted a group at a time (see motif.cu): segments of the group's tasks
// (tv0[m] task roots, tseg[m+1] prefix of their lower degrees, tcnt[m] counter offsets),
// then the walk over the scanned segment lengths (seg_pre[nseg+1]).
constexpr int64_t kC4GroupCounters = int64_t(16) << 20;  // 64 MB of counters per group
cudaError_t launch_c4_segments(const GView& g, const int32_t* tv0, const int64_t* tseg,
                               const int64_t* tcnt, int m, int64_t nseg, int64_t* seg_base,
                               int64_t* seg_len, int32_t* seg_cnt, cudaStream_t s);
// clear: walk again and reset the counters the first walk touched (instead of counting)
cudaError_t launch_c4_dense_walk(const int32_t* col, const int64_t* seg_pre,
                                 const int64_t* seg_base, const int32_t* seg_cnt, int64_t nseg,
                                 uint32_t* counters, unsigned long long* out, int grid,
                                 cudaStream_t s, bool clear = false);
// wedges and lower degree of each listed task: info[2t] = wedges, info[2t+1] = lower degree
cudaError_t launch_c4_task_info(const GView& g, const int32_t* list, int64_t n,
                                const long long* wedges, int64_t* info, cudaStream_t s);

// Batched graphs: per-graph diamond (slot_d) and tailed-triangle (slot_t) totals from the
// participation counters; a slot < 0 is skipped.
cudaError_t launch_part_reduce_graphs(const GView& g, const int32_t* gid,
                                      const unsigned long long* vpart, const unsigned* epart,
                                      unsigned long long* out, int stride, int slot_d, int slot_t,
                                      cudaStream_t s);

}  // namespace xgm

// Task generation and scheduling for the clique kernels (sched.cu).
#pragma once
#include "clique.cuh"
#include "graph.cuh"

namespace xgm {

// Variant codes per vertex task (var[]).
enum : uint8_t {
  VAR_WARP = 0, VAR_CTA = 1, VAR_SPLIT = 2, VAR_WIDE = 3, VAR_SEARCH = 4, VAR_BUCKET = 5,
  VAR_GROUP = 6, VAR_SKIP = 7
};
constexpr int kNumVar = 7;
// k_feat code of the batched multi-pattern launch (triangles + 4-cliques + triangle
// participation per task): the learned model's depth feature is 0.75 for it, between
// the 4-clique (0.5) and 5-clique (1.0) tasks, so its timings do not collide with the
// 4-clique count's.
constexpr int kFeatMulti = 16;

// Device buffers of one schedule; sized for a graph's vertex count and reused.
struct TaskBuf {
  int64_t cap_v = 0;
  int32_t* cta = nullptr;
  int32_t* warp = nullptr;
  int32_t* wide = nullptr;
  int32_t* search = nullptr;
  int32_t* bucket = nullptr;
  int32_t* group = nullptr;
  int32_t* split_v = nullptr;
  int64_t* split_off = nullptr;
  int64_t* n = nullptr;       // [9] see TaskLists; n[8] = hubs eligible to run whole
  uint8_t* var = nullptr;     // [cap_v] variant per vertex
  int64_t* w = nullptr;       // [cap_v] scratch
  float* cost = nullptr;      // [cap_v] predicted log-cost (learned policy)
  long long* log = nullptr;   // [6 * cap_v + split cap] per-task timing log (optional)
  int64_t log_cap = 0;
  int hub_max = 0;            // hubs left whole for the hub kernel (TaskLists::hub_max)
  int hash_only = 0;          // TaskLists::hash_only

  TaskLists lists(bool with_log) const;
};

cudaError_t taskbuf_reserve(TaskBuf& tb, int64_t nv, cudaStream_t s);
void taskbuf_free(TaskBuf& tb, cudaStream_t s);

// Plain degree-threshold heuristic (the role of WARP_LIMIT / BLOCK_LIMIT,
// xgminer/include/glumin/common.h:114-116, and the |W| <= 32 switch of
// clique5_warp_edge_taskallocate.cuh:26): out-degree s < k-1 -> skip,
// s <= group_max -> GROUP, s <= bucket_max -> BUCKET, s <= search_max -> SEARCH,
// s <= warp_max -> WARP, s <= wide_max -> WIDE, s <= cta_max -> CTA, else SPLIT
// (group_max, bucket_max and search_max are 0 in the plain heuristic).  Lists keep
// vertex order.
cudaError_t classify_heuristic(const DevGraph& g, int k, int warp_max, int wide_max, int cta_max,
                               TaskBuf& tb, cudaStream_t s, int search_max = 0,
                               int bucket_max = 0, int group_max = 0);

// Variant per out-degree bucket (XGM_SCHED_TUNED); roots with out-degree < kmin skip.
cudaError_t classify_table(const DevGraph& g, int kmin, const xgm_tune_table& tab, TaskBuf& tb,
                           cudaStream_t s);

// Compacts tb.var into the task lists.  With `order` (learned policy) each list is
// ordered by descending tb.cost (binned), heaviest predicted tasks first.  Hubs with
// kCtaCap < out-degree <= hub_max get no sub-tasks (the hub kernel runs them whole).
cudaError_t build_lists(const DevGraph& g, TaskBuf& tb, bool order, cudaStream_t s,
                        int hub_max = 0);

}  // namespace xgm

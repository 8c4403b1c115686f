// Clique / triangle counting on the degree-oriented DAG (clique.cu).
#pragma once
#include "common.cuh"

namespace xgm {

constexpr int kCtaThreads = 512;            // threads of the persistent counting CTA
constexpr int kCtaWarps = kCtaThreads / 32;
constexpr int kCtaCap = 1024;               // largest local set a CTA task holds
constexpr int kHashSize = 4096;             // open-addressing table for the local set
constexpr int kWarpCap = 32;                // largest local set a warp task holds
constexpr int kWideCap = 128;               // largest local set a wide-warp task holds
constexpr int kWideWords = 4;               // bitmap words per row of a wide-warp task
constexpr int kGroupCap = 8;                // largest local set of an eight-lane group task
constexpr int kGroupsPerWarp = 32 / kGroupCap;
constexpr int kHubThreads = 1024;           // threads of the hub kernel's CTA (one per SM)
constexpr int kHubCap = 1536;               // largest local set a hub task holds

// Task lists of one counting launch.  Sizes live on the device (`n`), so task
// generation and counting run without a host round trip and can be graph-captured:
//   n[0] = hub edge sub-tasks, n[1] = CTA vertex tasks, n[2] = warp vertex tasks,
//   n[3] = hub vertices, n[4] = wide-warp vertex tasks, n[5] = binary-search warp tasks,
//   n[6] = bucket-filtered binary-search warp tasks, n[7] = eight-lane group tasks.
// Hub sub-task t belongs to hub split_v[h] with split_off[h] <= t < split_off[h+1];
// its second vertex is the (t - split_off[h])-th out-neighbour of the hub.
// Per-task timing logs (clock64 cycles) are indexed like the lists; any may be null.
struct TaskLists {
  const int32_t* cta = nullptr;    // vertex tasks run by one CTA (out-degree <= kCtaCap)
  const int32_t* warp = nullptr;   // vertex tasks run by one warp (out-degree <= kWarpCap)
  const int32_t* wide = nullptr;   // vertex tasks run by one warp with 4-word rows (<= kWideCap)
  const int32_t* search = nullptr; // warp tasks (<= kWarpCap) built by binary search
  const int32_t* bucket = nullptr; // warp tasks (<= kWarpCap), bucket-filtered search
  const int32_t* group = nullptr;  // tasks run four to a warp (<= kGroupCap)
  const int32_t* split_v = nullptr;
  const int64_t* split_off = nullptr;
  const int64_t* n = nullptr;
  // hubs (split_v) with kCtaCap < out-degree <= hub_max may run whole in the hub kernel:
  // those with no sub-tasks in split_off (split_off[h + 1] == split_off[h]) do (0: every
  // hub is split)
  int hub_max = 0;
  // CTA tasks test membership with the Bloom filter and hash even where the span bitmap
  // fits (xgm_sched XGM_SCHED_HASH_ONLY)
  int hash_only = 0;
  long long* log_cta = nullptr;
  long long* log_warp = nullptr;
  long long* log_split = nullptr;
  long long* log_wide = nullptr;
  long long* log_search = nullptr;
  long long* log_bucket = nullptr;
  long long* log_group = nullptr;
};

// Per-graph outputs of batched launches: task totals go to out[gid[v0] * stride + slot]
// (and slot2 in multi mode).  gid == null: one global total.
struct GOut {
  const int32_t* gid = nullptr;
  unsigned long long* out = nullptr;
  int stride = 0;
  int slot = 0;
  int slot2 = -1;
};

// Work-queue heads, zeroed before each launch.
struct QueueHeads {
  unsigned long long split, cta, warp, wide, search, bucket, group, hub;
};

size_t clique_smem_bytes();
// Resident counting CTAs per SM (dynamic shared memory bound).
cudaError_t clique_occupancy(int* per_sm);

// k in {3, ..., 7}: adds the k-clique count of g (DAG) over the listed tasks to *count;
// with t.hub_max set, a second launch (the hub kernel) counts the whole hubs.
cudaError_t launch_clique(int k, const GView& g, const TaskLists& t, QueueHeads* q,
                          unsigned long long* count, uint32_t* err, int grid, cudaStream_t s,
                          const GOut& o = GOut{});

// Batched multi-pattern launch (4-clique machinery): per task, triangles -> o.slot,
// 4-cliques -> o.slot2 (-1: none), and triangle participation into vpart / epart.
// Tasks must be classified with k = 3 so out-degree-2 roots are included.
cudaError_t launch_multi(const GView& g, const TaskLists& t, QueueHeads* q,
                         unsigned long long* vpart, unsigned* epart, uint32_t* err, int grid,
                         cudaStream_t s, const GOut& o);

// Triangle participation from the same task lists run with k = 3: every triangle adds
// 1 to vpart[] of its three vertices and 1 to epart[] of its three edges (edge = index
// of the entry in the rank-space col array, stored on the lower endpoint).  Feeds the
// tailed-triangle and diamond plans.
cudaError_t launch_triangle_participation(const GView& g, const TaskLists& t, QueueHeads* q,
                                          unsigned long long* vpart, unsigned* epart,
                                          uint32_t* err, int grid, cudaStream_t s);

// Sum over k-cliques (k in {3, 4}) of the out-degree of each clique's highest-ranked
// vertex; gives the W-dependent terms of the plans' algorithmic bytes.
cudaError_t launch_clique_weighted(int k, const GView& g, const TaskLists& t, QueueHeads* q,
                                   unsigned long long* sum, uint32_t* err, int grid,
                                   cudaStream_t s);

int clique_grid(int num_sms);

}  // namespace xgm

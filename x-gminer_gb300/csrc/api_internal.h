// Internal definitions behind the C ABI.
#pragma once
#include <string>

#include "clique.cuh"
#include "graph.cuh"
#include "sched.cuh"
#include "setprog.cuh"

namespace xgm {

// Small device-side scalars of one call, zeroed by one memset and read back by one copy.
struct Scalars {
  unsigned long long count;
  unsigned long long aux;
  uint32_t err;
  uint32_t pad;
  QueueHeads q;
  unsigned long long c4heads[2];
  int64_t n[8];  // task list sizes, copied back for the stats
  unsigned long long terms[6];  // motif-identity sums (launch_motif_terms)
};

struct Model;  // learned cost model (learned.cu)

}  // namespace xgm

struct xgm_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  xgm::Scalars* d_sc = nullptr;
  xgm::Scalars* h_sc = nullptr;  // pinned
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  xgm::TaskBuf tb;
  // motif buffers (grown on demand)
  unsigned long long* vpart = nullptr;
  int64_t vpart_cap = 0;
  unsigned* epart = nullptr;
  int64_t epart_cap = 0;
  uint32_t* c4_scratch = nullptr;
  int64_t c4_scratch_cap = 0;
  long long* wedges = nullptr;
  uint8_t* c4_flag_large = nullptr;
  uint8_t* c4_flag_small = nullptr;
  int64_t* c4_pos = nullptr;
  int32_t* c4_large = nullptr;
  int32_t* c4_small = nullptr;
  int64_t* c4_n = nullptr;
  int64_t c4_vcap = 0;
  // grouped dense 4-cycle tasks (motif.cu): counters (kept zeroed), task info,
  // segment arrays and the groups' task tables
  uint32_t* c4_counters = nullptr;
  int64_t* c4_info = nullptr;
  int64_t c4_info_cap = 0;
  int64_t* c4_seg_base = nullptr;
  int64_t* c4_seg_pre = nullptr;
  int32_t* c4_seg_cnt = nullptr;
  int64_t c4_seg_cap = 0;
  int32_t* c4_tv0 = nullptr;
  int64_t* c4_ttab = nullptr;  // per group: tseg[m+1] then tcnt[m]
  int64_t c4_task_cap = 0;
  int clique_grid = 0;
  // set-operation programs (setprog.cu): per-warp slot scratch, split records, heads
  int32_t* prog_scratch = nullptr;
  int64_t prog_scratch_cap = 0;
  void* prog_split = nullptr;
  unsigned long long* prog_heads = nullptr;
};

struct xgm_graph {
  xgm_ctx* ctx = nullptr;
  xgm::DevGraph g;
};

struct xgm_plan {
  int pattern = 0;
  int induced = 0;     // vertex-induced motif counts (via the motif identities)
  uint64_t scale = 1;  // embeddings per match in the caller's convention (GLUMIN P2: 2)
  xgm::Prog prog;      // XGM_PATTERN_PROGRAM: the set-operation program
};

namespace xgm {

xgm_status finish_status(xgm_ctx* ctx, xgm_status st);
xgm_status check_device_flag(xgm_ctx* ctx, uint32_t flag);
xgm_status ctx_sync_scalars(xgm_ctx* ctx);

// count.cu
xgm_status count_dispatch(xgm_ctx* ctx, const DevGraph& g, int pattern, const xgm_sched& sp,
                          uint64_t* out, xgm_stats& st);
xgm_status algo_bytes_dispatch(xgm_ctx* ctx, const DevGraph& g, int pattern, uint64_t* out);
// One plan (pattern, edge- or vertex-induced), and the k = 3 / k = 4 motif census.
xgm_status count_plan(xgm_ctx* ctx, const DevGraph& g, int pattern, int induced,
                      const xgm_sched& sp, uint64_t* out, xgm_stats& st);
xgm_status count_motifs(xgm_ctx* ctx, const DevGraph& g, int k, const xgm_sched& sp,
                        uint64_t* out, xgm_stats& st);
xgm_status count_kernels(xgm_ctx* ctx, const DevGraph& g, int pattern, const xgm_sched& sp,
                         int* n_kernels);
void motif_buffers_free(xgm_ctx* ctx);
// setprog.cu
xgm_status count_program(xgm_ctx* ctx, const DevGraph& g, const Prog& p, uint64_t* out,
                         xgm_stats& st);
void program_buffers_free(xgm_ctx* ctx);
// k_feat: clique size the learned model's features describe (default k).
// hub: the launch is a clique count that runs the hub kernel (sp.hub_max applies).
xgm_status schedule_into(TaskBuf& tb, const DevGraph& g, int k, const xgm_sched& sp,
                         cudaStream_t s, int k_feat = 0, bool hub = false);
bool sched_may_bucket(const xgm_sched& sp);  // the policy can assign the BUCKET variant
int ensure_clique_grid(xgm_ctx* ctx);
int match_pattern(const xgm_plan_desc* d);  // builtin id, 0 unsupported, -1 malformed
// Builtin id for a pattern name (0 if unknown); GLUMIN ids also set induced / scale.
int pattern_from_name(const char* name, int* induced = nullptr, uint64_t* scale = nullptr);

}  // namespace xgm

// Learned cost model for the scheduler (learned.cu).
#pragma once
#include <cuda_fp16.h>

#include "graph.cuh"
#include "sched.cuh"

namespace xgm {

constexpr int kFeat = XGM_MODEL_FEATURES;
constexpr int kShapeFeat = kFeat - XGM_NUM_VARIANTS;  // task shape + depth; then one-hot
static_assert(kShapeFeat == 5, "features: 4 task-shape values, the clique depth, a variant one-hot");
constexpr int kHidden = XGM_MODEL_HIDDEN;
constexpr int kParams = XGM_MODEL_PARAMS;
constexpr int kOffB1 = kHidden * kFeat;
constexpr int kOffW2 = kOffB1 + kHidden;
constexpr int kOffB2 = kOffW2 + kHidden;

}  // namespace xgm

struct xgm_model {
  xgm_ctx* ctx = nullptr;
  __half* wh = nullptr;    // [kParams] fp16 weights used for inference / forward
  float* master = nullptr; // [kParams] fp32 master copy (training)
  float* m = nullptr;      // Adam first moment
  float* v = nullptr;      // Adam second moment
  long long step = 0;
};

namespace xgm {

// Learned schedule: per vertex task the features, the MLP's predicted log2 warp-cycles
// for each variant the task fits, the chosen variant (tb.var) and its cost (tb.cost).
// Without need_cost (no cost ordering) tasks that fit one variant skip the model.
// margin <= 0: the default margin.  k sets which tasks are skipped (out-degree < k-1);
// k_feat (default k) is the clique size the features describe.
cudaError_t classify_learned(const DevGraph& g, int k, const xgm_model& m, TaskBuf& tb,
                             bool need_cost, float margin, cudaStream_t s, int k_feat = 0);

}  // namespace xgm

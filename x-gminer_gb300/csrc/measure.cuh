// Algorithmic-bytes passes (measure.cu).
#pragma once
#include "common.cuh"

namespace xgm {
cudaError_t launch_bytes_basic(const GView& g, int kind, unsigned long long* out, cudaStream_t s);
cudaError_t launch_sum_ll(const long long* x, int64_t n, unsigned long long* out, cudaStream_t s);
}  // namespace xgm

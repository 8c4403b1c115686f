// Device-wide scan and radix sort (prim.cu).
#pragma once
#include "common.cuh"

namespace xgm {

// Exclusive prefix sum into int64 (in and out may alias).  `total` (device, optional)
// receives the sum of all n inputs.
cudaError_t scan_excl(const int64_t* in, int64_t* out, int64_t n, int64_t* total, cudaStream_t s);
cudaError_t scan_excl(const int32_t* in, int64_t* out, int64_t n, int64_t* total, cudaStream_t s);
cudaError_t scan_excl(const uint8_t* in, int64_t* out, int64_t n, int64_t* total, cudaStream_t s);

// Stable LSD radix sort of keys[0..n) over bits [shift0, shift0 + bits), 8 bits per
// pass; tmp must hold n keys.  The result is left in keys, or, when `where` is given,
// in whichever of keys / tmp the last pass wrote (*where), saving the copy back.
cudaError_t radix_sort_u64(uint64_t* keys, uint64_t* tmp, int64_t n, int bits, cudaStream_t s,
                           int shift0 = 0, uint64_t** where = nullptr);

}  // namespace xgm

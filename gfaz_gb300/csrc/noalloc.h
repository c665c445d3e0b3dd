// Allocation-free inverse delta (C entry point gfz_inverse_delta_noalloc).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gfz {

// Largest stream one call accepts, in steps.
constexpr uint64_t kNoAllocMaxSteps = 1ull << 26;

// Undoes `delta_round` rounds of per-traversal delta coding of `in` into
// `out` (both device-accessible, n steps; in == out works in place) on
// `stream`, using only the library's static device scratch.  Synchronises
// `stream`.  Throws std::invalid_argument on bad arguments or sizes beyond
// kNoAllocMaxSteps, CudaError on a CUDA failure, std::runtime_error when a
// kernel reports an error.
void inverse_delta_noalloc(const int32_t *in, int32_t *out, uint64_t n, const uint64_t *offsets, uint64_t ntrav,
                           int delta_round, cudaStream_t stream);

}  // namespace gfz

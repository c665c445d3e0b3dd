/*
 * Force-included (g++ -include) ONLY when oracle/build_ref.sh compiles the
 * reference's src/cli/decompress_command.cpp without CUDA.  That file names
 * gpu_decompression::kDefaultRollingOutputChunkBytes and
 * resolve_omp_thread_count outside its ENABLE_CUDA guard
 * (src/cli/decompress_command.cpp:31,98,137,170), so a CPU-only build needs
 * these two declarations.  The constant mirrors the reference default of
 * 1 GiB (include/gpu/decompression/decompression_workflow_gpu.hpp:11-12).
 */
#pragma once
#include <cstddef>
#include "utils/threading_utils.hpp"

namespace gpu_decompression {
constexpr std::size_t kDefaultRollingOutputChunkBytes =
    1024ull * 1024ull * 1024ull;
}

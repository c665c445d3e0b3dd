// Host entropy stage and column encodings of the .gfaz container.
//
// zstd is the host entropy coder, loaded at run time from libzstd.so.1 with
// the reference's parameters (src/codec/codec.cpp:104-216): level from
// GFA_COMPRESSION_ZSTD_LEVEL (1..22, default 9), nbWorkers from
// GFA_COMPRESSION_ZSTD_WORKERS or the active host thread count, one
// ZSTD_compress2 call per column.  The other encodings (zigzag varints,
// delta varints, orientation bits) follow codec.cpp:247-526.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace gfz {

struct Block {
  std::vector<uint8_t> payload;
  uint64_t original_size = 0;
};

// Host thread policy (include/utils/threading_utils.hpp:13-49): n > 0 -> n;
// n < 0 -> all; 0 -> GFAZ_NUM_THREADS, OMP_NUM_THREADS, else
// min(8, max(1, nproc / 2)).
int resolve_threads(int n);

// Number of zstd workers for the current call scope.
void set_zstd_threads(int resolved_threads);
unsigned zstd_version();
bool zstd_available(std::string *why = nullptr);

Block zstd_bytes(const void *data, size_t n);
std::vector<uint8_t> unzstd(const Block &b);  // empty on failure (reference behaviour)

Block zstd_i32(const std::vector<int32_t> &v);
Block zstd_u32(const std::vector<uint32_t> &v);
Block zstd_str(const std::string &s);
Block zstd_chars(const std::vector<char> &v);
Block zstd_f32(const std::vector<float> &v);
std::vector<int32_t> unzstd_i32(const Block &b);
std::vector<uint32_t> unzstd_u32(const Block &b);
std::string unzstd_str(const Block &b);
std::vector<char> unzstd_chars(const Block &b);
std::vector<float> unzstd_f32(const Block &b);

Block delta_varint_u32(const std::vector<uint32_t> &v);
std::vector<uint32_t> undelta_varint_u32(const Block &b, size_t n);
Block orientations(const std::vector<char> &o);
std::vector<char> unorientations(const Block &b, size_t n);
Block varint_i64(const std::vector<int64_t> &v);
std::vector<int64_t> unvarint_i64(const Block &b, size_t n);

// concatenated strings + u32 lengths <-> list
void join_strings(const std::vector<std::string> &v, std::string &cat, std::vector<uint32_t> &lens);
// throws `prefix + "string column is truncated"` on overrun when strict
std::vector<std::string> split_strings(const std::string &cat, const std::vector<uint32_t> &lens, bool strict,
                                       const char *prefix);

}  // namespace gfz

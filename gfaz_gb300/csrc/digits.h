// Decimal digits without tables or divisions by variable amounts: the
// SWAR split of a number into 4-, 2- and 1-digit lanes with
// multiply-and-shift reciprocals that are exact over each lane's range.
// Shared by the text kernels and a host check of every value below 10^8.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define GFZ_HD __host__ __device__ __forceinline__
#else
#define GFZ_HD inline
#endif

namespace gfz {

// Powers of ten 10^0 .. 10^9 (a device copy for kernels, read through the
// read-only cache, and a host copy).
#if defined(__CUDACC__)
static __device__ const uint32_t g_pow10[10] = {1u, 10u, 100u, 1000u, 10000u, 100000u, 1000000u, 10000000u,
                                                100000000u, 1000000000u};
#endif
static const uint32_t g_pow10_host[10] = {1u, 10u, 100u, 1000u, 10000u, 100000u, 1000000u, 10000000u,
                                          100000000u, 1000000000u};

// Decimal digits of v (1 for 0): t = floor(bits(w) * log10(2)), with
// 1233 / 4096 for log10(2) (exact on 1..32 bits), is the digit count of
// w = v | 1 or one less, and one comparison with 10^t decides (setting the
// low bit moves no value across a power of ten above 1, and makes 0 count
// as one digit).
GFZ_HD uint32_t dec_count(uint32_t v) {
  const uint32_t w = v | 1u;
#if defined(__CUDA_ARCH__)
  const uint32_t bits = 32u - (uint32_t)__clz(w);
  const uint32_t t = (bits * 1233u) >> 12;
  const uint32_t p = __ldg(&g_pow10[t]);
#else
  const uint32_t bits = 32u - (uint32_t)__builtin_clz(w);
  const uint32_t t = (bits * 1233u) >> 12;
  const uint32_t p = g_pow10_host[t];
#endif
  return t + 1u - (w < p ? 1u : 0u);
}

// The 8 decimal digits of v < 10^8 as byte values 0..9, the most
// significant digit in the lowest byte (the order they are written in).
//   x / 100 = (x * 5243) >> 19   exact for x < 43699
//   y / 10  = (y * 103) >> 10    exact for y < 179
// The second split runs on two 16-bit lanes of one 32-bit word at once
// (lane products stay below 2^14, so no carry crosses a lane).
GFZ_HD uint64_t digits8(uint32_t v) {
  const uint32_t hi = v / 10000u, lo = v - hi * 10000u;
  const uint32_t qh = (hi * 5243u) >> 19, ql = (lo * 5243u) >> 19;
  const uint32_t ph = qh | ((hi - qh * 100u) << 16);
  const uint32_t pl = ql | ((lo - ql * 100u) << 16);
  const uint32_t th = ((ph * 103u) >> 10) & 0x000F000Fu;
  const uint32_t tl = ((pl * 103u) >> 10) & 0x000F000Fu;
  const uint32_t bh = th | ((ph - th * 10u) << 8);
  const uint32_t bl = tl | ((pl - tl * 10u) << 8);
  return (uint64_t)bh | ((uint64_t)bl << 32);
}

// The nd (1..8) trailing digits of v < 10^8 as ASCII, first digit in the
// lowest byte; the bytes above nd are zero.
GFZ_HD uint64_t ascii_digits(uint32_t v, uint32_t nd) {
  return (digits8(v) + 0x3030303030303030ull) >> (8u * (8u - nd));
}

}  // namespace gfz

// Checks gfz::digits8 / gfz::ascii_digits against plain division for every
// value below 10^8 (or below argv[1]), and gfz::dec_count against
// comparisons with the powers of ten for every 32-bit value.  Exit status 0
// when all agree.
#include <cstdio>
#include <cstdlib>

#include "digits.h"

int main(int argc, char **argv) {
  const uint32_t n = argc > 1 ? (uint32_t)std::strtoul(argv[1], nullptr, 10) : 100000000u;
  for (uint32_t v = 0; v < n; ++v) {
    uint64_t want = 0;
    uint32_t x = v;
    for (int i = 7; i >= 0; --i) {
      want |= (uint64_t)(x % 10u) << (8 * i);
      x /= 10u;
    }
    if (gfz::digits8(v) != want) {
      std::printf("digits8 mismatch at %u\n", v);
      return 1;
    }
    uint32_t nd = 1;
    for (uint32_t p = 10; p <= v && nd < 8; p *= 10) ++nd;
    char buf[16];
    const int len = std::snprintf(buf, sizeof buf, "%u", v);
    if (v % 997u == 0 || v < 100000u) {  // ASCII form on a sample
      const uint64_t a = gfz::ascii_digits(v, nd);
      for (int i = 0; i < 8; ++i) {
        const char c = (char)((a >> (8 * i)) & 0xFF);
        if ((i < len && c != buf[i]) || (i >= len && c != 0)) {
          std::printf("ascii_digits mismatch at %u\n", v);
          return 1;
        }
      }
    }
  }
  for (uint64_t v = 0; v <= 0xFFFFFFFFull; ++v) {
    const uint32_t x = (uint32_t)v;
    uint32_t want = 1;
    for (uint64_t p = 10; p <= x; p *= 10) ++want;
    if (gfz::dec_count(x) != want) {
      std::printf("dec_count mismatch at %u\n", x);
      return 1;
    }
  }
  std::printf("ok %u\n", n);
  return 0;
}

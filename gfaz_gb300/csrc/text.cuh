// Device helpers for GFA P/W text: decimal digits, traversal lookup and
// staged byte copies (the formats of format_*_line_numeric,
// src/io/gfa_write_utils.cpp:238-290).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "digits.h"

namespace gfz {

__device__ __forceinline__ uint32_t dec_digits(uint32_t v) { return dec_count(v); }

__device__ __forceinline__ void put_dec(char *dst, uint32_t v, uint32_t nd) {
  for (uint32_t i = nd; i-- > 0;) {
    dst[i] = (char)('0' + v % 10u);
    v /= 10u;
  }
}

// Largest t with off[t] <= p (p < off[ntrav]).
__device__ __forceinline__ uint64_t trav_of(const uint64_t *off, uint64_t ntrav, uint64_t p) {
  uint64_t lo = 0, hi = ntrav;  // answer in [0, ntrav)
  while (hi - lo > 1) {
    const uint64_t mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= p) lo = mid; else hi = mid;
  }
  return lo;
}

// Copies len bytes from a 16-byte aligned shared buffer (with >= 16 bytes of
// slack after len) to global memory using 16-byte stores where aligned.
template <int BLOCK>
__device__ __forceinline__ void block_copy_out(const char *sbuf, uint32_t len, char *dst) {
  const uint32_t mis = (uint32_t)((uintptr_t)dst & 15u);
  uint32_t head = (16u - mis) & 15u;
  if (head > len) head = len;
  for (uint32_t i = threadIdx.x; i < head; i += BLOCK) dst[i] = sbuf[i];
  const uint32_t body = (len - head) >> 4;
  const uint32_t *sw = reinterpret_cast<const uint32_t *>(sbuf);
  const uint32_t r = head & 3u, sh = 8u * r;
  for (uint32_t v = threadIdx.x; v < body; v += BLOCK) {
    const uint32_t o = head + 16u * v;
    const uint32_t w = o >> 2;
    uint4 val;
    if (r == 0) {
      val = make_uint4(sw[w], sw[w + 1], sw[w + 2], sw[w + 3]);
    } else {
      const uint32_t a0 = sw[w], a1 = sw[w + 1], a2 = sw[w + 2], a3 = sw[w + 3], a4 = sw[w + 4];
      val = make_uint4(__funnelshift_r(a0, a1, sh), __funnelshift_r(a1, a2, sh), __funnelshift_r(a2, a3, sh),
                       __funnelshift_r(a3, a4, sh));
    }
    __stcs(reinterpret_cast<uint4 *>(dst + o), val);  // evict-first: nothing here reads the text again
  }
  for (uint32_t i = head + 16u * body + threadIdx.x; i < len; i += BLOCK) dst[i] = sbuf[i];
}

// Text staging of one output tile: 2048 steps of up to 11 bytes; tiles
// whose text is longer (long line pieces, ten-digit ids) write to global
// memory directly.
constexpr uint32_t kTextBuf = 24 * 1024;

// The four decimal characters of every x < 10000 ("0000" .. "9999"), the
// first in the low byte; 40 KB that stays in L1 while text is written.
struct Dec4Table {
  uint32_t v[10000];
  constexpr Dec4Table() : v() {
    for (uint32_t x = 0; x < 10000; ++x)
      v[x] = (uint32_t)('0' + x / 1000) | ((uint32_t)('0' + x / 100 % 10) << 8) |
             ((uint32_t)('0' + x / 10 % 10) << 16) | ((uint32_t)('0' + x % 10) << 24);
  }
};
__device__ const Dec4Table g_dec4 = Dec4Table();

// Two decimal characters of x < 100, the first in the low byte.
__device__ __forceinline__ uint32_t dec_pair(uint32_t x) {
  const uint32_t t = x / 10u;
  return ('0' + t) | (('0' + (x - 10u * t)) << 8);
}

// Writes a byte stream into a zeroed shared word buffer with 32-bit stores.
// Bytes accumulate in a 64-bit register and leave as whole words; the
// stream's first word (when it does not start on a word boundary) and its
// last partial word may be shared with the neighbouring streams and are
// OR-ed in atomically.
struct WordWriter {
  uint32_t *buf;
  uint32_t w;               // next word to write
  uint32_t n;               // bytes pending in acc (< 4 between calls)
  uint32_t limit;           // words in buf; words beyond are dropped
  uint32_t acc;
  bool shared_first;
  bool overflow;            // a word fell outside buf
  __device__ __forceinline__ void init(uint32_t *b, uint32_t byte_off, uint32_t words) {
    buf = b;
    w = byte_off >> 2;
    n = byte_off & 3u;
    limit = words;
    acc = 0;
    shared_first = n != 0;
    overflow = false;
  }
  __device__ __forceinline__ void store(uint32_t word, bool shared) { store_at(w, word, shared); }
  __device__ __forceinline__ void store_at(uint32_t at, uint32_t word, bool shared) {
    if (at >= limit) {
      overflow = true;
      return;
    }
    if (shared) atomicOr(&buf[at], word);
    else buf[at] = word;
  }
  // Appends len (<= 12) bytes: the low bytes of b0 then of b1 (bytes above
  // len zero).  Whole words leave with up to three stores.
  __device__ __forceinline__ void put12(unsigned long long b0, uint32_t b1, uint32_t len) {
    const uint32_t x0 = (uint32_t)b0, x1 = (uint32_t)(b0 >> 32);
    const uint32_t sh = 8u * n;
    const uint32_t w0 = acc | (x0 << sh);
    const uint32_t w1 = __funnelshift_l(x0, x1, sh);
    const uint32_t w2 = __funnelshift_l(x1, b1, sh);
    const uint32_t w3 = __funnelshift_l(b1, 0u, sh);
    const uint32_t t = n + len, k = t >> 2;
    if (k >= 1) {
      store_at(w, w0, shared_first);
      shared_first = false;
    }
    if (k >= 2) store_at(w + 1, w1, false);
    if (k >= 3) store_at(w + 2, w2, false);
    w += k;
    n = t & 3u;
    acc = k == 0 ? w0 : k == 1 ? w1 : k == 2 ? w2 : w3;
  }
  // Appends the low cnt (<= 4) bytes of x (bytes above cnt must be zero).
  __device__ __forceinline__ void put(uint32_t x, uint32_t cnt) {
    const uint32_t sh = 8u * n;
    const uint32_t lo = acc | (x << sh);
    const uint32_t spill = __funnelshift_l(x, 0u, sh);  // the bytes of x beyond this word
    n += cnt;
    if (n >= 4) {
      store(lo, shared_first);
      shared_first = false;
      ++w;
      acc = spill;
      n -= 4;
    } else {
      acc = lo;
    }
  }
  // Appends the decimal digits of v (nd = dec_digits(v)), most significant first.
  __device__ __forceinline__ void put_dec(uint32_t v, uint32_t nd) {
    uint32_t lo = v;
    if (nd > 8) {
      const uint32_t hi = v / 100000000u;
      lo = v - hi * 100000000u;
      const uint32_t ph = dec_pair(hi);
      if (nd == 9) put(ph >> 8, 1);
      else put(ph, 2);
    }
    const uint32_t a = lo / 10000u;
    unsigned long long c8 = (unsigned long long)g_dec4.v[a] | ((unsigned long long)g_dec4.v[lo - a * 10000u] << 32);
    const uint32_t k = nd > 8 ? 8u : nd;  // digits of lo to write
    c8 >>= 8u * (8u - k);
    if (k > 4) {
      put((uint32_t)c8, 4);
      put((uint32_t)(c8 >> 32), k - 4);
    } else {
      put((uint32_t)c8, k);
    }
  }
  __device__ __forceinline__ void finish() {
    if (n && acc) store(acc, true);
  }
};

}  // namespace gfz

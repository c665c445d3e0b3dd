// S and L line text on the device (the segment and link lines of the
// full-file writer): src/io/gfa_writer.cpp:597-650 with the field layout of
// src/io/gfa_write_utils.cpp:58-76, 292-330:
//   S\t<id>\t<sequence><extra>\n          id = 1-based segment index
//   L\t<from>\t<fo>\t<to>\t<to_o>\t<ovl><extra>\n
//                                          ovl = <num><op>, or * when op is 0
// <extra> is the line's optional-field text, formatted on the host (stream
// float formatting) and passed as a blob.
//
// Work split: one thread per 16 output bytes, written with one 16-byte
// store.  Each thread finds the line of its first byte by binary search
// over the line offsets and walks forward through the lines its bytes
// touch, rebuilding the line's head (the fields before the sequence /
// extra) in a small local buffer.
#include "common.cuh"
#include "kernels.h"
#include "text.cuh"

namespace gfz {

namespace {

constexpr int kSB = 256;
constexpr uint32_t kSTile = kSB * 16;

__device__ __forceinline__ uint32_t put_u32(uint8_t *h, uint32_t at, uint32_t v) {
  const uint32_t nd = dec_digits(v);
  put_dec(reinterpret_cast<char *>(h + at), v, nd);
  return at + nd;
}

__device__ __forceinline__ uint32_t extra_len(const StaticTextSource &S, uint64_t i) {
  return S.ex_off ? (uint32_t)(S.ex_off[i + 1] - S.ex_off[i]) : 0u;
}

// The line head: for S lines "S\t<id>\t", for L lines everything up to the
// extra.  Returns its length; *body = bytes that follow from the sequence
// column (S) or 0 (L).
__device__ __forceinline__ uint32_t line_head(const StaticTextSource &S, uint64_t i, uint8_t *h, uint32_t &body) {
  uint32_t n = 0;
  if (S.kind == 0) {
    h[n++] = 'S';
    h[n++] = '\t';
    n = put_u32(h, n, (uint32_t)(i + 1));
    h[n++] = '\t';
    body = S.seg_len[i];
    return n;
  }
  h[n++] = 'L';
  h[n++] = '\t';
  n = put_u32(h, n, S.lf[i]);
  h[n++] = '\t';
  h[n++] = (uint8_t)S.lfo[i];
  h[n++] = '\t';
  n = put_u32(h, n, S.lt[i]);
  h[n++] = '\t';
  h[n++] = (uint8_t)S.lto[i];
  h[n++] = '\t';
  if (S.lop[i] != '\0') {
    n = put_u32(h, n, S.lnum[i]);
    h[n++] = (uint8_t)S.lop[i];
  } else {
    h[n++] = '*';
  }
  body = 0;
  return n;
}

__global__ void k_static_len(StaticTextSource S, uint64_t *len) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < S.n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t l;
    if (S.kind == 0)  // "S\t" id "\t" sequence
      l = 3 + dec_digits((uint32_t)(i + 1)) + (uint64_t)S.seg_len[i];
    else  // "L\t" from "\t" o "\t" to "\t" o "\t" overlap
      l = 8 + dec_digits(S.lf[i]) + dec_digits(S.lt[i]) + (S.lop[i] != '\0' ? dec_digits(S.lnum[i]) + 1 : 1);
    len[i] = l + extra_len(S, i) + 1;  // extra, newline
  }
}

__global__ void __launch_bounds__(kSB) k_static_write(StaticTextSource S, const uint64_t *__restrict__ loff,
                                                      uint64_t total, char *out) {
  const uint64_t o = (uint64_t)blockIdx.x * kSTile + 16ull * threadIdx.x;
  if (o >= total) return;
  // line of byte o: every thread searches the offsets itself (the upper
  // levels of the search are the same for the whole block and stay in L1)
  uint64_t i = trav_of(loff, S.n, o);
  uint8_t h[48];
  uint32_t body, hl = line_head(S, i, h, body);
  uint64_t ls = loff[i], le = loff[i + 1];
  uint32_t el = extra_len(S, i);
  uint32_t w[4] = {0, 0, 0, 0};
  const int cnt = total - o < 16 ? (int)(total - o) : 16;
  for (int k = 0; k < cnt; ++k) {
    const uint64_t p = o + k;
    if (p >= le) {
      ++i;
      hl = line_head(S, i, h, body);
      ls = le;
      le = loff[i + 1];
      el = extra_len(S, i);
    }
    const uint64_t j = p - ls;
    uint32_t c;
    if (j < hl) c = h[j];
    else if (j < hl + body) c = (uint8_t)S.seq[S.seq_off[i] + (j - hl)];
    else if (j < hl + body + el) c = (uint8_t)S.ex[S.ex_off[i] + (j - hl - body)];
    else c = '\n';
    w[k >> 2] |= c << (8 * (k & 3));
  }
  if (cnt == 16) {
    *reinterpret_cast<uint4 *>(out + o) = make_uint4(w[0], w[1], w[2], w[3]);
  } else {
    for (int k = 0; k < cnt; ++k) out[o + k] = (char)((w[k >> 2] >> (8 * (k & 3))) & 0xFFu);
  }
}

inline unsigned grid_for(uint64_t n, int block, unsigned cap = 152u * 16u) {
  uint64_t g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (unsigned)g;
}

}  // namespace

void launch_static_len(const StaticTextSource &S, uint64_t *len, cudaStream_t st) {
  if (S.n) k_static_len<<<grid_for(S.n, 256), 256, 0, st>>>(S, len);
}

void launch_static_write(const StaticTextSource &S, const uint64_t *loff, uint64_t total, char *out,
                         cudaStream_t st) {
  const uint64_t nt = (total + kSTile - 1) / kSTile;
  if (nt) k_static_write<<<(unsigned)nt, kSB, 0, st>>>(S, loff, total, out);
}

}  // namespace gfz

// Decompression-side kernels: rule-length table, expansion offsets,
// expansion, segmented inverse delta and P/W-line text emission.
//
// Semantics follow the reference CPU path:
//   expansion      src/workflows/decompression_workflow.cpp:70-106 (a symbol
//                  v with |v| in [min_id, min_id + R) is a rule; +R expands
//                  first then second, -R expands -second then -first)
//   inverse delta  src/codec/codec.cpp:29-41, applied delta_round times
//   text           src/io/gfa_write_utils.cpp:238-290 (P: "<id><+|->" joined
//                  by ',', W: "<>|<><id>" concatenated; decimal digits)
#include "common.cuh"
#include "text.cuh"
#include "kernels.h"

namespace gfz {

namespace {

constexpr int kBlock = 256;

inline unsigned grid_for(uint64_t n, int block, unsigned cap = 152u * 16u) {
  uint64_t g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (unsigned)g;
}


// ---------------------------------------------------------------------------
// Rule lengths
// ---------------------------------------------------------------------------
__global__ void k_rule_len_pass(const int32_t *__restrict__ first, const int32_t *__restrict__ second,
                                uint64_t nrules, uint32_t min_id, uint32_t *rlen, DevStatus *status, int slot,
                                uint64_t lo, uint64_t hi) {
  uint32_t open = 0;
  for (uint64_t i = lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < hi;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (rlen[i]) continue;
    const uint32_t a = abs32(first[i]), b = abs32(second[i]);
    const uint32_t la = is_rule(a, min_id, nrules) ? ((volatile uint32_t *)rlen)[a - min_id] : 1u;
    const uint32_t lb = is_rule(b, min_id, nrules) ? ((volatile uint32_t *)rlen)[b - min_id] : 1u;
    if (la && lb) {
      const unsigned long long s = (unsigned long long)la + lb;
      if (s > 0xFFFFFFFFull) {
        atomicOr(&status->err, kErrLength);
        rlen[i] = 0xFFFFFFFFu;
      } else {
        rlen[i] = (uint32_t)s;
      }
    } else {
      open++;
    }
  }
  open = __reduce_add_sync(0xffffffffu, open);
  if ((threadIdx.x & 31) == 0 && open) atomicAdd(&status->pass_open[slot], (unsigned long long)open);
}

// ---------------------------------------------------------------------------
// Expansion offsets (exclusive scan of symbol expansion lengths)
// ---------------------------------------------------------------------------
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_symbol_positions(const int32_t *__restrict__ enc, uint64_t m,
                                                            uint32_t min_id, uint64_t nrules,
                                                            const uint32_t *__restrict__ rlen, uint64_t *pos,
                                                            unsigned long long *desc, uint32_t *tile_counter,
                                                            DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ uint32_t sl[padded_size(TILE)];
  __shared__ unsigned long long s_excl;
  const uint32_t tile = claim_tile(tile_counter);
  const uint64_t base = (uint64_t)tile * TILE;
  const uint32_t len = (uint32_t)min((uint64_t)TILE, m - base);
  for (uint32_t j = threadIdx.x; j < len; j += BLOCK) {
    const uint32_t a = abs32(enc[base + j]);
    sl[padi(j)] = is_rule(a, min_id, nrules) ? rlen[a - min_id] : 1u;
  }
  __syncthreads();
  unsigned long long mine = 0;
  const uint32_t j0 = threadIdx.x * ITEMS;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k)
    if (j0 + k < len) mine += sl[padi(j0 + k)];
  unsigned long long total;
  unsigned long long ex = block_excl_sum<BLOCK>(mine, total);
  if (threadIdx.x < 32) {
    const unsigned long long e = warp_lookback<SumOp>(desc, tile, total, &status->err);
    if (threadIdx.x == 0) s_excl = e;
  }
  __syncthreads();
  unsigned long long p = s_excl + ex;
  // write through shared memory for coalesced stores
  __syncthreads();
  unsigned long long vals[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    vals[k] = p;
    if (j0 + k < len) p += sl[padi(j0 + k)];
  }
#pragma unroll
  for (int k = 0; k < ITEMS; ++k)
    if (j0 + k < len) pos[base + j0 + k] = vals[k];
  if (base + len == m && threadIdx.x == 0) pos[m] = s_excl + total;
}

// ---------------------------------------------------------------------------
// Expansion: one thread per encoded symbol, explicit stack
// ---------------------------------------------------------------------------
constexpr int kStackDepth = 64;

__global__ void k_expand(const int32_t *__restrict__ enc, uint64_t m, const uint64_t *__restrict__ pos,
                         const int32_t *__restrict__ first, const int32_t *__restrict__ second, uint64_t nrules,
                         uint32_t min_id, int32_t *__restrict__ out, DevStatus *status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t v = enc[i];
    uint64_t p = pos[i];
    if (!is_rule(abs32(v), min_id, nrules)) {
      out[p] = v;
      continue;
    }
    int32_t stack[kStackDepth];
    int sp = 0;
    stack[sp++] = v;
    while (sp > 0) {
      const int32_t x = stack[--sp];
      const uint32_t a = abs32(x);
      if (!is_rule(a, min_id, nrules)) {
        out[p++] = x;
        continue;
      }
      if (sp + 2 > kStackDepth) {
        atomicOr(&status->err, kErrDepth);
        break;
      }
      const int32_t f = first[a - min_id], g = second[a - min_id];
      if (x > 0) {
        stack[sp++] = g;
        stack[sp++] = f;
      } else {
        stack[sp++] = neg32(f);
        stack[sp++] = neg32(g);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Segmented inverse delta (in-place inclusive prefix sum per traversal)
// ---------------------------------------------------------------------------
struct SegAgg {
  uint32_t f;    // a traversal starts inside
  uint32_t sum;  // sum since the last start (or of everything)
};
__device__ __forceinline__ SegAgg seg_compose(const SegAgg &a, const SegAgg &b) {
  return b.f ? b : SegAgg{a.f, a.sum + b.sum};
}
// Segmented-sum monoid for the look-back: state = running value at the
// end of the previous tile (wrapping int32 arithmetic).
struct SegOp {
  using T = SegAgg;
  using S = uint32_t;
  __device__ static T identity() { return SegAgg{0u, 0u}; }
  __device__ static T compose(const T &a, const T &b) { return seg_compose(a, b); }
  __device__ static S apply(const T &f, S s) { return f.f ? f.sum : s + f.sum; }
  __device__ static S initial() { return 0u; }
  __device__ static unsigned long long encode_agg(const T &a) {
    return ((unsigned long long)a.f << 32) | a.sum;
  }
  __device__ static T decode_agg(unsigned long long d) { return SegAgg{(uint32_t)(d >> 32) & 1u, (uint32_t)d}; }
  __device__ static unsigned long long encode_incl(S s) { return s; }
  __device__ static S decode_incl(unsigned long long d) { return (uint32_t)d; }
  __device__ static T shfl_down(const T &a, int o) {
    return SegAgg{__shfl_down_sync(0xffffffffu, a.f, o), __shfl_down_sync(0xffffffffu, a.sum, o)};
  }
  __device__ static T shfl0(const T &a) {
    return SegAgg{__shfl_sync(0xffffffffu, a.f, 0), __shfl_sync(0xffffffffu, a.sum, 0)};
  }
};

template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_inverse_delta(int32_t *x, uint64_t n, const uint64_t *__restrict__ off,
                                                         uint64_t ntrav, unsigned long long *desc,
                                                         uint32_t *tile_counter, DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  constexpr int NW = BLOCK / 32;
  __shared__ uint32_t sv[padded_size(TILE)];
  __shared__ uint32_t hb[TILE / 32 + 2];
  __shared__ uint64_t s_tlo;
  __shared__ SegAgg s_w[NW];
  __shared__ uint32_t s_carry;
  const uint32_t tile = claim_tile(tile_counter);
  const uint64_t base = (uint64_t)tile * TILE;
  const uint32_t len = (uint32_t)min((uint64_t)TILE, n - base);
  for (uint32_t j = threadIdx.x; j < TILE / 32 + 2; j += BLOCK) hb[j] = 0;
  for (uint32_t j = threadIdx.x; j < len; j += BLOCK) sv[padi(j)] = (uint32_t)x[base + j];
  mark_heads(off, ntrav, base, len, hb, &s_tlo);
  __syncthreads();
  const uint32_t j0 = threadIdx.x * ITEMS;
  SegAgg a{0u, 0u};
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t j = j0 + k;
    if (j < len) {
      if (bit_at(hb, j)) a = SegAgg{1u, sv[padi(j)]};
      else a.sum += sv[padi(j)];
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  SegAgg inc = a;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    SegAgg o{__shfl_up_sync(0xffffffffu, inc.f, d), __shfl_up_sync(0xffffffffu, inc.sum, d)};
    if (lane >= d) inc = seg_compose(o, inc);
  }
  SegAgg ex{__shfl_up_sync(0xffffffffu, inc.f, 1), __shfl_up_sync(0xffffffffu, inc.sum, 1)};
  if (lane == 0) ex = SegAgg{0u, 0u};
  if (lane == 31) s_w[warp] = inc;
  __syncthreads();
  SegAgg wpre{0u, 0u}, total{0u, 0u};
  for (int w = 0; w < NW; ++w) {
    if (w == warp) wpre = total;
    total = seg_compose(total, s_w[w]);
  }
  ex = seg_compose(wpre, ex);
  if (warp == 0) {
    const uint32_t carry = warp_lookback<SegOp>(desc, tile, total, &status->err);
    if (lane == 0) s_carry = carry;
  }
  __syncthreads();
  uint32_t run = ex.f ? ex.sum : s_carry + ex.sum;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t j = j0 + k;
    if (j < len) {
      run = bit_at(hb, j) ? sv[padi(j)] : run + sv[padi(j)];
      sv[padi(j)] = run;
    }
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < len; j += BLOCK) x[base + j] = (int32_t)sv[padi(j)];
}

// ---------------------------------------------------------------------------
// Text emission
// ---------------------------------------------------------------------------
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_emit_text(const int32_t *__restrict__ x, uint64_t n,
                                                     const uint64_t *__restrict__ off, uint64_t ntrav, TextMeta meta,
                                                     char *__restrict__ text, unsigned long long *desc,
                                                     uint32_t *tile_counter, DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ int32_t sv[padded_size(TILE)];
  __shared__ __align__(16) char sbuf[kTextBuf + 32];
  __shared__ unsigned long long s_off;
  const uint32_t tile = claim_tile(tile_counter);
  const uint64_t base = (uint64_t)tile * TILE;
  const uint32_t len = (uint32_t)min((uint64_t)TILE, n - base);
  for (uint32_t j = threadIdx.x; j < len; j += BLOCK) sv[padi(j)] = x[base + j];
  __syncthreads();
  const uint32_t j0 = threadIdx.x * ITEMS;
  const bool pmode = meta.mode == 0;
  // per element: traversal boundaries and text length
  uint64_t t = 0;
  unsigned long long mine = 0;
  uint32_t flags = 0;  // bit 2k: first step, bit 2k+1: last step
  if (j0 < len) {
    t = trav_of(off, ntrav, base + j0);
    uint64_t tt = t;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const uint32_t j = j0 + k;
      if (j >= len) break;
      const uint64_t p = base + j;
      while (__ldg(off + tt + 1) <= p) ++tt;
      const bool fst = p == __ldg(off + tt);
      const bool lst = p + 1 == __ldg(off + tt + 1);
      flags |= ((uint32_t)fst << (2 * k)) | ((uint32_t)lst << (2 * k + 1));
      mine += dec_digits(abs32(sv[padi(j)])) + 1u + ((pmode && !lst) ? 1u : 0u);
      if (fst) mine += meta.pre_off[tt + 1] - meta.pre_off[tt];
      if (lst) mine += meta.suf_off[tt + 1] - meta.suf_off[tt];
    }
  }
  unsigned long long total;
  const unsigned long long ex = block_excl_sum<BLOCK>(mine, total);
  if (threadIdx.x < 32) {
    const unsigned long long e = warp_lookback<SumOp>(desc, tile, total, &status->err);
    if (threadIdx.x == 0) s_off = e;
  }
  __syncthreads();
  const unsigned long long toff = s_off;
  const bool last_tile = base + len == n;
  if (last_tile && threadIdx.x == 0) status->u64[7] = toff + total + meta.tail_len;
  if (text == nullptr) return;
  const bool staged = total <= kTextBuf;
  char *dst = staged ? sbuf + ex : text + toff + ex;
  if (j0 < len) {
    uint64_t tt = t;
    uint32_t o = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const uint32_t j = j0 + k;
      if (j >= len) break;
      const uint64_t p = base + j;
      while (__ldg(off + tt + 1) <= p) ++tt;
      const bool fst = (flags >> (2 * k)) & 1u, lst = (flags >> (2 * k + 1)) & 1u;
      if (fst) {
        const uint64_t a = meta.pre_off[tt], b = meta.pre_off[tt + 1];
        for (uint64_t q = a; q < b; ++q) dst[o++] = meta.blob[q];
      }
      const int32_t v = sv[padi(j)];
      const uint32_t av = abs32(v), nd = dec_digits(av);
      if (pmode) {
        put_dec(dst + o, av, nd);
        o += nd;
        dst[o++] = v < 0 ? '-' : '+';
        if (!lst) dst[o++] = ',';
      } else {
        dst[o++] = v < 0 ? '<' : '>';
        put_dec(dst + o, av, nd);
        o += nd;
      }
      if (lst) {
        const uint64_t a = meta.suf_off[tt], b = meta.suf_off[tt + 1];
        for (uint64_t q = a; q < b; ++q) dst[o++] = meta.blob[q];
      }
    }
  }
  if (staged) {
    __syncthreads();
    block_copy_out<BLOCK>(sbuf, (uint32_t)total, text + toff);
  }
  if (last_tile && meta.tail_len) {
    for (uint64_t q = threadIdx.x; q < meta.tail_len; q += BLOCK) text[toff + total + q] = meta.tail[q];
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
constexpr int kScanItems = 16;
constexpr int kDeltaItems = 16;
constexpr int kTextItems = 8;

void launch_rule_len_pass(const int32_t *first, const int32_t *second, uint64_t nrules, uint32_t min_id,
                          uint32_t *rlen, DevStatus *status, int slot, cudaStream_t st, uint64_t lo, uint64_t hi) {
  hi = std::min(hi, nrules);
  if (lo >= hi) return;
  k_rule_len_pass<<<grid_for(hi - lo, kBlock), kBlock, 0, st>>>(first, second, nrules, min_id, rlen, status, slot,
                                                                 lo, hi);
}

uint64_t scan_num_tiles(uint64_t n) {
  constexpr uint64_t TILE = kBlock * kScanItems;
  return (n + TILE - 1) / TILE;
}

void launch_symbol_positions(const int32_t *enc, uint64_t m, uint32_t min_id, uint64_t nrules, const uint32_t *rlen,
                             uint64_t *pos, unsigned long long *desc, uint32_t *tile_counter, DevStatus *status,
                             cudaStream_t st) {
  if (!m) return;
  k_symbol_positions<kBlock, kScanItems><<<(unsigned)scan_num_tiles(m), kBlock, 0, st>>>(
      enc, m, min_id, nrules, rlen, pos, desc, tile_counter, status);
}

void launch_expand(const int32_t *enc, uint64_t m, const uint64_t *pos, const int32_t *first, const int32_t *second,
                   uint64_t nrules, uint32_t min_id, int32_t *out, DevStatus *status, cudaStream_t st) {
  if (!m) return;
  k_expand<<<grid_for(m, kBlock, 152u * 64u), kBlock, 0, st>>>(enc, m, pos, first, second, nrules, min_id, out,
                                                               status);
}

static_assert((uint64_t)kBlock * kDeltaItems == kInverseDeltaTile, "inverse delta tile size");

uint64_t inverse_delta_num_tiles(uint64_t n) { return (n + kInverseDeltaTile - 1) / kInverseDeltaTile; }

void launch_inverse_delta(int32_t *x, uint64_t n, const uint64_t *off, uint64_t ntrav, unsigned long long *desc,
                          uint32_t *tile_counter, DevStatus *status, cudaStream_t st) {
  if (!n) return;
  k_inverse_delta<kBlock, kDeltaItems><<<(unsigned)inverse_delta_num_tiles(n), kBlock, 0, st>>>(
      x, n, off, ntrav, desc, tile_counter, status);
}

uint64_t text_num_tiles(uint64_t n) {
  constexpr uint64_t TILE = kBlock * kTextItems;
  return (n + TILE - 1) / TILE;
}

void launch_emit_text(const int32_t *x, uint64_t n, const uint64_t *off, uint64_t ntrav, TextMeta meta, char *text,
                      unsigned long long *desc, uint32_t *tile_counter, DevStatus *status, cudaStream_t st) {
  if (!n) return;
  k_emit_text<kBlock, kTextItems><<<(unsigned)text_num_tiles(n), kBlock, 0, st>>>(x, n, off, ntrav, meta, text, desc,
                                                                                  tile_counter, status);
}

}  // namespace gfz

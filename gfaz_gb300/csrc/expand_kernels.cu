// Prefix-sum expansion decoder: rule expansion, inverse delta coding and GFA
// text emission without a per-tile carry.
//
// With one round of delta coding (the reference default, codec.cpp:45-76)
// the decoded step at output position p is the running sum of the expanded
// deltas from its traversal's start to p.  Each rule R is therefore stored
// once as the inclusive prefix sums of its expansion, pre_R[0 .. len_R),
// and each encoded symbol i gets S_i, the sum of the whole expansions of the
// symbols before it in its traversal (a segmented scan over the encoded
// stream, which is ~40x shorter than the output).  The step at offset o of
// symbol i is then S_i + prefix(symbol, o), where for a reversed rule -R
// (expansion -x_{len-1}, ..., -x_0, as the reference's expansion writes it,
// path_decompression_gpu_rolling.cpp:215-370) prefix(-R, o) =
// -(pre_R[len-1] - pre_R[len-2-o]).  Every output tile is independent: the
// step kernel writes values directly; text is one length pass, a scan over
// tiles and one write pass.  With delta_round == 0 the same buffers give
// the plain expansion (differences of adjacent prefix values).
#include "common.cuh"
#include "kernels.h"
#include "text.cuh"

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
// Rule prefix buffer
// ---------------------------------------------------------------------------
// Inclusive prefix value at offset o (o < len) of the expansion of symbol c.
__device__ __forceinline__ uint32_t child_prefix(int32_t c, uint32_t o, const RulePrefixView &rv) {
  const uint32_t a = abs32(c);
  if (!is_rule(a, rv.min_id, rv.nrules)) return (uint32_t)c;
  const uint64_t r = a - rv.min_id;
  const uint64_t b = rv.roff[r];
  if (c > 0) return (uint32_t)rv.rpre[b + o];
  const uint32_t L = rv.rlen[r];
  const uint32_t tot = (uint32_t)rv.rpre[b + L - 1];
  const uint32_t before = o + 1 < L ? (uint32_t)rv.rpre[b + L - 2 - o] : 0u;
  return 0u - (tot - before);
}

// One build pass: every rule whose rule children were built in an earlier
// pass (built[c] in [1, pass)) writes pre_R = pre_first ++ (total_first +
// pre_second) and records built[R] = pass.  Rules still waiting are counted
// in status->u64[6].
__global__ void k_rule_prefix_pass(const int32_t *__restrict__ first, const int32_t *__restrict__ second,
                                   RulePrefixView rv, int32_t *rpre, uint32_t *built, uint32_t pass,
                                   DevStatus *status) {
  __shared__ uint32_t s_open;
  if (threadIdx.x == 0) s_open = 0;
  __syncthreads();
  uint32_t open = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < rv.nrules;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (built[i]) continue;
    const int32_t f = first[i], g = second[i];
    const uint32_t af = abs32(f), ag = abs32(g);
    const bool rf = is_rule(af, rv.min_id, rv.nrules), rg = is_rule(ag, rv.min_id, rv.nrules);
    const uint32_t bf = rf ? built[af - rv.min_id] : 1u, bg = rg ? built[ag - rv.min_id] : 1u;
    const bool ready = (!rf || (bf != 0 && bf < pass)) && (!rg || (bg != 0 && bg < pass));
    if (!ready) {
      open++;
      continue;
    }
    const uint32_t lf = rf ? rv.rlen[af - rv.min_id] : 1u, lg = rg ? rv.rlen[ag - rv.min_id] : 1u;
    if ((uint64_t)lf + lg != rv.rlen[i]) {
      atomicOr(&status->err, kErrLength);
      built[i] = pass;
      continue;
    }
    const uint64_t b = rv.roff[i];
    uint32_t last = 0;
    for (uint32_t o = 0; o < lf; ++o) {
      last = child_prefix(f, o, rv);
      rpre[b + o] = (int32_t)last;
    }
    for (uint32_t o = 0; o < lg; ++o) rpre[b + lf + o] = (int32_t)(last + child_prefix(g, o, rv));
    built[i] = pass;
  }
  open = __reduce_add_sync(0xffffffffu, open);
  if ((threadIdx.x & 31) == 0 && open) atomicAdd(&s_open, open);
  __syncthreads();
  if (threadIdx.x == 0 && s_open) atomicAdd(&status->u64[6], (unsigned long long)s_open);
}

// Exclusive scan of n values into out[0 .. n] (out[n] = total), decoupled
// look-back over tiles of BLOCK * ITEMS.
template <int BLOCK, int ITEMS, typename T>
__global__ void __launch_bounds__(BLOCK) k_excl_scan(const T *__restrict__ in, uint64_t n, uint64_t *out,
                                                     unsigned long long *desc, uint32_t *tile_counter,
                                                     DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ unsigned long long s_excl;
  const uint32_t tile = claim_tile(tile_counter);
  const uint64_t base = (uint64_t)tile * TILE;
  const uint64_t j0 = base + (uint64_t)threadIdx.x * ITEMS;
  unsigned long long v[ITEMS], mine = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    v[k] = j0 + k < n ? (unsigned long long)in[j0 + k] : 0ull;
    mine += v[k];
  }
  unsigned long long total;
  const unsigned long long ex = block_excl_sum<BLOCK>(mine, total);
  if (threadIdx.x < 32) {
    const unsigned long long e = warp_lookback<SumOp>(desc, tile, total, &status->err);
    if (threadIdx.x == 0) s_excl = e;
  }
  __syncthreads();
  unsigned long long p = s_excl + ex;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    if (j0 + k < n) out[j0 + k] = p;
    p += v[k];
  }
  if (base + TILE >= n && threadIdx.x == 0) out[n] = s_excl + total;
}

// ---------------------------------------------------------------------------
// Encoded symbols
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t symbol_total(int32_t v, const RulePrefixView &rv) {
  const uint32_t a = abs32(v);
  if (!is_rule(a, rv.min_id, rv.nrules)) return (uint32_t)v;
  const uint64_t r = a - rv.min_id;
  const uint32_t tot = (uint32_t)rv.rpre[rv.roff[r] + rv.rlen[r] - 1];
  return v > 0 ? tot : 0u - tot;
}

// rec[i] = {symbol, prefix buffer base, rule length (0 for a step), total of
// its expansion}; tot[i] = that total again (scanned in place afterwards).
__global__ void k_symbol_records(const int32_t *__restrict__ enc, uint64_t m, RulePrefixView rv, int4 *rec,
                                 int32_t *tot) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t v = enc[i];
    const uint32_t a = abs32(v);
    uint32_t b = 0, L = 0, t = (uint32_t)v;
    if (is_rule(a, rv.min_id, rv.nrules)) {
      const uint64_t r = a - rv.min_id;
      b = (uint32_t)rv.roff[r];
      L = rv.rlen[r];
      const uint32_t rt = (uint32_t)rv.rpre[b + L - 1];
      t = v > 0 ? rt : 0u - rt;
    }
    rec[i] = make_int4(v, (int32_t)b, (int32_t)L, (int32_t)t);
    if (tot) tot[i] = (int32_t)t;
  }
}

// With inclusive segmented sums in incl: rec[i].w = incl[i] - rec[i].w, the
// sum of the expansions before symbol i in its traversal.
__global__ void k_symbol_exclusive(int4 *rec, const int32_t *__restrict__ incl, uint64_t m) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
    rec[i].w = (int32_t)((uint32_t)incl[i] - (uint32_t)rec[i].w);
}

// tile_sym[k] = the symbol holding output step min(k * tile, total - 1):
// the largest i < m with pos[i] <= that step (pos strictly increasing).
__global__ void k_tile_symbols(const uint64_t *__restrict__ pos, uint64_t m, uint64_t total, uint64_t ntiles,
                               uint32_t tile, uint64_t *tile_sym) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k <= ntiles; k += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t p = k * (uint64_t)tile;
    if (p >= total) p = total - 1;
    uint64_t lo = 0, hi = m - 1;
    while (lo < hi) {
      const uint64_t mid = (lo + hi + 1) >> 1;
      if (pos[mid] <= p) lo = mid; else hi = mid - 1;
    }
    tile_sym[k] = lo;
  }
}

// ---------------------------------------------------------------------------
// Per-thread step values
// ---------------------------------------------------------------------------
// Symbols of one output tile staged in shared memory: pos[0 .. cnt] and the
// records of symbols lo .. lo + cnt - 1.  Tiles spanning more than kStageSyms
// symbols (little compression) read both from global memory instead.
constexpr uint32_t kStageSyms = 512;
struct SymStage {
  uint64_t pos[kStageSyms + 1];
  int4 rec[kStageSyms];
  uint64_t lo;
  uint32_t cnt;
  bool staged;
};

template <int BLOCK>
__device__ __forceinline__ void stage_symbols(const ExpandSource &E, uint64_t tile, SymStage &S) {
  const uint64_t lo = E.tile_sym[tile], hi = E.tile_sym[tile + 1];
  const uint64_t cnt = hi - lo + 1;
  const bool staged = cnt <= kStageSyms;
  if (staged) {
    for (uint32_t k = threadIdx.x; k <= cnt; k += BLOCK) S.pos[k] = E.pos[lo + k];
    for (uint32_t k = threadIdx.x; k < cnt; k += BLOCK) S.rec[k] = E.rec[lo + k];
  }
  if (threadIdx.x == 0) {
    S.lo = lo;
    S.cnt = (uint32_t)(staged ? cnt : 0);
    S.staged = staged;
  }
  __syncthreads();
}

// Step at offset o of a symbol with record r (prefix buffer rpre).
template <int DELTA>
__device__ __forceinline__ int32_t symbol_step(const int4 &r, uint32_t rtot, uint32_t o, const int32_t *__restrict__ rpre) {
  const int32_t v = r.x;
  const uint32_t b = (uint32_t)r.y, L = (uint32_t)r.z, s = (uint32_t)r.w;
  if (L == 0) return DELTA ? (int32_t)(s + (uint32_t)v) : v;
  if (DELTA) {
    if (v > 0) return (int32_t)(s + (uint32_t)rpre[b + o]);
    const uint32_t before = o + 1 < L ? (uint32_t)rpre[b + L - 2 - o] : 0u;
    return (int32_t)(s - (rtot - before));
  }
  const uint32_t q = v > 0 ? o : L - 1 - o;
  const uint32_t x = (uint32_t)rpre[b + q] - (q ? (uint32_t)rpre[b + q - 1] : 0u);
  return v > 0 ? (int32_t)x : (int32_t)(0u - x);
}

// Values of output steps p0 .. p0 + ITEMS - 1 (those below total) of the
// staged tile; returns how many are valid.
template <int ITEMS, int DELTA>
__device__ __forceinline__ uint32_t thread_values(const ExpandSource &E, const SymStage &S, uint64_t tile,
                                                  uint64_t p0, int32_t (&val)[ITEMS]) {
  if (p0 >= E.total) return 0;
  // the symbol holding p0: largest i with pos[i] <= p0
  uint64_t i;
  uint64_t start, end;
  int4 r;
  if (S.staged) {
    uint32_t lo = 0, hi = S.cnt - 1;
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (S.pos[mid] <= p0) lo = mid; else hi = mid - 1;
    }
    i = lo;
    start = S.pos[lo];
    end = S.pos[lo + 1];
    r = S.rec[lo];
  } else {
    uint64_t lo = E.tile_sym[tile], hi = E.tile_sym[tile + 1];
    while (lo < hi) {
      const uint64_t mid = (lo + hi + 1) >> 1;
      if (E.pos[mid] <= p0) lo = mid; else hi = mid - 1;
    }
    i = lo;
    start = E.pos[lo];
    end = E.pos[lo + 1];
    r = E.rec[lo];
  }
  uint32_t rtot = (!DELTA || r.x >= 0 || r.z == 0) ? 0u : (uint32_t)E.rules.rpre[(uint32_t)r.y + (uint32_t)r.z - 1];
  uint32_t cnt = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint64_t p = p0 + k;
    if (p < E.total) {
      if (p >= end) {  // next symbol (symbols are at least one step long)
        ++i;
        start = end;
        if (S.staged) {
          end = S.pos[i + 1];
          r = S.rec[i];
        } else {
          end = E.pos[i + 1];
          r = E.rec[i];
        }
        if (DELTA && r.x < 0 && r.z != 0) rtot = (uint32_t)E.rules.rpre[(uint32_t)r.y + (uint32_t)r.z - 1];
      }
      val[k] = symbol_step<DELTA>(r, rtot, (uint32_t)(p - start), E.rules.rpre);
      cnt = k + 1;
    }
  }
  return cnt;
}

// ---------------------------------------------------------------------------
// Step output
// ---------------------------------------------------------------------------
template <int BLOCK, int ITEMS, int DELTA>
__global__ void __launch_bounds__(BLOCK) k_expand_steps(ExpandSource E, int32_t *__restrict__ out) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ SymStage S;
  const uint64_t tile = blockIdx.x;
  stage_symbols<BLOCK>(E, tile, S);
  const uint64_t p0 = tile * TILE + (uint64_t)threadIdx.x * ITEMS;
  int32_t val[ITEMS];
  const uint32_t cnt = thread_values<ITEMS, DELTA>(E, S, tile, p0, val);
  if (cnt == ITEMS && (reinterpret_cast<uintptr_t>(out + p0) & 15u) == 0) {
#pragma unroll
    for (int k = 0; k < ITEMS; k += 4)
      *reinterpret_cast<int4 *>(out + p0 + k) = make_int4(val[k], val[k + 1], val[k + 2], val[k + 3]);
  } else {
#pragma unroll
    for (int k = 0; k < ITEMS; ++k)
      if ((uint32_t)k < cnt) out[p0 + k] = val[k];
  }
}

// ---------------------------------------------------------------------------
// Text
// ---------------------------------------------------------------------------
// Text bytes of one step: the number, its orientation mark and (P lines,
// not last) the comma.
__device__ __forceinline__ uint32_t step_text_len(int32_t v, bool pmode, bool last) {
  return dec_digits(abs32(v)) + 1u + ((pmode && !last) ? 1u : 0u);
}

// Per-thread text length of steps p0 .. p0 + ITEMS - 1; fst/lst bits of
// those steps come from the output head bitmap.
template <int ITEMS>
__device__ __forceinline__ unsigned long long thread_text_len(const int32_t (&val)[ITEMS], uint32_t cnt, uint64_t p0,
                                                              const TextSource &T, uint32_t &hd) {
  hd = 0;
  if (!cnt) return 0;
  const uint64_t w = p0 >> 5;
  const unsigned long long two = ((unsigned long long)T.heads[w + 1] << 32) | T.heads[w];
  hd = (uint32_t)(two >> (p0 & 31));  // bit k: step p0 + k starts a traversal (ITEMS <= 31)
  const bool pmode = T.meta.mode == 0;
  unsigned long long len = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    if ((uint32_t)k < cnt) {
      const bool fst = (hd >> k) & 1u, lst = (hd >> (k + 1)) & 1u;
      len += step_text_len(val[k], pmode, lst);
      if (fst | lst) {
        const uint64_t t = trav_of(T.off, T.ntrav, p0 + k);
        if (fst) len += T.meta.pre_off[t + 1] - T.meta.pre_off[t];
        if (lst) len += T.meta.suf_off[t + 1] - T.meta.suf_off[t];
      }
    }
  }
  return len;
}

template <int BLOCK, int ITEMS, int DELTA>
__global__ void __launch_bounds__(BLOCK) k_text_lengths(ExpandSource E, TextSource T, uint64_t *tile_len) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ SymStage S;
  const uint64_t tile = blockIdx.x;
  stage_symbols<BLOCK>(E, tile, S);
  const uint64_t p0 = tile * TILE + (uint64_t)threadIdx.x * ITEMS;
  int32_t val[ITEMS];
  const uint32_t cnt = thread_values<ITEMS, DELTA>(E, S, tile, p0, val);
  uint32_t hd;
  unsigned long long len = thread_text_len<ITEMS>(val, cnt, p0, T, hd);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) len += __shfl_xor_sync(0xffffffffu, len, d);
  __shared__ unsigned long long s_w[BLOCK / 32];
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = len;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < BLOCK / 32; ++w) t += s_w[w];
    tile_len[tile] = t;
  }
}

template <int BLOCK, int ITEMS, int DELTA>
__global__ void __launch_bounds__(BLOCK) k_text_write(ExpandSource E, TextSource T, const uint64_t *__restrict__ tile_off,
                                                      char *__restrict__ text) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ __align__(16) char sbuf[kTextBuf + 32];
  __shared__ SymStage S;
  const uint64_t tile = blockIdx.x;
  stage_symbols<BLOCK>(E, tile, S);
  const uint64_t p0 = tile * TILE + (uint64_t)threadIdx.x * ITEMS;
  int32_t val[ITEMS];
  const uint32_t cnt = thread_values<ITEMS, DELTA>(E, S, tile, p0, val);
  uint32_t hd;
  const unsigned long long mine = thread_text_len<ITEMS>(val, cnt, p0, T, hd);
  unsigned long long total;
  const unsigned long long ex = block_excl_sum<BLOCK>(mine, total);
  const uint64_t toff = tile_off[tile];
  const bool staged = total <= kTextBuf;
  char *dst = staged ? sbuf + ex : text + toff + ex;
  const bool pmode = T.meta.mode == 0;
  uint32_t o = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    if ((uint32_t)k < cnt) {
      const bool fst = (hd >> k) & 1u, lst = (hd >> (k + 1)) & 1u;
      uint64_t t = 0;
      if (fst | lst) t = trav_of(T.off, T.ntrav, p0 + k);
      if (fst)
        for (uint64_t q = T.meta.pre_off[t]; q < T.meta.pre_off[t + 1]; ++q) dst[o++] = T.meta.blob[q];
      const int32_t v = val[k];
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
      if (lst)
        for (uint64_t q = T.meta.suf_off[t]; q < T.meta.suf_off[t + 1]; ++q) dst[o++] = T.meta.blob[q];
    }
  }
  if (staged) {
    __syncthreads();
    block_copy_out<BLOCK>(sbuf, (uint32_t)total, text + toff);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
constexpr int kExpandItems = 8;
constexpr uint32_t kExpandTile = kBlock * kExpandItems;
constexpr int kScanItemsU = 16;

uint64_t expand_num_tiles(uint64_t total) { return (total + kExpandTile - 1) / kExpandTile; }
uint64_t excl_scan_tiles(uint64_t n) {
  constexpr uint64_t TILE = kBlock * kScanItemsU;
  return (n + TILE - 1) / TILE;
}

void launch_rule_prefix_pass(const int32_t *first, const int32_t *second, RulePrefixView rv, int32_t *rpre,
                             uint32_t *built, uint32_t pass, DevStatus *status, cudaStream_t st) {
  if (!rv.nrules) return;
  k_rule_prefix_pass<<<grid_for(rv.nrules, kBlock, 152u * 32u), kBlock, 0, st>>>(first, second, rv, rpre, built, pass,
                                                                                 status);
}

void launch_excl_scan_u32(const uint32_t *in, uint64_t n, uint64_t *out, unsigned long long *desc,
                          uint32_t *tile_counter, DevStatus *status, cudaStream_t st) {
  k_excl_scan<kBlock, kScanItemsU, uint32_t><<<(unsigned)std::max<uint64_t>(excl_scan_tiles(n), 1), kBlock, 0, st>>>(
      in, n, out, desc, tile_counter, status);
}

void launch_excl_scan_u64(const uint64_t *in, uint64_t n, uint64_t *out, unsigned long long *desc,
                          uint32_t *tile_counter, DevStatus *status, cudaStream_t st) {
  k_excl_scan<kBlock, kScanItemsU, uint64_t><<<(unsigned)std::max<uint64_t>(excl_scan_tiles(n), 1), kBlock, 0, st>>>(
      in, n, out, desc, tile_counter, status);
}

void launch_symbol_records(const int32_t *enc, uint64_t m, RulePrefixView rv, int4 *rec, int32_t *tot,
                           cudaStream_t st) {
  if (!m) return;
  k_symbol_records<<<grid_for(m, kBlock), kBlock, 0, st>>>(enc, m, rv, rec, tot);
}

void launch_symbol_exclusive(int4 *rec, const int32_t *incl, uint64_t m, cudaStream_t st) {
  if (!m) return;
  k_symbol_exclusive<<<grid_for(m, kBlock), kBlock, 0, st>>>(rec, incl, m);
}

void launch_tile_symbols(const uint64_t *pos, uint64_t m, uint64_t total, uint64_t *tile_sym, cudaStream_t st) {
  const uint64_t nt = expand_num_tiles(total);
  if (!m || !total) return;
  k_tile_symbols<<<grid_for(nt + 1, kBlock), kBlock, 0, st>>>(pos, m, total, nt, kExpandTile, tile_sym);
}

void launch_expand_steps(const ExpandSource &E, int delta, int32_t *out, cudaStream_t st) {
  const uint64_t nt = expand_num_tiles(E.total);
  if (!nt) return;
  if (delta)
    k_expand_steps<kBlock, kExpandItems, 1><<<(unsigned)nt, kBlock, 0, st>>>(E, out);
  else
    k_expand_steps<kBlock, kExpandItems, 0><<<(unsigned)nt, kBlock, 0, st>>>(E, out);
}

void launch_text_lengths(const ExpandSource &E, const TextSource &T, int delta, uint64_t *tile_len, cudaStream_t st) {
  const uint64_t nt = expand_num_tiles(E.total);
  if (!nt) return;
  if (delta)
    k_text_lengths<kBlock, kExpandItems, 1><<<(unsigned)nt, kBlock, 0, st>>>(E, T, tile_len);
  else
    k_text_lengths<kBlock, kExpandItems, 0><<<(unsigned)nt, kBlock, 0, st>>>(E, T, tile_len);
}

void launch_text_write(const ExpandSource &E, const TextSource &T, int delta, const uint64_t *tile_off, char *text,
                       cudaStream_t st) {
  const uint64_t nt = expand_num_tiles(E.total);
  if (!nt) return;
  if (delta)
    k_text_write<kBlock, kExpandItems, 1><<<(unsigned)nt, kBlock, 0, st>>>(E, T, tile_off, text);
  else
    k_text_write<kBlock, kExpandItems, 0><<<(unsigned)nt, kBlock, 0, st>>>(E, T, tile_off, text);
}

}  // namespace gfz

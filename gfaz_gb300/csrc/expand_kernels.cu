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
// in status->pass_open[slot].
// Prefix value at offset o of rule i = first ++ second (lf steps of first).
__device__ __forceinline__ uint32_t rule_prefix_at(int32_t f, int32_t g, uint32_t lf, uint32_t tf, uint32_t o,
                                                   const RulePrefixView &rv) {
  return o < lf ? child_prefix(f, o, rv) : tf + child_prefix(g, o - lf, rv);
}

// Value ranges of the text length shortcut, folded over offsets: delta 1:
// prefix values (all, and {0} plus all but the last); delta 0: expansion
// values.
struct RangeAcc {
  int32_t mnA = INT32_MAX, mxA = INT32_MIN, mnB = 0, mxB = 0;
  __device__ __forceinline__ void add(int32_t y, bool not_last) {
    mnA = min(mnA, y);
    mxA = max(mxA, y);
    if (not_last) {
      mnB = min(mnB, y);
      mxB = max(mxB, y);
    }
  }
};

// rules longer than this are written by a whole warp (16 measured best of
// 4 to 256: prefix build 0.47 ms per step at 16, 0.49 at 8, 0.62 at 32)
constexpr uint32_t kWarpRule = 16;

__global__ void k_rule_prefix_pass(const int32_t *__restrict__ first, const int32_t *__restrict__ second,
                                   RulePrefixView rv, int32_t *rpre, int4 *rstat, int delta, uint32_t *built,
                                   uint32_t pass, DevStatus *status, int slot, uint64_t lo, uint64_t hi) {
  __shared__ uint32_t s_open;
  if (threadIdx.x == 0) s_open = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  uint32_t open = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // whole warps walk the rules [lo, hi) together so that long rules can be
  // shared
  const uint64_t span = (hi - lo + 31) & ~31ull;
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < span; j += stride) {
    const uint64_t i = lo + j;
    bool ready = false;
    int32_t f = 0, g = 0;
    uint32_t lf = 0, lg = 0;
    if (i < hi && !built[i]) {
      f = first[i];
      g = second[i];
      const uint32_t af = abs32(f), ag = abs32(g);
      const bool rf = is_rule(af, rv.min_id, rv.nrules), rg = is_rule(ag, rv.min_id, rv.nrules);
      const uint32_t bf = rf ? built[af - rv.min_id] : 1u, bg = rg ? built[ag - rv.min_id] : 1u;
      ready = (!rf || (bf != 0 && bf < pass)) && (!rg || (bg != 0 && bg < pass));
      if (!ready) {
        open++;
      } else {
        lf = rf ? rv.rlen[af - rv.min_id] : 1u;
        lg = rg ? rv.rlen[ag - rv.min_id] : 1u;
        if ((uint64_t)lf + lg != rv.rlen[i]) {
          atomicOr(&status->err, kErrLength);
          built[i] = pass;
          ready = false;
        }
      }
    }
    const uint32_t L = lf + lg;
    if (ready && L <= kWarpRule) {
      const uint64_t b = rv.roff[i];
      const uint32_t tf = child_prefix(f, lf - 1, rv);
      RangeAcc r;
      uint32_t prev = 0;
      for (uint32_t o = 0; o < L; ++o) {
        const uint32_t x = rule_prefix_at(f, g, lf, tf, o, rv);
        rpre[b + o] = (int32_t)x;
        r.add(delta ? (int32_t)x : (int32_t)(x - prev), delta && o + 1 < L);
        prev = x;
      }
      rstat[i] = make_int4(r.mnA, r.mxA, r.mnB, r.mxB);
      built[i] = pass;
    }
    // long rules: one at a time, the warp's lanes on consecutive offsets;
    // each lane first loads its own rule's buffer offset and first part's
    // total, so that the serial walk over the warp's rules waits on no load
    // before its first offsets
    const bool is_long = ready && L > kWarpRule;
    uint64_t my_b = 0;
    uint32_t my_tf = 0;
    if (is_long) {
      my_b = rv.roff[i];
      my_tf = child_prefix(f, lf - 1, rv);
    }
    uint32_t longs = __ballot_sync(0xffffffffu, is_long);
    while (longs) {
      const int src = __ffs(longs) - 1;
      longs &= longs - 1;
      const uint64_t ri = __shfl_sync(0xffffffffu, i, src);
      const int32_t rf_ = __shfl_sync(0xffffffffu, f, src), rg_ = __shfl_sync(0xffffffffu, g, src);
      const uint32_t rlf = __shfl_sync(0xffffffffu, lf, src), rL = __shfl_sync(0xffffffffu, L, src);
      const uint64_t b = __shfl_sync(0xffffffffu, my_b, src);
      const uint32_t tf = __shfl_sync(0xffffffffu, my_tf, src);
      RangeAcc r;
      for (uint32_t o0 = 0; o0 < rL; o0 += 32) {
        const uint32_t o = o0 + lane;
        if (o < rL) {
          const uint32_t x = rule_prefix_at(rf_, rg_, rlf, tf, o, rv);
          rpre[b + o] = (int32_t)x;
          int32_t y = (int32_t)x;
          if (!delta) y = (int32_t)(x - (o ? rule_prefix_at(rf_, rg_, rlf, tf, o - 1, rv) : 0u));
          r.add(y, delta && o + 1 < rL);
        }
      }
      r.mnA = __reduce_min_sync(0xffffffffu, r.mnA);
      r.mxA = __reduce_max_sync(0xffffffffu, r.mxA);
      r.mnB = __reduce_min_sync(0xffffffffu, r.mnB);
      r.mxB = __reduce_max_sync(0xffffffffu, r.mxB);
      if (lane == src) {
        rstat[ri] = make_int4(r.mnA, r.mxA, r.mnB, r.mxB);
        built[ri] = pass;
      }
    }
  }
  open = __reduce_add_sync(0xffffffffu, open);
  if (lane == 0 && open) atomicAdd(&s_open, open);
  __syncthreads();
  if (threadIdx.x == 0 && s_open) atomicAdd(&status->pass_open[slot], (unsigned long long)s_open);
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

// With inclusive segmented sums in incl: rec[i].w = S_i = incl[i] -
// rec[i].w, the sum of the expansions before symbol i in its traversal; for
// a reversed rule (symbol < 0), S_i minus the rule's total, which is
// incl[i] itself (its expansion sums to minus that total), so that its
// steps need no gather of the total: step o is rec.w + the rule's prefix
// at L - 2 - o (0 for the last step).
__global__ void k_symbol_exclusive(int4 *rec, const int32_t *__restrict__ incl, uint64_t m) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    const int4 r = rec[i];
    rec[i].w = (r.x < 0 && r.z != 0) ? incl[i] : (int32_t)((uint32_t)incl[i] - (uint32_t)r.w);
  }
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
// symbols (little compression) read both from global memory instead.  256
// symbols (an output tile of 2048 steps holds about 50 on the
// chromosome-scale workload) keep the text kernel's shared memory at 31 KB,
// for seven resident blocks per SM.
constexpr uint32_t kStageSyms = 256;
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
    // evict-first loads: a tile's symbols are read by it (and its
    // neighbour's edge) only, and L2 is better left to the prefix buffer
    const unsigned long long *pos = reinterpret_cast<const unsigned long long *>(E.pos) + lo;
    for (uint32_t k = threadIdx.x; k <= cnt; k += BLOCK) S.pos[k] = __ldcs(pos + k);
    for (uint32_t k = threadIdx.x; k < cnt; k += BLOCK) S.rec[k] = __ldcs(E.rec + lo + k);
  }
  if (threadIdx.x == 0) {
    S.lo = lo;
    S.cnt = (uint32_t)(staged ? cnt : 0);
    S.staged = staged;
  }
  __syncthreads();
}

// Step at offset o of a symbol with record r (prefix buffer rpre; with
// DELTA, r.w as k_symbol_exclusive leaves it).
template <int DELTA>
__device__ __forceinline__ int32_t symbol_step(const int4 &r, uint32_t o, const int32_t *__restrict__ rpre) {
  const int32_t v = r.x;
  const uint32_t b = (uint32_t)r.y, L = (uint32_t)r.z, s = (uint32_t)r.w;
  if (L == 0) return DELTA ? (int32_t)(s + (uint32_t)v) : v;
  if (DELTA) {
    if (v > 0) return (int32_t)(s + (uint32_t)rpre[b + o]);
    const uint32_t before = o + 1 < L ? (uint32_t)rpre[b + L - 2 - o] : 0u;
    return (int32_t)(s + before);
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
      }
      val[k] = symbol_step<DELTA>(r, (uint32_t)(p - start), E.rules.rpre);
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
__device__ __forceinline__ bool head_at(const uint32_t *heads, uint64_t q) { return (heads[q >> 5] >> (q & 31)) & 1u; }

// Digit count shared by every value in [lo, hi] (exact, no wrap-around), or
// 0 when the values differ in length or the range leaves int32.
__device__ __forceinline__ uint32_t uniform_digits(long long lo, long long hi) {
  if (lo < INT32_MIN || hi > INT32_MAX) return 0;
  uint32_t a, b;
  if (lo >= 0) {
    a = dec_digits((uint32_t)lo);
    b = dec_digits((uint32_t)hi);
  } else if (hi <= 0) {
    a = dec_digits((uint32_t)(-lo));
    b = dec_digits((uint32_t)(-hi));
  } else {
    a = 1;
    b = dec_digits((uint32_t)max(-lo, hi));
  }
  return a == b ? a : 0u;
}

// The digit count all steps of symbol r share (0 if they differ).
template <int DELTA>
__device__ __forceinline__ uint32_t symbol_digits(const int4 &r, const RulePrefixView &rv) {
  const int32_t v = r.x;
  const uint32_t L = (uint32_t)r.z;
  if (L == 0) return dec_digits(abs32(DELTA ? (int32_t)((uint32_t)r.w + (uint32_t)v) : v));
  const int4 st = rv.rstat[abs32(v) - rv.min_id];
  if (DELTA) {
    if (v > 0) return uniform_digits((long long)r.w + st.x, (long long)r.w + st.y);
    // a reversed rule's steps are r.w + {0, its prefix values but the last}
    return uniform_digits((long long)r.w + st.z, (long long)r.w + st.w);
  }
  return v > 0 ? uniform_digits(st.x, st.y) : uniform_digits(-(long long)st.y, -(long long)st.x);
}

// Text bytes of steps [from, to) of symbol r (none of them the last step of
// its traversal): digits plus the orientation mark and, in P lines, a comma.
template <int DELTA>
__device__ __forceinline__ unsigned long long steps_text(const int4 &r, uint32_t dig, uint32_t from, uint32_t to,
                                                         bool pmode, const int32_t *__restrict__ rpre) {
  const uint32_t per = pmode ? 2u : 1u;
  if (dig) return (unsigned long long)(to - from) * (dig + per);
  unsigned long long len = 0;
  for (uint32_t o = from; o < to; ++o) len += dec_digits(abs32(symbol_step<DELTA>(r, o, rpre))) + per;
  return len;
}

__device__ __forceinline__ uint64_t pre_len(const TextSource &T, uint64_t t) { return T.meta.pre_off[t + 1] - T.meta.pre_off[t]; }
__device__ __forceinline__ uint64_t suf_len(const TextSource &T, uint64_t t) { return T.meta.suf_off[t + 1] - T.meta.suf_off[t]; }

// slen[i]: the line prefix (first symbol of a traversal), the steps, and the
// line suffix (last symbol); sdig[i]: the shared digit count or 0.
template <int DELTA>
__global__ void k_symbol_text(ExpandSource E, TextSource T, uint64_t *slen, uint8_t *sdig) {
  const bool pmode = T.meta.mode == 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E.m; i += (uint64_t)gridDim.x * blockDim.x) {
    const int4 r = E.rec[i];
    const uint64_t start = E.pos[i], end = E.pos[i + 1];
    const uint32_t dig = symbol_digits<DELTA>(r, E.rules);
    unsigned long long len = steps_text<DELTA>(r, dig, 0, (uint32_t)(end - start), pmode, E.rules.rpre);
    const bool fst = head_at(T.heads, start), lst = head_at(T.heads, end);
    if (fst | lst) {
      const uint64_t t = trav_of(T.off, T.ntrav, start);
      if (fst) len += pre_len(T, t);
      if (lst) len += suf_len(T, t) - (pmode ? 1ull : 0ull);  // no comma after the last step
    }
    slen[i] = len;
    sdig[i] = (uint8_t)dig;
  }
}

// Text offset of output step p (p < total) held by symbol r (index i,
// steps from `start`): where the text of p begins, before the line prefix
// if p opens its traversal.
template <int DELTA>
__device__ __forceinline__ unsigned long long step_offset(const ExpandSource &E, const TextSource &T,
                                                          const uint64_t *soff, const uint8_t *sdig, uint64_t i,
                                                          const int4 &r, uint64_t start, uint64_t p, bool pmode) {
  unsigned long long o = soff[i];
  if (p == start) return o;
  if (head_at(T.heads, start)) o += pre_len(T, trav_of(T.off, T.ntrav, start));
  return o + steps_text<DELTA>(r, sdig[i], 0, (uint32_t)(p - start), pmode, E.rules.rpre);
}

// Text offset of the first step of every output tile: where the tile's
// text begins (before the line prefix when that step opens a traversal).
template <int DELTA>
__global__ void k_tile_text_off(ExpandSource E, TextSource T, const uint64_t *__restrict__ soff,
                                const uint8_t *__restrict__ sdig, uint64_t ntiles, uint32_t tile_steps,
                                uint64_t *__restrict__ toff) {
  const bool pmode = T.meta.mode == 0;
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < ntiles;
       k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = E.tile_sym[k];
    const int4 r = E.rec[i];
    toff[k] = step_offset<DELTA>(E, T, soff, sdig, i, r, E.pos[i], k * tile_steps, pmode);
  }
}

// One output tile per block: the steps' values from the rule prefix buffer,
// each thread's text length from its values, a block scan for the thread
// offsets, the text packed into 32-bit words in shared memory and written
// out with 16-byte stores.  toff[tile] (k_tile_text_off) places the tile;
// its end must meet the next tile's start (or the body end), else the
// per-symbol lengths and the text disagree and kErrLength is raised.
// Seven resident blocks per SM (32 registers, 31 KB of shared memory): the
// kernel is bound by issue and gather latency, and more warps cover both
// (4.49 against 5.22 ms per step at five blocks).
template <int BLOCK, int ITEMS, int DELTA>
__global__ void __launch_bounds__(BLOCK, 7) k_text_write(ExpandSource E, TextSource T, const uint64_t *__restrict__ toff,
                                                      char *__restrict__ text, uint64_t tile0, uint64_t ntiles) {
  static_assert(ITEMS <= 8, "digit counts are packed 4 bits per step");
  constexpr uint32_t TILE = BLOCK * ITEMS;
  constexpr uint32_t kWords = kTextBuf / 4 + 8;
  __shared__ __align__(16) uint32_t sbuf[kWords];
  __shared__ SymStage S;
  const uint64_t tile = tile0 + blockIdx.x;
  const bool pmode = T.meta.mode == 0;
  const uint32_t per = pmode ? 2u : 1u;
  stage_symbols<BLOCK>(E, tile, S);
  const uint64_t P0 = tile * TILE;
  const uint64_t p0 = P0 + (uint64_t)threadIdx.x * ITEMS;
  int32_t val[ITEMS];
  const uint32_t cnt = thread_values<ITEMS, DELTA>(E, S, tile, p0, val);
  const uint32_t hd = cnt ? (uint32_t)((((unsigned long long)T.heads[(p0 >> 5) + 1] << 32) | T.heads[p0 >> 5]) >> (p0 & 31)) : 0u;
  // text bytes of my steps, line pieces included
  uint32_t ndp = 0;  // digit counts, 4 bits per step
  unsigned long long len = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    if ((uint32_t)k < cnt) {
      const uint32_t nd = dec_digits(abs32(val[k]));
      ndp |= nd << (4 * k);
      len += nd + per;
    }
  }
  const uint32_t edges = cnt ? (hd & ((2u << cnt) - 1u)) : 0u;
  if (edges) {
    for (int k = 0; k < ITEMS; ++k) {
      if ((uint32_t)k >= cnt) break;
      const bool fst = (hd >> k) & 1u, lst = (hd >> (k + 1)) & 1u;
      if (fst | lst) {
        const uint64_t t = trav_of(T.off, T.ntrav, p0 + k);
        if (fst) len += pre_len(T, t);
        if (lst) len += suf_len(T, t) - (pmode ? 1ull : 0ull);
      }
    }
  }
  unsigned long long total;
  const unsigned long long my = block_excl_sum<BLOCK>(len, total);
  const unsigned long long t0 = toff[tile];
  if (threadIdx.x == 0) {
    const unsigned long long want = tile + 1 < ntiles ? toff[tile + 1] : T.cap;
    if (t0 + total != want) atomicOr(T.err, kErrLength);
  }
  if (total <= kTextBuf) {
    const uint32_t nw = (uint32_t)(total / 4) + 2;
    // only words that receive OR-ed bytes need clearing: a word two threads
    // share holds a thread's first byte past the word's start (that thread
    // clears it), and the tile's last, partial word (the last thread clears
    // it); every other word is stored whole by one thread
    if (my & 3u) sbuf[(uint32_t)my >> 2] = 0;
    if (threadIdx.x == BLOCK - 1) sbuf[(uint32_t)total >> 2] = 0;
    __syncthreads();
    WordWriter wr;
    wr.init(sbuf, (uint32_t)my, nw);
    if (pmode && !edges) {
      // the common case: P-line steps with no line start or end among them,
      // every one digits, mark and comma
#pragma unroll 1
      for (int k = 0; k < ITEMS; ++k) {
        if ((uint32_t)k < cnt) {
          const int32_t v = val[k];
          const uint32_t av = abs32(v), nd = (ndp >> (4 * k)) & 15u;
          const uint32_t tail = (v < 0 ? '-' : '+') | ((uint32_t)',' << 8);
          if (nd <= 8) {
            const unsigned long long D = ascii_digits(av, nd);
            const uint32_t sh = 8u * nd;
            const unsigned long long s0 = sh < 64 ? D | ((unsigned long long)tail << sh) : D;
            const uint32_t s1 = sh > 48 ? (uint32_t)((unsigned long long)tail >> (64u - sh)) : 0u;
            wr.put12(s0, s1, nd + 2u);
          } else {
            wr.put_dec(av, nd);
            wr.put(tail, 2);
          }
        }
      }
    } else {
#pragma unroll 1  // a rolled loop keeps the kernel inside the instruction cache
    for (int k = 0; k < ITEMS; ++k) {
      if ((uint32_t)k < cnt) {
        const bool fst = (hd >> k) & 1u, lst = (hd >> (k + 1)) & 1u;
        uint64_t t = 0;
        if (fst | lst) t = trav_of(T.off, T.ntrav, p0 + k);
        if (fst)
          for (uint64_t q = T.meta.pre_off[t]; q < T.meta.pre_off[t + 1]; ++q) wr.put((uint8_t)T.meta.blob[q], 1);
        const int32_t v = val[k];
        const uint32_t av = abs32(v), nd = (ndp >> (4 * k)) & 15u;
        if (nd <= 8) {
          // the whole step in one append: digits, mark, comma (P) or mark, digits (W)
          const unsigned long long D = ascii_digits(av, nd);
          unsigned long long s0;
          uint32_t s1, len;
          if (pmode) {
            const uint32_t tail = (v < 0 ? '-' : '+') | (lst ? 0u : ((uint32_t)',' << 8));
            const uint32_t sh = 8u * nd;
            s0 = sh < 64 ? D | ((unsigned long long)tail << sh) : D;
            s1 = sh > 48 ? (uint32_t)((unsigned long long)tail >> (64u - sh)) : 0u;
            len = nd + (lst ? 1u : 2u);
          } else {
            s0 = (unsigned long long)(v < 0 ? '<' : '>') | (D << 8);
            s1 = (uint32_t)(D >> 56);
            len = nd + 1u;
          }
          wr.put12(s0, s1, len);
        } else if (pmode) {
          wr.put_dec(av, nd);
          const uint32_t mark = v < 0 ? '-' : '+';
          if (lst) wr.put(mark, 1);
          else wr.put(mark | ((uint32_t)',' << 8), 2);
        } else {
          wr.put(v < 0 ? '<' : '>', 1);
          wr.put_dec(av, nd);
        }
        if (lst)
          for (uint64_t q = T.meta.suf_off[t]; q < T.meta.suf_off[t + 1]; ++q) wr.put((uint8_t)T.meta.blob[q], 1);
      }
    }
    }
    wr.finish();
    if (wr.overflow) atomicOr(T.err, kErrLength);
    __syncthreads();
    if (t0 + total <= T.cap) block_copy_out<BLOCK>(reinterpret_cast<const char *>(sbuf), (uint32_t)total, text + t0);
    else if (threadIdx.x == 0) atomicOr(T.err, kErrLength);
    return;
  }
  // a tile with very long line pieces: bytes straight to global memory
  // (each thread's bytes end where the next thread's begin)
  unsigned long long o = t0 + my;
  char dec[10];
  auto put = [&](char c) {
    if (o < T.cap) text[o] = c;
    else atomicOr(T.err, kErrLength);
    ++o;
  };
#pragma unroll 1
  for (int k = 0; k < ITEMS; ++k) {
    if ((uint32_t)k < cnt) {
      const bool fst = (hd >> k) & 1u, lst = (hd >> (k + 1)) & 1u;
      uint64_t t = 0;
      if (fst | lst) t = trav_of(T.off, T.ntrav, p0 + k);
      if (fst)
        for (uint64_t q = T.meta.pre_off[t]; q < T.meta.pre_off[t + 1]; ++q) put(T.meta.blob[q]);
      const int32_t v = val[k];
      const uint32_t av = abs32(v), nd = (ndp >> (4 * k)) & 15u;
      put_dec(dec, av, nd);
      if (!pmode) put(v < 0 ? '<' : '>');
      for (uint32_t q = 0; q < nd; ++q) put(dec[q]);
      if (pmode) {
        put(v < 0 ? '-' : '+');
        if (!lst) put(',');
      }
      if (lst)
        for (uint64_t q = T.meta.suf_off[t]; q < T.meta.suf_off[t + 1]; ++q) put(T.meta.blob[q]);
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Line ends
// ---------------------------------------------------------------------------
// Positions of the '\n' bytes of text[0, n), unordered: out[0] counts them
// all, out[1 .. cap] holds the first cap found.  16 bytes per thread and
// step; the text buffer starts 16-byte aligned.
__global__ void k_find_newlines(const char *__restrict__ text, uint64_t n, unsigned long long *out, uint64_t cap) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * 16;
  for (uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) * 16; i < n; i += stride) {
    if (i + 16 <= n) {
      const uint4 v = *reinterpret_cast<const uint4 *>(text + i);
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        uint32_t eq = __vcmpeq4(w[k], 0x0A0A0A0Au);
        while (eq) {
          const int b = (__ffs(eq) - 1) >> 3;
          eq &= ~(0xFFu << (8 * b));
          const unsigned long long at = atomicAdd(&out[0], 1ull);
          if (at < cap) out[1 + at] = i + 4 * k + b;
        }
      }
    } else {
      for (uint64_t j = i; j < n; ++j)
        if (text[j] == '\n') {
          const unsigned long long at = atomicAdd(&out[0], 1ull);
          if (at < cap) out[1 + at] = j;
        }
    }
  }
}

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
                             int4 *rstat, int delta, uint32_t *built, uint32_t pass, DevStatus *status, int slot,
                             cudaStream_t st, uint64_t lo, uint64_t hi) {
  hi = std::min(hi, rv.nrules);
  if (lo >= hi) return;
  k_rule_prefix_pass<<<grid_for(hi - lo, kBlock, 152u * 32u), kBlock, 0, st>>>(first, second, rv, rpre, rstat,
                                                                               delta, built, pass, status, slot, lo,
                                                                               hi);
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

void launch_symbol_text(const ExpandSource &E, const TextSource &T, int delta, uint64_t *slen, uint8_t *sdig,
                        cudaStream_t st) {
  if (!E.m) return;
  if (delta)
    k_symbol_text<1><<<grid_for(E.m, kBlock), kBlock, 0, st>>>(E, T, slen, sdig);
  else
    k_symbol_text<0><<<grid_for(E.m, kBlock), kBlock, 0, st>>>(E, T, slen, sdig);
}

void launch_find_newlines(const char *text, uint64_t n, unsigned long long *out, uint64_t cap, cudaStream_t st) {
  if (!n) return;
  k_find_newlines<<<grid_for((n + 15) / 16, kBlock), kBlock, 0, st>>>(text, n, out, cap);
}

void launch_tile_text_off(const ExpandSource &E, const TextSource &T, int delta, const uint64_t *soff,
                          const uint8_t *sdig, uint64_t *toff, cudaStream_t st) {
  const uint64_t nt = expand_num_tiles(E.total);
  if (!nt) return;
  if (delta)
    k_tile_text_off<1><<<grid_for(nt, kBlock), kBlock, 0, st>>>(E, T, soff, sdig, nt, kExpandTile, toff);
  else
    k_tile_text_off<0><<<grid_for(nt, kBlock), kBlock, 0, st>>>(E, T, soff, sdig, nt, kExpandTile, toff);
}

void launch_text_write(const ExpandSource &E, const TextSource &T, int delta, const uint64_t *toff, char *text,
                       cudaStream_t st, uint64_t tile0, uint64_t tile1) {
  const uint64_t nt = expand_num_tiles(E.total);
  tile1 = std::min(tile1, nt);
  if (tile0 >= tile1) return;
  const unsigned grid = (unsigned)(tile1 - tile0);
  if (delta)
    k_text_write<kBlock, kExpandItems, 1><<<grid, kBlock, 0, st>>>(E, T, toff, text, tile0, nt);
  else
    k_text_write<kBlock, kExpandItems, 0><<<grid, kBlock, 0, st>>>(E, T, toff, text, tile0, nt);
}

}  // namespace gfz

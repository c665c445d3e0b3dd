// Compression-side kernels: delta coding, 2-mer counting, greedy replacement,
// used-rule collection, signed-order radix sort, id assignment and remap.
//
// Semantics follow the reference CPU path:
//   delta          src/codec/codec.cpp:45-76
//   counting       src/grammar/rule_generator.cpp:148-260 (pairs seen >= 2
//                  times, overlapping occurrences counted, never across
//                  traversals; the threshold argument has no effect)
//   replacement    src/grammar/path_encoder.cpp:13-84 (within one round the
//                  stack encoder equals greedy left-to-right replacement:
//                  inside each maximal run of candidate positions the even
//                  offsets from the run start are replaced)
//   id order       src/workflows/compression_workflow.cpp:630-680 (used rules
//                  sorted by signed packed key, ids next_id + rank)
#include "common.cuh"
#include "kernels.h"

namespace gfz {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ uint32_t warp_max_u32(uint32_t v) {
  return __reduce_max_sync(0xffffffffu, v);
}

// ---------------------------------------------------------------------------
// Delta encode + max |x|
// ---------------------------------------------------------------------------
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_delta_encode(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                                        uint64_t n, const uint64_t *__restrict__ off,
                                                        uint64_t ntrav, uint32_t *max_abs) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ int32_t sv[TILE + 1];
  __shared__ uint32_t hb[TILE / 32 + 2];
  __shared__ uint64_t s_tlo;
  const uint64_t base = (uint64_t)blockIdx.x * TILE;
  const uint32_t len = (uint32_t)min((uint64_t)TILE, n - base);
  for (uint32_t j = threadIdx.x; j < TILE / 32 + 2; j += BLOCK) hb[j] = 0;
  if (threadIdx.x == 0) sv[0] = base ? in[base - 1] : 0;
  for (uint32_t j = threadIdx.x; j < len; j += BLOCK) sv[1 + j] = in[base + j];
  mark_heads(off, ntrav, base, len, hb, &s_tlo);
  __syncthreads();
  uint32_t mx = 0;
  for (uint32_t j = threadIdx.x; j < len; j += BLOCK) {
    int32_t v = sv[1 + j];
    if (!bit_at(hb, j)) v = (int32_t)((uint32_t)v - (uint32_t)sv[j]);
    out[base + j] = v;
    mx = max(mx, abs32(v));
  }
  mx = warp_max_u32(mx);
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(max_abs, mx);
}

__global__ void k_max_abs(const int32_t *__restrict__ in, uint64_t n, uint32_t *max_abs) {
  uint32_t mx = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    mx = max(mx, abs32(in[i]));
  mx = warp_max_u32(mx);
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(max_abs, mx);
}

// ---------------------------------------------------------------------------
// Open-addressed pair table
// ---------------------------------------------------------------------------
constexpr uint32_t kMaxProbe = 4096;

struct InsertCounts {
  uint32_t fresh = 0, repeated = 0;
};

__device__ __forceinline__ void mark_repeated(uint32_t *flags, uint64_t h, InsertCounts &c) {
  if (!(flags[h] & kFlagRepeated)) {
    uint32_t old = atomicOr(&flags[h], kFlagRepeated);
    if (!(old & kFlagRepeated)) c.repeated++;
  }
}

// Inserts a canonical key; `known_repeat` marks it repeated unconditionally
// (another occurrence was seen in the same warp).  Returns false when the
// probe bound is exceeded.
__device__ __forceinline__ bool table_insert(const PairTable &tab, unsigned long long key, bool known_repeat,
                                             InsertCounts &c) {
  const uint64_t mask = tab.cap - 1;
  uint64_t h = hash64(key) & mask;
  for (uint32_t p = 0; p < kMaxProbe; ++p) {
    unsigned long long cur = tab.keys[h];
    if (cur == kEmptyKey) {
      unsigned long long old = atomicCAS(&tab.keys[h], kEmptyKey, key);
      if (old == kEmptyKey) {
        c.fresh++;
        if (known_repeat) mark_repeated(tab.flags, h, c);
        return true;
      }
      cur = old;
    }
    if (cur == key) {
      mark_repeated(tab.flags, h, c);
      return true;
    }
    h = (h + 1) & mask;
  }
  return false;
}

template <int BLOCK, int ITEMS, bool DEDUP>
__global__ void __launch_bounds__(BLOCK) k_count_pairs(const int32_t *__restrict__ s, uint64_t n,
                                                       const uint64_t *__restrict__ off, uint64_t ntrav,
                                                       PairTable tab, DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ int32_t sv[TILE + 1];
  __shared__ uint32_t hb[TILE / 32 + 2];
  __shared__ uint64_t s_tlo;
  __shared__ uint32_t s_fresh, s_rep;
  const uint64_t base = (uint64_t)blockIdx.x * TILE;
  const uint32_t len = (uint32_t)min((uint64_t)TILE, n - base);
  for (uint32_t j = threadIdx.x; j < TILE / 32 + 2; j += BLOCK) hb[j] = 0;
  if (threadIdx.x == 0) { s_fresh = 0; s_rep = 0; }
  const uint32_t ld = len + (base + len < n ? 1u : 0u);
  for (uint32_t j = threadIdx.x; j < ld; j += BLOCK) sv[j] = s[base + j];
  mark_heads(off, ntrav, base, len, hb, &s_tlo);
  __syncthreads();
  InsertCounts c;
  bool abort = (*(volatile uint32_t *)&status->err & kErrTableFull) != 0;
#pragma unroll 4
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t j = threadIdx.x + k * BLOCK;
    const bool valid = j < len && !bit_at(hb, j + 1);
    unsigned long long key = valid ? canon2(pack2(sv[j], sv[j + 1])) : kEmptyKey;
    bool leader = valid, rep = false;
    if (DEDUP) {
      const uint32_t m = __match_any_sync(0xffffffffu, key);
      leader = valid && (m & lanemask_lt()) == 0;
      rep = __popc(m) > 1;
    }
    if (leader && !abort) {
      if (!table_insert(tab, key, rep, c)) {
        atomicOr(&status->err, kErrTableFull);
        abort = true;
      }
    }
  }
  if (c.fresh) atomicAdd(&s_fresh, c.fresh);
  if (c.repeated) atomicAdd(&s_rep, c.repeated);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_fresh) atomicAdd(&status->u64[0], (unsigned long long)s_fresh);
    if (s_rep) atomicAdd(&status->u64[1], (unsigned long long)s_rep);
  }
}

// ---------------------------------------------------------------------------
// Greedy replacement (apply)
// ---------------------------------------------------------------------------
// Per-thread / per-tile aggregate of the run-parity recurrence
//   x_p = c_p ? !x_{p-1} : 0      (x_p = 1 <=> position p is replaced)
// as a function of the incoming x: outgoing x and number of replaced
// positions for x_in = 0 and x_in = 1.
struct ParAgg {
  uint32_t xo;    // bit0 = x_out(0), bit1 = x_out(1)
  uint32_t c0, c1;
};
__device__ __forceinline__ ParAgg par_identity() { return ParAgg{2u, 0u, 0u}; }
__device__ __forceinline__ uint32_t par_x(const ParAgg &a, uint32_t x) { return (a.xo >> x) & 1u; }
__device__ __forceinline__ uint32_t par_c(const ParAgg &a, uint32_t x) { return x ? a.c1 : a.c0; }
// a then b
__device__ __forceinline__ ParAgg par_compose(const ParAgg &a, const ParAgg &b) {
  const uint32_t a0 = par_x(a, 0), a1 = par_x(a, 1);
  ParAgg r;
  r.xo = par_x(b, a0) | (par_x(b, a1) << 1);
  r.c0 = a.c0 + par_c(b, a0);
  r.c1 = a.c1 + par_c(b, a1);
  return r;
}
__device__ __forceinline__ unsigned long long par_encode(const ParAgg &a) {
  return (unsigned long long)(a.xo & 3u) | ((unsigned long long)a.c0 << 2) | ((unsigned long long)a.c1 << 26);
}
__device__ __forceinline__ ParAgg par_decode(unsigned long long d) {
  return ParAgg{(uint32_t)(d & 3u), (uint32_t)((d >> 2) & 0xFFFFFFu), (uint32_t)((d >> 26) & 0xFFFFFFu)};
}
// Run-parity monoid for the look-back: state = (x after the tile, replaced
// positions so far).
struct ParState {
  uint32_t x;
  unsigned long long c;
};
struct ParOp {
  using T = ParAgg;
  using S = ParState;
  __device__ static T identity() { return par_identity(); }
  __device__ static T compose(const T &a, const T &b) { return par_compose(a, b); }
  __device__ static S apply(const T &f, const S &s) { return S{par_x(f, s.x), s.c + par_c(f, s.x)}; }
  __device__ static S initial() { return S{0u, 0ull}; }
  __device__ static unsigned long long encode_agg(const T &a) { return par_encode(a); }
  __device__ static T decode_agg(unsigned long long d) { return par_decode(d); }
  __device__ static unsigned long long encode_incl(const S &s) { return (unsigned long long)s.x | (s.c << 1); }
  __device__ static S decode_incl(unsigned long long d) { return S{(uint32_t)(d & 1u), d >> 1}; }
  __device__ static T shfl_down(const T &a, int o) {
    return T{__shfl_down_sync(0xffffffffu, a.xo, o), __shfl_down_sync(0xffffffffu, a.c0, o),
             __shfl_down_sync(0xffffffffu, a.c1, o)};
  }
  __device__ static T shfl0(const T &a) {
    return T{__shfl_sync(0xffffffffu, a.xo, 0), __shfl_sync(0xffffffffu, a.c0, 0), __shfl_sync(0xffffffffu, a.c1, 0)};
  }
};

__device__ __forceinline__ ParAgg par_shfl_up(const ParAgg &a, int delta) {
  ParAgg r;
  r.xo = __shfl_up_sync(0xffffffffu, a.xo, delta);
  r.c0 = __shfl_up_sync(0xffffffffu, a.c0, delta);
  r.c1 = __shfl_up_sync(0xffffffffu, a.c1, delta);
  return r;
}

template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_apply(const int32_t *__restrict__ s, uint64_t n,
                                                 const uint64_t *__restrict__ off, uint64_t ntrav, PairTable tab,
                                                 int32_t temp_base, int32_t *__restrict__ out,
                                                 uint64_t *__restrict__ new_off, unsigned long long *desc,
                                                 uint32_t *tile_counter, DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  constexpr int NW = BLOCK / 32;
  static_assert(TILE < (1u << 16), "tile must fit 16-bit local indices");
  static_assert(32 % ITEMS == 0, "a thread's candidate bits must sit in one bitmap word");
  __shared__ int32_t sv[padded_size(TILE + 1)];
  __shared__ int32_t so[padded_size(TILE)];
  __shared__ uint32_t sslot[padded_size(TILE)];  // table slot | orientation bit (31)
  __shared__ uint16_t lidx[padded_size(TILE)];
  __shared__ uint32_t hb[TILE / 32 + 2];
  __shared__ uint32_t scand[TILE / 32];  // candidate positions
  __shared__ uint32_t sused[TILE / 32];  // slot already flagged used
  __shared__ uint64_t s_tlo;
  __shared__ ParAgg s_warp[NW];
  __shared__ uint32_t s_in_x;
  __shared__ unsigned long long s_in_c;

  const uint32_t tile = claim_tile(tile_counter);
  const uint64_t base = (uint64_t)tile * TILE;
  const uint32_t len = (uint32_t)min((uint64_t)TILE, n - base);
  for (uint32_t j = threadIdx.x; j < TILE / 32 + 2; j += BLOCK) hb[j] = 0;
  const uint32_t ld = len + (base + len < n ? 1u : 0u);
  for (uint32_t j = threadIdx.x; j < ld; j += BLOCK) sv[padi(j)] = s[base + j];
  const uint64_t tlo = mark_heads(off, ntrav, base, len, hb, &s_tlo);
  __syncthreads();

  // Phase A: candidate lookup for positions j = tid + k * BLOCK; the ITEMS
  // first probes are issued back to back, then collisions are resolved.
  {
    const uint64_t mask = tab.cap - 1;
    unsigned long long ck[ITEMS];
    uint64_t hs[ITEMS];
    unsigned long long cur[ITEMS];
    uint32_t fwdb = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const uint32_t j = threadIdx.x + k * BLOCK;
      ck[k] = kEmptyKey;
      hs[k] = 0;
      cur[k] = kEmptyKey;
      if (j < len && !bit_at(hb, j + 1)) {
        const unsigned long long key = pack2(sv[padi(j)], sv[padi(j + 1)]);
        const unsigned long long r = rev2(key);
        const bool fwd = key_le(key, r);
        ck[k] = fwd ? key : r;
        fwdb |= (uint32_t)fwd << k;
        hs[k] = hash64(ck[k]) & mask;
        cur[k] = tab.keys[hs[k]];
      }
    }
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      if (ck[k] == kEmptyKey) continue;
      uint32_t p = 0;
      while (cur[k] != ck[k]) {
        if (cur[k] == kEmptyKey || ++p >= kMaxProbe) {
          atomicOr(&status->err, kErrLookupMiss);
          ck[k] = kEmptyKey;
          break;
        }
        hs[k] = (hs[k] + 1) & mask;
        cur[k] = tab.keys[hs[k]];
      }
    }
    // lanes of a warp cover one aligned 32-position word per k: build the
    // candidate / already-used bitmap words with ballots
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const uint32_t j = threadIdx.x + k * BLOCK;
      const uint32_t fl = ck[k] != kEmptyKey ? tab.flags[hs[k]] : 0u;
      const bool cand = (fl & kFlagRepeated) != 0;
      if (cand) sslot[padi(j)] = (uint32_t)hs[k] | (((fwdb >> k) & 1u) << 31);
      const uint32_t cw = __ballot_sync(0xffffffffu, cand);
      const uint32_t uw = __ballot_sync(0xffffffffu, cand && (fl & kFlagUsed));
      if ((threadIdx.x & 31) == 0) {
        scand[j >> 5] = cw;
        sused[j >> 5] = uw;
      }
    }
  }
  __syncthreads();

  // Phase B: the run-parity recurrence over my ITEMS consecutive positions
  const uint32_t j0 = threadIdx.x * ITEMS;
  const uint32_t cbits = j0 < TILE ? (scand[j0 >> 5] >> (j0 & 31)) & ((1u << ITEMS) - 1u) : 0u;

  // thread aggregate
  ParAgg a;
  {
    uint32_t x0 = 0, x1 = 1, c0 = 0, c1 = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const uint32_t c = (cbits >> k) & 1u;
      x0 = c & (x0 ^ 1u);
      x1 = c & (x1 ^ 1u);
      c0 += x0;
      c1 += x1;
    }
    a = ParAgg{x0 | (x1 << 1), c0, c1};
  }
  // block exclusive scan
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  ParAgg inc = a;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    ParAgg o = par_shfl_up(inc, d);
    if (lane >= d) inc = par_compose(o, inc);
  }
  ParAgg excl = par_shfl_up(inc, 1);
  if (lane == 0) excl = par_identity();
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  ParAgg wpre = par_identity(), total = par_identity();
  for (int w = 0; w < NW; ++w) {
    if (w == warp) wpre = total;
    total = par_compose(total, s_warp[w]);
  }
  excl = par_compose(wpre, excl);

  if (warp == 0) {
    const ParState in = warp_lookback<ParOp>(desc, tile, total, &status->err);
    if (lane == 0) {
      s_in_x = in.x;
      s_in_c = in.c;
    }
  }
  __syncthreads();
  const uint32_t in_x = s_in_x;
  const unsigned long long in_c = s_in_c;
  // Replay the recurrence over my positions from the carried-in state: which
  // positions are kept (not consumed) and which kept ones are replaced.
  const uint32_t x_init = par_x(excl, in_x);
  const uint32_t c_init = par_c(excl, in_x);  // replaced positions in this tile before j0
  uint32_t keptbits = 0, xbits = 0;
  {
    uint32_t x = x_init;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      if (j0 + k < len) {
        const uint32_t prev = x;
        x = ((cbits >> k) & 1u) & (prev ^ 1u);
        keptbits |= (prev ^ 1u) << k;
        xbits |= x << k;
      }
    }
  }
  // kept positions of the tile before j0: j0 minus the consumed ones, i.e.
  // the carried-in position plus the partner of every replaced position
  // before j0 except a replaced j0 - 1, whose partner is j0 itself
  const uint32_t kept_base = j0 - in_x - c_init + x_init;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    uint32_t mark = 0xFFFFFFFFu;  // slot to flag as used (none)
    if ((keptbits >> k) & 1u) {
      const uint32_t j = j0 + k;
      const uint32_t lo = kept_base + __popc(keptbits & ((1u << k) - 1u));
      int32_t v = sv[padi(j)];
      if ((xbits >> k) & 1u) {
        const uint32_t sl = sslot[padi(j)];
        const uint32_t slot = sl & 0x7FFFFFFFu;
        const int32_t sym = temp_base + (int32_t)slot;
        v = (sl >> 31) ? sym : neg32(sym);
        if (!bit_at(sused, j)) mark = slot;
      }
      so[padi(lo)] = v;
      lidx[padi(j)] = (uint16_t)lo;
    }
    // one store per distinct slot in the warp; every writer stores the same
    // value (candidate slots only ever gain the used flag here)
    const uint32_t peers = __match_any_sync(0xffffffffu, mark);
    if (mark != 0xFFFFFFFFu && (peers & lanemask_lt()) == 0) tab.flags[mark] = kFlagRepeated | kFlagUsed;
  }
  __syncthreads();
  // positions consumed inside the tile: the carried-in one (in_x) plus the
  // partner of every replaced position except a replaced last position,
  // whose partner opens the next tile (x_out)
  const uint32_t tile_rep = par_c(total, in_x);
  const uint32_t kept = len - in_x - tile_rep + par_x(total, in_x);
  const uint64_t out_base = base - in_c + in_x;
  for (uint32_t j = threadIdx.x; j < kept; j += BLOCK) out[out_base + j] = so[padi(j)];
  const bool last_tile = base + len == n;
  for (uint64_t t = tlo + threadIdx.x; t <= ntrav; t += BLOCK) {
    const uint64_t q = off[t];
    if (q < base + len) new_off[t] = out_base + lidx[padi((uint32_t)(q - base))];
    else if (last_tile && q == n) new_off[t] = out_base + kept;
    else break;
  }
  if (last_tile && threadIdx.x == 0) status->u64[2] = out_base + kept;
}

// ---------------------------------------------------------------------------
// Used-rule collection, radix sort, id assignment, remap
// ---------------------------------------------------------------------------
constexpr unsigned long long kSignFlip = 0x8000000000000000ULL;

__global__ void k_collect_used(PairTable tab, unsigned long long *keys_out, uint32_t *slots_out,
                               DevStatus *status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < tab.cap;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const bool used = (tab.flags[i] & kFlagUsed) != 0;
    const uint32_t act = __activemask();
    const uint32_t m = __ballot_sync(act, used);
    if (!m) continue;
    const int leader = __ffs(m) - 1;
    unsigned long long basepos = 0;
    if ((int)(threadIdx.x & 31) == leader) basepos = atomicAdd(&status->u64[3], (unsigned long long)__popc(m));
    basepos = __shfl_sync(act, basepos, leader);
    if (used) {
      const uint64_t p = basepos + __popc(m & lanemask_lt());
      keys_out[p] = tab.keys[i] ^ kSignFlip;
      slots_out[p] = (uint32_t)i;
    }
  }
}

__global__ void k_key_or_and(const unsigned long long *keys, uint64_t n, DevStatus *status) {
  unsigned long long o = 0, a = ~0ULL;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    o |= keys[i];
    a &= keys[i];
  }
  for (int d = 16; d > 0; d >>= 1) {
    o |= __shfl_xor_sync(0xffffffffu, o, d);
    a &= __shfl_xor_sync(0xffffffffu, a, d);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicOr(&status->u64[4], o);
    atomicAnd(&status->u64[5], a);
  }
}

constexpr int kRadixItems = 8;
constexpr uint32_t kRadixChunk = kBlock * kRadixItems;

__global__ void __launch_bounds__(kBlock) k_radix_hist(const unsigned long long *keys, uint64_t n, int shift,
                                                       uint32_t *hist, uint32_t nb) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t b0 = (uint64_t)blockIdx.x * kRadixChunk;
  for (int it = 0; it < kRadixItems; ++it) {
    const uint64_t i = b0 + it * kBlock + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xFF], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * nb + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of hist[0..e) in place by one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_hist(uint32_t *hist, uint64_t e) {
  __shared__ uint32_t part[1024];
  const uint64_t per = (e + 1023) / 1024;
  const uint64_t lo = threadIdx.x * per, hi = min(e, lo + per);
  uint32_t sum = 0;
  for (uint64_t i = lo; i < hi; ++i) sum += hist[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {
    uint32_t v = threadIdx.x >= (unsigned)d ? part[threadIdx.x - d] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - sum;
  for (uint64_t i = lo; i < hi; ++i) {
    const uint32_t v = hist[i];
    hist[i] = run;
    run += v;
  }
}

__global__ void __launch_bounds__(kBlock) k_radix_scatter(const unsigned long long *keys, const uint32_t *vals,
                                                          unsigned long long *keys_out, uint32_t *vals_out,
                                                          uint64_t n, int shift, const uint32_t *hist,
                                                          uint32_t nb) {
  constexpr int NW = kBlock / 32;
  __shared__ uint32_t base_off[256];
  __shared__ uint32_t running[256];
  __shared__ uint32_t wcnt[NW][256];
  base_off[threadIdx.x] = hist[(uint64_t)threadIdx.x * nb + blockIdx.x];
  running[threadIdx.x] = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t b0 = (uint64_t)blockIdx.x * kRadixChunk;
  for (int it = 0; it < kRadixItems; ++it) {
    for (int w = 0; w < NW; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const uint64_t i = b0 + it * kBlock + threadIdx.x;
    const bool valid = i < n;
    unsigned long long key = 0;
    uint32_t val = 0, d = 256;
    if (valid) {
      key = keys[i];
      val = vals[i];
      d = (uint32_t)((key >> shift) & 0xFF);
    }
    const uint32_t m = __match_any_sync(0xffffffffu, d);
    const uint32_t lrank = __popc(m & lanemask_lt());
    if (valid && lrank == 0) wcnt[warp][d] = __popc(m);
    __syncthreads();
    if (valid) {
      uint32_t pre = 0;
      for (int w = 0; w < warp; ++w) pre += wcnt[w][d];
      const uint32_t dst = base_off[d] + running[d] + pre + lrank;
      keys_out[dst] = key;
      vals_out[dst] = val;
    }
    __syncthreads();
    uint32_t add = 0;
    for (int w = 0; w < NW; ++w) add += wcnt[w][threadIdx.x];
    running[threadIdx.x] += add;
    __syncthreads();
    (void)lane;
  }
}

__global__ void k_assign_ids(const unsigned long long *sorted_keys, const uint32_t *sorted_slots, uint64_t u,
                             uint32_t next_id, PairTable tab, long long *rulebook) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < u; r += (uint64_t)gridDim.x * blockDim.x) {
    tab.vals[sorted_slots[r]] = next_id + (uint32_t)r;
    rulebook[r] = (long long)(sorted_keys[r] ^ kSignFlip);
  }
}

__global__ void k_remap(int32_t *s, uint64_t n, int32_t temp_base, const uint32_t *__restrict__ vals) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t v = s[i];
    const uint32_t a = abs32(v);
    if (a >= (uint32_t)temp_base) {
      const int32_t f = (int32_t)vals[a - (uint32_t)temp_base];
      s[i] = v < 0 ? neg32(f) : f;
    }
  }
}

// ---------------------------------------------------------------------------
// Append encoder
// ---------------------------------------------------------------------------
__global__ void k_build_rule_table(const int32_t *first, const int32_t *second, uint64_t lo, uint64_t hi,
                                   uint32_t start, PairTable tab, DevStatus *status) {
  const uint64_t mask = tab.cap - 1;
  for (uint64_t i = lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < hi;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = pack2(first[i], second[i]);
    if (key == kEmptyKey) {
      atomicOr(&status->err, kErrBadSymbol);
      continue;
    }
    uint64_t h = hash64(key) & mask;
    for (uint32_t p = 0;; ++p) {
      if (p >= kMaxProbe) {
        atomicOr(&status->err, kErrTableFull);
        break;
      }
      unsigned long long old = atomicCAS(&tab.keys[h], kEmptyKey, key);
      if (old == kEmptyKey || old == key) {
        // the first stored occurrence keeps its id (emplace semantics)
        atomicMin(&tab.vals[h], start + (uint32_t)(i - lo));
        break;
      }
      h = (h + 1) & mask;
    }
  }
}

__device__ __forceinline__ bool table_find(const PairTable &tab, unsigned long long key, uint32_t &id) {
  if (key == kEmptyKey) return false;
  const uint64_t mask = tab.cap - 1;
  uint64_t h = hash64(key) & mask;
  for (uint32_t p = 0; p < kMaxProbe; ++p) {
    const unsigned long long cur = tab.keys[h];
    if (cur == key) {
      id = tab.vals[h];
      return true;
    }
    if (cur == kEmptyKey) return false;
    h = (h + 1) & mask;
  }
  return false;
}

// The reference stack encoder (path_encoder.cpp:31-79): after each push the
// top pair is checked once, forward key first, then the reversed key; a
// match replaces the pair by +id / -id.  With a multi-round rulebook a new
// rule symbol can pair with the next push (cascade), exactly as on the CPU.
__global__ void k_stack_encode(int32_t *s, const uint64_t *off, uint64_t *len, uint64_t ntrav, PairTable tab,
                               DevStatus *status) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < ntrav;
       t += (uint64_t)gridDim.x * blockDim.x) {
    int32_t *seq = s + off[t];
    const uint64_t n = len[t];
    uint64_t top = 0;
    for (uint64_t i = 0; i < n; ++i) {
      seq[top++] = seq[i];
      if (top >= 2) {
        const unsigned long long k = pack2(seq[top - 2], seq[top - 1]);
        uint32_t id;
        if (table_find(tab, k, id)) {
          top -= 2;
          seq[top++] = (int32_t)id;
        } else if (table_find(tab, rev2(k), id)) {
          top -= 2;
          seq[top++] = neg32((int32_t)id);
        }
      }
    }
    len[t] = top;
  }
  (void)status;
}

__global__ void k_gather_ranges(const int32_t *src, const uint64_t *starts, const uint64_t *dst_off, uint64_t nr,
                                int32_t *dst) {
  // one block per range, strided copy
  for (uint64_t r = blockIdx.x; r < nr; r += gridDim.x) {
    const uint64_t s0 = starts[r], d0 = dst_off[r], l = dst_off[r + 1] - dst_off[r];
    for (uint64_t i = threadIdx.x; i < l; i += blockDim.x) dst[d0 + i] = src[s0 + i];
  }
}

inline unsigned grid_for(uint64_t n, int block, unsigned cap = 152u * 16u) {
  uint64_t g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (unsigned)g;
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
constexpr int kDeltaItems = 16;
constexpr int kCountItems = 16;
constexpr int kApplyItems = 8;

void launch_delta_encode(const int32_t *in, int32_t *out, uint64_t n, const uint64_t *off, uint64_t ntrav,
                         uint32_t *max_abs, cudaStream_t st) {
  if (!n) return;
  constexpr uint64_t TILE = kBlock * kDeltaItems;
  k_delta_encode<kBlock, kDeltaItems><<<(unsigned)((n + TILE - 1) / TILE), kBlock, 0, st>>>(in, out, n, off, ntrav,
                                                                                            max_abs);
}

void launch_max_abs(const int32_t *in, uint64_t n, uint32_t *max_abs, cudaStream_t st) {
  if (!n) return;
  k_max_abs<<<grid_for(n, kBlock), kBlock, 0, st>>>(in, n, max_abs);
}

void launch_count_pairs(const int32_t *s, uint64_t n, const uint64_t *off, uint64_t ntrav, PairTable tab,
                        DevStatus *status, bool warp_dedup, cudaStream_t st) {
  if (!n) return;
  constexpr uint64_t TILE = kBlock * kCountItems;
  const unsigned g = (unsigned)((n + TILE - 1) / TILE);
  if (warp_dedup)
    k_count_pairs<kBlock, kCountItems, true><<<g, kBlock, 0, st>>>(s, n, off, ntrav, tab, status);
  else
    k_count_pairs<kBlock, kCountItems, false><<<g, kBlock, 0, st>>>(s, n, off, ntrav, tab, status);
}

uint64_t apply_num_tiles(uint64_t n) {
  constexpr uint64_t TILE = kBlock * kApplyItems;
  return (n + TILE - 1) / TILE;
}

void launch_apply(const int32_t *s, uint64_t n, const uint64_t *off, uint64_t ntrav, PairTable tab,
                  int32_t temp_base, int32_t *out, uint64_t *new_off, unsigned long long *desc,
                  uint32_t *tile_counter, DevStatus *status, cudaStream_t st) {
  if (!n) return;
  k_apply<kBlock, kApplyItems><<<(unsigned)apply_num_tiles(n), kBlock, 0, st>>>(
      s, n, off, ntrav, tab, temp_base, out, new_off, desc, tile_counter, status);
}

void launch_collect_used(PairTable tab, unsigned long long *keys_out, uint32_t *slots_out, DevStatus *status,
                         cudaStream_t st) {
  k_collect_used<<<grid_for(tab.cap, kBlock), kBlock, 0, st>>>(tab, keys_out, slots_out, status);
}

void launch_key_or_and(const unsigned long long *keys, uint64_t n, DevStatus *status, cudaStream_t st) {
  if (!n) return;
  k_key_or_and<<<grid_for(n, kBlock, 304), kBlock, 0, st>>>(keys, n, status);
}

uint64_t radix_blocks(uint64_t n) { return (n + kRadixChunk - 1) / kRadixChunk; }

bool radix_sort_pairs(unsigned long long *keys, uint32_t *vals, unsigned long long *keys_tmp, uint32_t *vals_tmp,
                      uint64_t n, uint32_t byte_mask, uint32_t *hist, cudaStream_t st) {
  if (n <= 1) return false;
  const uint32_t nb = (uint32_t)radix_blocks(n);
  bool in_tmp = false;
  for (int b = 0; b < 8; ++b) {
    if (!((byte_mask >> b) & 1u)) continue;
    const unsigned long long *ki = in_tmp ? keys_tmp : keys;
    const uint32_t *vi = in_tmp ? vals_tmp : vals;
    unsigned long long *ko = in_tmp ? keys : keys_tmp;
    uint32_t *vo = in_tmp ? vals : vals_tmp;
    k_radix_hist<<<nb, kBlock, 0, st>>>(ki, n, 8 * b, hist, nb);
    k_scan_hist<<<1, 1024, 0, st>>>(hist, (uint64_t)nb * 256);
    k_radix_scatter<<<nb, kBlock, 0, st>>>(ki, vi, ko, vo, n, 8 * b, hist, nb);
    in_tmp = !in_tmp;
  }
  return in_tmp;
}

void launch_assign_ids(const unsigned long long *sorted_keys, const uint32_t *sorted_slots, uint64_t u,
                       uint32_t next_id, PairTable tab, long long *rulebook, cudaStream_t st) {
  if (!u) return;
  k_assign_ids<<<grid_for(u, kBlock), kBlock, 0, st>>>(sorted_keys, sorted_slots, u, next_id, tab, rulebook);
}

void launch_remap(int32_t *s, uint64_t n, int32_t temp_base, const uint32_t *vals, cudaStream_t st) {
  if (!n) return;
  k_remap<<<grid_for(n, kBlock), kBlock, 0, st>>>(s, n, temp_base, vals);
}

void launch_build_rule_table(const int32_t *first, const int32_t *second, uint64_t lo, uint64_t hi, uint32_t start,
                             PairTable tab, DevStatus *status, cudaStream_t st) {
  if (hi <= lo) return;
  k_build_rule_table<<<grid_for(hi - lo, kBlock), kBlock, 0, st>>>(first, second, lo, hi, start, tab, status);
}

void launch_stack_encode(int32_t *s, const uint64_t *off, uint64_t *len, uint64_t ntrav, PairTable tab,
                         DevStatus *status, cudaStream_t st) {
  if (!ntrav) return;
  k_stack_encode<<<grid_for(ntrav, 32), 32, 0, st>>>(s, off, len, ntrav, tab, status);
}

void launch_gather_ranges(const int32_t *src, const uint64_t *starts, const uint64_t *dst_off, uint64_t nr,
                          int32_t *dst, cudaStream_t st) {
  if (!nr) return;
  k_gather_ranges<<<(unsigned)(nr < 4096 ? nr : 4096), kBlock, 0, st>>>(src, starts, dst_off, nr, dst);
}

}  // namespace gfz

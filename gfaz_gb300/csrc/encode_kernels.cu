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

// Max-reduces v over the block into *dst with one global atomic per block
// (one per warp would serialise on the single address).  All threads call it.
template <int BLOCK>
__device__ __forceinline__ void block_max_to(uint32_t v, uint32_t *dst) {
  __shared__ uint32_t s_max;
  if (threadIdx.x == 0) s_max = 0;
  __syncthreads();
  v = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && v) atomicMax(&s_max, v);
  __syncthreads();
  if (threadIdx.x == 0 && s_max) atomicMax(dst, s_max);
}

// ---------------------------------------------------------------------------
// Delta encode + max |x|
// ---------------------------------------------------------------------------
// One tile of BLOCK * ITEMS steps per block.  The tile and the step before it
// are staged in shared memory; each thread then turns 4 consecutive steps
// into deltas and writes them as one 16-byte vector.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_delta_encode(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                                        uint64_t n, const uint64_t *__restrict__ off,
                                                        uint64_t ntrav, uint32_t *max_abs) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ __align__(16) int32_t sv[TILE + 4];  // sv[4 + j] = in[base + j], sv[3] = in[base - 1]
  __shared__ uint32_t hb[TILE / 32 + 2];
  __shared__ uint64_t s_tlo;
  const uint64_t base = (uint64_t)blockIdx.x * TILE;
  const uint32_t len = (uint32_t)min((uint64_t)TILE, n - base);
  for (uint32_t j = threadIdx.x; j < TILE / 32 + 2; j += BLOCK) hb[j] = 0;
  if (threadIdx.x == 0) sv[3] = base ? in[base - 1] : 0;
  stage_in<BLOCK, TILE>(in + base, len, sv + 4);
  mark_heads(off, ntrav, base, len, hb, &s_tlo);
  __syncthreads();
  uint32_t mx = 0;
  const bool vec = len == TILE && (reinterpret_cast<uintptr_t>(out + base) & 15u) == 0;
  for (uint32_t g = threadIdx.x; 4 * g < len; g += BLOCK) {
    const uint32_t j = 4 * g;
    const int4 c = *reinterpret_cast<const int4 *>(&sv[4 + j]);
    const uint32_t h = (hb[j >> 5] >> (j & 31)) & 0xFu;  // traversal starts among the 4
    int4 d;
    d.x = (h & 1u) ? c.x : (int32_t)((uint32_t)c.x - (uint32_t)sv[3 + j]);
    d.y = (h & 2u) ? c.y : (int32_t)((uint32_t)c.y - (uint32_t)c.x);
    d.z = (h & 4u) ? c.z : (int32_t)((uint32_t)c.z - (uint32_t)c.y);
    d.w = (h & 8u) ? c.w : (int32_t)((uint32_t)c.w - (uint32_t)c.z);
    if (vec) {
      reinterpret_cast<int4 *>(out + base)[g] = d;
      mx = max(mx, max(max(abs32(d.x), abs32(d.y)), max(abs32(d.z), abs32(d.w))));
    } else {
      const int32_t dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (j + e < len) {
          out[base + j + e] = dv[e];
          mx = max(mx, abs32(dv[e]));
        }
    }
  }
  block_max_to<BLOCK>(mx, max_abs);
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_max_abs(const int32_t *__restrict__ in, uint64_t n, uint32_t *max_abs) {
  uint32_t mx = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    mx = max(mx, abs32(in[i]));
  block_max_to<BLOCK>(mx, max_abs);
}

// ---------------------------------------------------------------------------
// Open-addressed pair table (linear probing over 16-byte slots)
// ---------------------------------------------------------------------------
constexpr uint32_t kMaxProbe = 4096;
// Flipping the sign bit makes unsigned order of packed keys their signed order.
constexpr unsigned long long kSignFlip = 0x8000000000000000ULL;

__device__ __forceinline__ void load_slot(const PairSlot *p, unsigned long long &key, uint32_t &flags) {
  const ulonglong2 w = *reinterpret_cast<const ulonglong2 *>(p);
  key = w.x;
  flags = (uint32_t)w.y;
}

__global__ void k_copy_bytes(const char *__restrict__ src, char *__restrict__ dst, uint64_t n) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t done = 0;
  if ((((uintptr_t)src | (uintptr_t)dst) & 15u) == 0) {
    const uint64_t words = n / 16;
    for (uint64_t i = tid; i < words; i += stride)
      reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(src)[i];
    done = words * 16;
  }
  for (uint64_t i = done + tid; i < n; i += stride) dst[i] = src[i];
}

__global__ void k_zero_bytes(char *dst, uint64_t n) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t gap = (16u - ((uintptr_t)dst & 15u)) & 15u;
  const uint64_t lead = gap < n ? gap : n;
  for (uint64_t i = tid; i < lead; i += stride) dst[i] = 0;
  const uint64_t words = (n - lead) / 16;
  uint4 *w = reinterpret_cast<uint4 *>(dst + lead);
  for (uint64_t i = tid; i < words; i += stride) w[i] = make_uint4(0u, 0u, 0u, 0u);
  for (uint64_t i = lead + words * 16 + tid; i < n; i += stride) dst[i] = 0;
}

__global__ void k_table_clear(PairTable tab, uint32_t val_init, uint32_t *bits_a, uint32_t *bits_b) {
  const uint4 empty = make_uint4((uint32_t)kEmptyKey, (uint32_t)(kEmptyKey >> 32), 0u, val_init);
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = tid; i < tab.cap; i += stride) reinterpret_cast<uint4 *>(tab.slots)[i] = empty;
  const uint64_t words = (tab.cap + 31) / 32;
  for (uint64_t i = tid; i < words; i += stride) {
    if (bits_a) bits_a[i] = 0;
    if (bits_b) bits_b[i] = 0;
  }
}

struct InsertCounts {
  uint32_t fresh = 0, repeated = 0;
};

// Sets the repeated flag of slot h; counts the key if this call set it, and
// then also sets bit h of rep_bits (when given: the repeated slots as a
// bitmap, cap bits, read by the slot-reference classification).
__device__ __forceinline__ void mark_repeated(const PairTable &tab, uint32_t h, uint32_t *rep_bits,
                                              InsertCounts &c) {
  const uint32_t old = atomicOr(&tab.slots[h].flags, kFlagRepeated);
  if (!(old & kFlagRepeated)) {
    c.repeated++;
    if (rep_bits) atomicOr(&rep_bits[h >> 5], 1u << (h & 31));
  }
}

// Inserts one occurrence of canonical `key` starting at slot h, whose
// contents (cur, fl) were already loaded.  `more` = the caller folded a
// second occurrence into this call.  On return h is the key's slot.
// Returns false when the probe bound is exceeded.
__device__ __forceinline__ bool insert_at(const PairTable &tab, unsigned long long key, bool more, uint32_t &h,
                                          unsigned long long cur, uint32_t fl, uint32_t *rep_bits, InsertCounts &c) {
  const uint32_t mask = (uint32_t)(tab.cap - 1);
  for (uint32_t p = 0; p < kMaxProbe; ++p) {
    if (cur == kEmptyKey) {
      const unsigned long long old = atomicCAS(&tab.slots[h].key, kEmptyKey, key);
      if (old == kEmptyKey) {
        c.fresh++;
        if (more) mark_repeated(tab, h, rep_bits, c);
        return true;
      }
      cur = old;
      fl = 0;
    }
    if (cur == key) {
      // a stale flag word can only miss bits, so a set bit needs no atomic
      if (!(fl & kFlagRepeated)) mark_repeated(tab, h, rep_bits, c);
      return true;
    }
    h = (h + 1) & mask;
    load_slot(&tab.slots[h], cur, fl);
  }
  return false;
}

// Slot references (one u32 per stream position, written by the counts when
// asked): the slot of the pair starting at the position, with bit 31 set
// when the pair is the reverse of its canonical key; kNoPair where no pair
// starts (a traversal's last step).  Tables up to 2^30 slots.
constexpr uint32_t kNoPair = 0xFFFFFFFFu;
constexpr uint32_t kRevBit = 0x80000000u;

// The ITEMS + 1 steps a thread looks at: positions j0 .. j0 + ITEMS of the
// staged tile (two 16-byte shared loads plus one element).
template <int ITEMS>
__device__ __forceinline__ void thread_steps(const int32_t *sv, uint32_t j0, int32_t (&v)[ITEMS + 1]) {
  static_assert(ITEMS == 8, "eight consecutive steps per thread");
  const int4 a = *reinterpret_cast<const int4 *>(&sv[j0]);
  const int4 b = *reinterpret_cast<const int4 *>(&sv[j0 + 4]);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  v[8] = sv[j0 + 8];
}

// Counts one staged tile: thread t handles the pairs starting at positions
// j0 = t * ITEMS .. j0 + ITEMS - 1.  A run of equal keys inside a thread is
// inserted once (flagged repeated when longer than one); with DEDUP the
// lanes of a warp also fold equal keys of the same item index.
// The slot references of K consecutive positions (see kNoPair): h = the
// slots of the inserted positions, whose runs' dropped positions take their
// predecessor's; cnt of them are stored at dst (16-byte stores when whole
// and aligned).
template <int K>
__device__ __forceinline__ void store_srefs(uint32_t *dst, uint32_t cnt, uint32_t validb, uint32_t dropped,
                                            uint32_t revb, const uint32_t (&h)[K]) {
  uint32_t r[K];
  uint32_t prev = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const uint32_t slot = ((dropped >> k) & 1u) ? prev : h[k];
    prev = slot;
    r[k] = ((validb >> k) & 1u) ? (slot | (((revb >> k) & 1u) ? kRevBit : 0u)) : kNoPair;
  }
  if (cnt == (uint32_t)K && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
#pragma unroll
    for (int k = 0; k < K; k += 4)  // evict-first, as the table is what L2 should hold
      __stcs(reinterpret_cast<uint4 *>(dst + k), make_uint4(r[k], r[k + 1], r[k + 2], r[k + 3]));
  } else {
#pragma unroll
    for (int k = 0; k < K; ++k)
      if ((uint32_t)k < cnt) dst[k] = r[k];
  }
}

// len = positions of the tile with a successor in the stream, tlen = all
// its positions.  With sref (not with DEDUP: a lane whose key another lane
// inserted does not learn the slot) the tile's slot references are stored
// at sref[j] for tile position j; rep_bits as in mark_repeated.
template <int ITEMS, bool DEDUP>
__device__ __forceinline__ void count_tile(const int32_t *sv, const uint32_t *hb, uint32_t len, uint32_t tlen,
                                           const PairTable &tab, DevStatus *status, InsertCounts &c,
                                           uint32_t *sref, uint32_t *rep_bits) {
  const uint32_t j0 = threadIdx.x * ITEMS;
  int32_t v[ITEMS + 1];
  thread_steps<ITEMS>(sv, j0, v);
  const uint32_t hd = bits_from(hb, j0);  // bit k: position j0 + k starts a traversal
  unsigned long long key[ITEMS];
  uint32_t validb = 0, sameb = 0, revb = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const bool valid = j0 + k < len && !((hd >> (k + 1)) & 1u);
    const unsigned long long f = pack2(v[k], v[k + 1]);
    key[k] = canon2(f);
    revb |= (uint32_t)(key[k] != f) << k;
    validb |= (uint32_t)valid << k;
    if (k > 0) sameb |= (uint32_t)(key[k] == key[k - 1]) << k;
  }
  // drop a position whose key equals its valid predecessor's; the first of
  // the run then carries the extra occurrence
  const uint32_t dropped = validb & (validb << 1) & sameb;
  uint32_t insb = validb & ~dropped;
  uint32_t moreb = insb & (dropped >> 1);
  if (DEDUP) {
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const bool ins = (insb >> k) & 1u;
      const uint32_t m = __match_any_sync(0xffffffffu, ins ? key[k] : kEmptyKey);
      if (ins && (m & lanemask_lt()) != 0) insb &= ~(1u << k);  // a lower lane inserts it
      else if (ins && __popc(m) > 1) moreb |= 1u << k;
    }
  }
  if ((*(volatile uint32_t *)&status->err & kErrTableFull) != 0) insb = 0;
  const uint32_t mask = (uint32_t)(tab.cap - 1);
  uint32_t h[ITEMS];
  unsigned long long cur[ITEMS];
  uint32_t fl[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    h[k] = hash_pair(key[k]) & mask;
    cur[k] = kEmptyKey;
    fl[k] = 0;
    if ((insb >> k) & 1u) load_slot(&tab.slots[h[k]], cur[k], fl[k]);
  }
  bool abort = false;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    if (((insb >> k) & 1u) && !abort) {
      if (!insert_at(tab, key[k], (moreb >> k) & 1u, h[k], cur[k], fl[k], rep_bits, c)) {
        atomicOr(&status->err, kErrTableFull);
        abort = true;
      }
    }
  }
  if (!DEDUP && sref && j0 < tlen) store_srefs<ITEMS>(sref + j0, min((uint32_t)ITEMS, tlen - j0), validb, dropped, revb, h);
}

// Persistent: block b counts tiles b, b + gridDim.x, ..., the next tile
// streaming into the other pipeline stage while this one is counted.
template <int BLOCK, int ITEMS, bool DEDUP>
__global__ void __launch_bounds__(BLOCK, 4) k_count_pairs(const int32_t *__restrict__ s, uint64_t n,
                                                          const uint32_t *__restrict__ heads, uint64_t head_words,
                                                          PairTable tab, DevStatus *status, uint32_t *sref,
                                                          uint32_t *rep_bits) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  __shared__ __align__(128) TilePipe<TILE> P;
  __shared__ uint32_t s_fresh, s_rep;
  const uint64_t ntiles = (n + TILE - 1) / TILE;
  uint64_t tile = blockIdx.x;
  if (tile >= ntiles) return;
  if (threadIdx.x == 0) {
    mbar_init(&P.bar[0], 1);
    mbar_init(&P.bar[1], 1);
    mbar_init_fence();
    s_fresh = 0;
    s_rep = 0;
  }
  __syncthreads();
  uint32_t phases = 0;
  bool bulk_cur = pipe_issue<BLOCK, TILE>(P, 0, tile, s, n, heads, head_words);
  InsertCounts c;
  for (int b = 0;; b ^= 1) {
    const uint64_t next = tile + gridDim.x;
    const bool has_next = next < ntiles;
    const bool bulk_next = has_next && pipe_issue<BLOCK, TILE>(P, b ^ 1, next, s, n, heads, head_words);
    if (!pipe_wait<TILE>(P, b, bulk_cur, phases)) {
      // a bulk copy did not land: report, let the other stage's copy finish
      if (threadIdx.x == 0) atomicOr(&status->err, kErrTimeout);
      if (bulk_next) mbar_wait(&P.bar[b ^ 1], (phases >> (b ^ 1)) & 1u);
      return;
    }
    const uint32_t len = (uint32_t)min((uint64_t)TILE, n - tile * TILE);
    // pairs start at positions with a successor inside the stream (the head
    // bitmap marks position n too, but a caller may pass a shorter n)
    const uint32_t plen = tile * TILE + len < n ? len : len - 1;
    count_tile<ITEMS, DEDUP>(P.sv[b], P.hb[b], plen, len, tab, status, c, sref ? sref + tile * TILE : nullptr,
                             rep_bits);
    pipe_release();
    if (!has_next) break;
    tile = next;
    bulk_cur = bulk_next;
  }
  const uint32_t f = __reduce_add_sync(0xffffffffu, c.fresh);
  const uint32_t r = __reduce_add_sync(0xffffffffu, c.repeated);
  if ((threadIdx.x & 31) == 0) {
    if (f) atomicAdd(&s_fresh, f);
    if (r) atomicAdd(&s_rep, r);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_fresh) atomicAdd(&status->u64[0], (unsigned long long)s_fresh);
    if (s_rep) atomicAdd(&status->u64[1], (unsigned long long)s_rep);
  }
}

// The count for streams whose pairs are mostly new (late rounds): one pair
// per thread, read straight from global memory, with no staging and no
// block barrier, so every insert is an independent chain and the memory
// system sees as many of them at once as threads are resident.
__global__ void __launch_bounds__(kBlock) k_count_flat(const int32_t *__restrict__ s, uint64_t n,
                                                       const uint32_t *__restrict__ heads, PairTable tab,
                                                       DevStatus *status, uint32_t *sref, uint32_t *rep_bits) {
  __shared__ uint32_t s_fresh, s_rep;
  if (threadIdx.x == 0) {
    s_fresh = 0;
    s_rep = 0;
  }
  __syncthreads();
  InsertCounts c;
  const uint32_t mask = (uint32_t)(tab.cap - 1);
  uint32_t it = 0;
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
       p += (uint64_t)gridDim.x * blockDim.x) {
    // a full table (some chain ran past the probe limit) ends every thread
    // within 16 of its pairs
    if ((++it & 15u) == 0 && (*(volatile uint32_t *)&status->err & kErrTableFull)) break;
    const uint64_t q = p + 1;
    if (q >= n || ((heads[q >> 5] >> (q & 31)) & 1u)) {  // no pair: q ends the stream or opens a traversal
      if (sref) sref[p] = kNoPair;
      continue;
    }
    const unsigned long long f = pack2(s[p], s[q]);
    const unsigned long long key = canon2(f);
    uint32_t h = hash_pair(key) & mask;
    unsigned long long cur;
    uint32_t fl;
    load_slot(&tab.slots[h], cur, fl);
    if (!insert_at(tab, key, false, h, cur, fl, rep_bits, c)) {
      atomicOr(&status->err, kErrTableFull);
      break;
    }
    if (sref) sref[p] = h | (key != f ? kRevBit : 0u);
  }
  const uint32_t f = __reduce_add_sync(0xffffffffu, c.fresh);
  const uint32_t r = __reduce_add_sync(0xffffffffu, c.repeated);
  if ((threadIdx.x & 31) == 0) {
    if (f) atomicAdd(&s_fresh, f);
    if (r) atomicAdd(&s_rep, r);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_fresh) atomicAdd(&status->u64[0], (unsigned long long)s_fresh);
    if (s_rep) atomicAdd(&status->u64[1], (unsigned long long)s_rep);
  }
}

// Four consecutive pairs per thread, read straight from global memory;
// a run of equal keys inside the thread is inserted once (flagged repeated
// when longer than one), as in the tiled kernel, but with no barrier.
// Six resident blocks per SM (at most 40 registers, a few bytes spilled):
// more warps to cover the slot loads' latency than the 52 registers it
// takes unbounded allow (round 1 1.78 against 1.86 ms).
__global__ void __launch_bounds__(kBlock, 6) k_count_flat4(const int32_t *__restrict__ s, uint64_t n,
                                                        const uint32_t *__restrict__ heads, PairTable tab,
                                                        DevStatus *status, uint32_t *sref, uint32_t *rep_bits) {
  constexpr int K = 4;
  __shared__ uint32_t s_fresh, s_rep;
  if (threadIdx.x == 0) {
    s_fresh = 0;
    s_rep = 0;
  }
  __syncthreads();
  InsertCounts c;
  const uint32_t mask = (uint32_t)(tab.cap - 1);
  const bool aligned = (reinterpret_cast<uintptr_t>(s) & 15u) == 0;
  bool full = false;
  uint32_t it = 0;
  for (uint64_t p0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) * K; p0 < n && !full;
       p0 += (uint64_t)gridDim.x * blockDim.x * K) {
    if ((++it & 3u) == 0 && (*(volatile uint32_t *)&status->err & kErrTableFull)) break;  // as in k_count_flat
    int32_t v[K + 1];
    if (aligned && p0 + K < n) {
      // evict-first: the steps are read once here, and L2 is better left to
      // the table
      const int4 a = __ldcs(reinterpret_cast<const int4 *>(s + p0));
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
      v[4] = s[p0 + K];
    } else {
#pragma unroll
      for (int k = 0; k <= K; ++k) v[k] = p0 + k < n ? s[p0 + k] : 0;
    }
    const uint32_t w = (uint32_t)(p0 >> 5);
    const uint32_t hd = (uint32_t)((((unsigned long long)heads[w + 1] << 32) | heads[w]) >> (p0 & 31));
    unsigned long long key[K];
    uint32_t validb = 0, sameb = 0, revb = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const unsigned long long f = pack2(v[k], v[k + 1]);
      key[k] = canon2(f);
      revb |= (uint32_t)(key[k] != f) << k;
      validb |= (uint32_t)(p0 + k + 1 < n && !((hd >> (k + 1)) & 1u)) << k;
      if (k > 0) sameb |= (uint32_t)(key[k] == key[k - 1]) << k;
    }
    const uint32_t dropped = validb & (validb << 1) & sameb;
    const uint32_t insb = validb & ~dropped;
    const uint32_t moreb = insb & (dropped >> 1);
    uint32_t h[K];
    unsigned long long cur[K];
    uint32_t fl[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      h[k] = hash_pair(key[k]) & mask;
      cur[k] = kEmptyKey;
      fl[k] = 0;
      if ((insb >> k) & 1u) load_slot(&tab.slots[h[k]], cur[k], fl[k]);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (((insb >> k) & 1u) && !full &&
          !insert_at(tab, key[k], (moreb >> k) & 1u, h[k], cur[k], fl[k], rep_bits, c)) {
        atomicOr(&status->err, kErrTableFull);
        full = true;
      }
    }
    if (sref && !full) store_srefs<K>(sref + p0, (uint32_t)min((uint64_t)K, n - p0), validb, dropped, revb, h);
  }
  const uint32_t f = __reduce_add_sync(0xffffffffu, c.fresh);
  const uint32_t r = __reduce_add_sync(0xffffffffu, c.repeated);
  if ((threadIdx.x & 31) == 0) {
    if (f) atomicAdd(&s_fresh, f);
    if (r) atomicAdd(&s_rep, r);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_fresh) atomicAdd(&status->u64[0], (unsigned long long)s_fresh);
    if (s_rep) atomicAdd(&status->u64[1], (unsigned long long)s_rep);
  }
}

// Traversal-head bitmap: bit off[t] for every t <= ntrav (bits cleared).
__global__ void k_head_bits(const uint64_t *__restrict__ off, uint64_t ntrav, uint32_t *bits) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t <= ntrav; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t q = off[t];
    atomicOr(&bits[q >> 5], 1u << (q & 31));
  }
}

// Head bitmap of the positions lo .. lo + span of a longer stream: bit q - lo
// for every traversal start q = off[t] in that range (bits cleared).
__global__ void k_head_bits_range(const uint64_t *__restrict__ off, uint64_t ntrav, uint64_t lo, uint64_t span,
                                  uint32_t *bits) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t <= ntrav; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t q = off[t];
    if (q >= lo && q - lo <= span) atomicOr(&bits[(q - lo) >> 5], 1u << ((q - lo) & 31));
  }
}

// One delta round over a chunk: in[j + 1] is the step at chunk position j
// and in[0] the step before the chunk (any value when the chunk opens the
// stream); out[j] = in[j + 1] - in[j] unless position j opens a traversal
// (heads, chunk-relative).  Max |out| folds into *max_abs.
__global__ void __launch_bounds__(kBlock) k_delta_chunk(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                                        uint64_t len, const uint32_t *__restrict__ heads,
                                                        uint32_t *max_abs) {
  uint32_t m = 0;
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < len; j += (uint64_t)gridDim.x * blockDim.x) {
    const int32_t x = in[j + 1];
    const int32_t d = ((heads[j >> 5] >> (j & 31)) & 1u) ? x : (int32_t)((uint32_t)x - (uint32_t)in[j]);
    out[j] = d;
    m = max(m, abs32(d));
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(max_abs, m);
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

// First traversal starting at or after each tile: tile_trav[k] = the first
// t with off[t] >= k * tile (off sorted, off[ntrav] = n).
__global__ void k_tile_trav(const uint64_t *__restrict__ off, uint64_t ntrav, uint64_t ntiles, uint32_t tile,
                            uint64_t *tile_trav) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < ntiles; k += (uint64_t)gridDim.x * blockDim.x)
    tile_trav[k] = lower_bound_u64(off, ntrav, k * (uint64_t)tile);
}

// Greedy replacement in three passes, so that no tile waits on another:
//  classify: per tile, the candidate bits of its positions (one byte per
//            thread) and the tile's run-parity aggregate;
//  states:   exclusive scan of the tile aggregates into the carried-in state
//            (x, replaced count) of every tile;
//  emit:     per tile, the replay of the recurrence from its carried-in
//            state, a second lookup of the positions it replaces, and the
//            compacted output.
// Thread t owns positions j0 = t * ITEMS .. j0 + ITEMS - 1 of a tile.

// Lookup of the pairs at positions j0 + k (k < ITEMS) with bit k of `want`
// set: canonical key, slot (table index) and flag word; misses flag
// kErrLookupMiss.  All first probes are issued before any is resolved.
template <int ITEMS>
__device__ __forceinline__ void lookup_pairs(const int32_t (&v)[ITEMS + 1], uint32_t want, const PairTable &tab,
                                             uint32_t (&slot)[ITEMS], uint32_t (&fl)[ITEMS], uint32_t &fwdb,
                                             DevStatus *status) {
  const uint32_t mask = (uint32_t)(tab.cap - 1);
  unsigned long long key[ITEMS], cur[ITEMS];
  fwdb = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    key[k] = 0;
    cur[k] = 0;
    slot[k] = 0;
    fl[k] = 0;
    if ((want >> k) & 1u) {
      const unsigned long long f = pack2(v[k], v[k + 1]);
      const unsigned long long r = pack2(neg32(v[k + 1]), neg32(v[k]));
      const bool fw = key_le(f, r);
      key[k] = fw ? f : r;
      fwdb |= (uint32_t)fw << k;
      slot[k] = hash_pair(key[k]) & mask;
      load_slot(&tab.slots[slot[k]], cur[k], fl[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    uint32_t p = 0;
    while (cur[k] != key[k]) {
      if (cur[k] == kEmptyKey || ++p >= kMaxProbe) {
        atomicOr(&status->err, kErrLookupMiss);
        fl[k] = 0;
        break;
      }
      slot[k] = (slot[k] + 1) & mask;
      load_slot(&tab.slots[slot[k]], cur[k], fl[k]);
    }
  }
}

__host__ __device__ constexpr uint32_t par_pack8(uint32_t cbits) {
  uint32_t x0 = 0, x1 = 1, c0 = 0, c1 = 0;
  for (int k = 0; k < 8; ++k) {
    const uint32_t c = (cbits >> k) & 1u;
    x0 = c & (x0 ^ 1u);
    x1 = c & (x1 ^ 1u);
    c0 += x0;
    c1 += x1;
  }
  return x0 | (x1 << 1) | (c0 << 2) | (c1 << 6);
}
// The aggregate of every 8-position candidate pattern, packed as
// x_out(0) | x_out(1) << 1 | c0 << 2 | c1 << 6 (1 KB, read through L1):
// one load in place of the eight-step recurrence.
struct Par8Table {
  uint32_t v[256];
  constexpr Par8Table() : v() {
    for (uint32_t b = 0; b < 256; ++b) v[b] = par_pack8(b);
  }
};
__device__ const Par8Table g_par8 = Par8Table();

// The replay of eight positions from a carried-in x: index cbits | x_in << 8,
// value xbits | keptbits << 8 (x_p = c_p & !x_{p-1}; a position is kept
// unless its predecessor was replaced).
__host__ __device__ constexpr uint32_t replay8(uint32_t idx) {
  uint32_t x = idx >> 8, xbits = 0, kept = 0;
  for (int k = 0; k < 8; ++k) {
    const uint32_t prev = x;
    x = ((idx >> k) & 1u) & (prev ^ 1u);
    kept |= (prev ^ 1u) << k;
    xbits |= x << k;
  }
  return xbits | (kept << 8);
}
struct Replay8Table {
  uint32_t v[512];
  constexpr Replay8Table() : v() {
    for (uint32_t i = 0; i < 512; ++i) v[i] = replay8(i);
  }
};
__device__ const Replay8Table g_replay8 = Replay8Table();

__device__ __forceinline__ ParAgg par_of_bits(uint32_t cbits, int items) {
  if (items == 8) {
    const uint32_t t = __ldg(&g_par8.v[cbits & 0xFFu]);
    return ParAgg{t & 3u, (t >> 2) & 15u, (t >> 6) & 15u};
  }
  uint32_t x0 = 0, x1 = 1, c0 = 0, c1 = 0;
  for (int k = 0; k < items; ++k) {
    const uint32_t c = (cbits >> k) & 1u;
    x0 = c & (x0 ^ 1u);
    x1 = c & (x1 ^ 1u);
    c0 += x0;
    c1 += x1;
  }
  return ParAgg{x0 | (x1 << 1), c0, c1};
}

// Block-wide exclusive composition of the per-thread aggregates: returns
// this thread's exclusive prefix and, in total, the whole tile's aggregate.
template <int BLOCK>
__device__ __forceinline__ ParAgg block_par_scan(const ParAgg &a, ParAgg &total, ParAgg *s_warp) {
  constexpr int NW = BLOCK / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  ParAgg inc = a;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const ParAgg o = par_shfl_up(inc, d);
    if (lane >= d) inc = par_compose(o, inc);
  }
  ParAgg excl = par_shfl_up(inc, 1);
  if (lane == 0) excl = par_identity();
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  // the warps' exclusive prefixes and the total, scanned by warp 0 alone
  // (rather than every thread composing all warp aggregates in turn)
  static_assert(NW <= 32, "one lane per warp aggregate");
  __shared__ ParAgg s_pre[NW + 1];
  if (warp == 0) {
    ParAgg v = lane < NW ? s_warp[lane] : par_identity();
#pragma unroll
    for (int d = 1; d < NW; d <<= 1) {
      const ParAgg o = par_shfl_up(v, d);
      if (lane >= d) v = par_compose(o, v);
    }
    ParAgg e = par_shfl_up(v, 1);
    if (lane == 0) e = par_identity();
    if (lane < NW) s_pre[lane] = e;
    if (lane == NW - 1) s_pre[NW] = v;
  }
  __syncthreads();
  total = s_pre[NW];
  return par_compose(s_pre[warp], excl);
}

template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK, 4) k_apply_classify(const int32_t *__restrict__ s, uint64_t n,
                                                             const uint32_t *__restrict__ heads, uint64_t head_words,
                                                             PairTable tab, uint32_t *__restrict__ tword,
                                                             unsigned long long *__restrict__ tile_agg,
                                                             DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  static_assert(ITEMS == 8 && TILE <= 2048, "a thread word holds 8 candidate bits and 11-bit counts");
  __shared__ __align__(128) TilePipe<TILE> P;
  __shared__ ParAgg s_warp[BLOCK / 32];
  const uint64_t ntiles = (n + TILE - 1) / TILE;
  uint64_t tile = blockIdx.x;
  if (tile >= ntiles) return;
  if (threadIdx.x == 0) {
    mbar_init(&P.bar[0], 1);
    mbar_init(&P.bar[1], 1);
    mbar_init_fence();
  }
  __syncthreads();
  uint32_t phases = 0;
  bool bulk_cur = pipe_issue<BLOCK, TILE>(P, 0, tile, s, n, heads, head_words);
  const uint32_t j0 = threadIdx.x * ITEMS;
  for (int b = 0;; b ^= 1) {
    const uint64_t next = tile + gridDim.x;
    const bool has_next = next < ntiles;
    const bool bulk_next = has_next && pipe_issue<BLOCK, TILE>(P, b ^ 1, next, s, n, heads, head_words);
    if (!pipe_wait<TILE>(P, b, bulk_cur, phases)) {
      if (threadIdx.x == 0) atomicOr(&status->err, kErrTimeout);
      if (bulk_next) mbar_wait(&P.bar[b ^ 1], (phases >> (b ^ 1)) & 1u);
      return;
    }
    const uint32_t len = (uint32_t)min((uint64_t)TILE, n - tile * TILE);
    // positions with a successor inside the stream (as in the count)
    const uint32_t plen = tile * TILE + len < n ? len : len - 1;
    int32_t v[ITEMS + 1];
    thread_steps<ITEMS>(P.sv[b], j0, v);
    const uint32_t hd = bits_from(P.hb[b], j0);
    uint32_t validb = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) validb |= (uint32_t)(j0 + k < plen && !((hd >> (k + 1)) & 1u)) << k;
    uint32_t slot[ITEMS], fl[ITEMS], fwdb;
    lookup_pairs<ITEMS>(v, validb, tab, slot, fl, fwdb, status);
    uint32_t cbits = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) cbits |= (uint32_t)(((validb >> k) & 1u) && (fl[k] & kFlagRepeated)) << k;
    ParAgg total;
    const ParAgg excl = block_par_scan<BLOCK>(par_of_bits(cbits, ITEMS), total, s_warp);
    // my candidate bits and my exclusive prefix inside the tile (counts < 2048)
    tword[tile * BLOCK + threadIdx.x] = cbits | ((excl.xo & 3u) << 8) | (excl.c0 << 10) | (excl.c1 << 21);
    if (threadIdx.x == 0) tile_agg[tile] = par_encode(total);
    pipe_release();
    if (!has_next) break;
    tile = next;
    bulk_cur = bulk_next;
  }
}

// The same classification with one tile per block and the steps read
// straight from global memory: no staging pipeline and no barrier besides
// the block scan's, so more blocks are resident to hide the table probes.
// n_pos positions are classified (tiles of the launch), n_data >= n_pos
// steps are readable (one more when the stream continues past the range, as
// in a chunk of a longer stream); heads covers positions 0 .. n_pos.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_apply_classify_flat(const int32_t *__restrict__ s, uint64_t n_pos,
                                                               uint64_t n_data, const uint32_t *__restrict__ heads,
                                                               PairTable tab, uint32_t *__restrict__ tword,
                                                               unsigned long long *__restrict__ tile_agg,
                                                               DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  static_assert(ITEMS == 8 && TILE <= 2048, "a thread word holds 8 candidate bits and 11-bit counts");
  __shared__ ParAgg s_warp[BLOCK / 32];
  const uint64_t tile = blockIdx.x;
  const uint64_t p0 = tile * TILE + (uint64_t)threadIdx.x * ITEMS;
  int32_t v[ITEMS + 1];
  uint32_t validb = 0;
  if (p0 + ITEMS < n_data && (reinterpret_cast<uintptr_t>(s) & 15u) == 0) {
    const int4 a = *reinterpret_cast<const int4 *>(s + p0);
    const int4 b = *reinterpret_cast<const int4 *>(s + p0 + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    v[8] = s[p0 + ITEMS];
  } else {
#pragma unroll
    for (int k = 0; k <= ITEMS; ++k) v[k] = p0 + k < n_data ? s[p0 + k] : 0;
  }
  if (p0 < n_pos) {
    const uint32_t w = (uint32_t)(p0 >> 5);
    const uint32_t hd = (uint32_t)((((unsigned long long)heads[w + 1] << 32) | heads[w]) >> (p0 & 31));
#pragma unroll
    for (int k = 0; k < ITEMS; ++k)
      validb |= (uint32_t)(p0 + k < n_pos && p0 + k + 1 < n_data && !((hd >> (k + 1)) & 1u)) << k;
  }
  uint32_t slot[ITEMS], fl[ITEMS], fwdb;
  lookup_pairs<ITEMS>(v, validb, tab, slot, fl, fwdb, status);
  uint32_t cbits = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) cbits |= (uint32_t)(((validb >> k) & 1u) && (fl[k] & kFlagRepeated)) << k;
  ParAgg total;
  const ParAgg excl = block_par_scan<BLOCK>(par_of_bits(cbits, ITEMS), total, s_warp);
  tword[tile * BLOCK + threadIdx.x] = cbits | ((excl.xo & 3u) << 8) | (excl.c0 << 10) | (excl.c1 << 21);
  if (threadIdx.x == 0) tile_agg[tile] = par_encode(total);
}

// Classification from slot references: the candidate bit of a position is
// the repeated bit of its slot (rep_bits, set by the count), so no key is
// formed and no table probed.  One tile per block, as k_apply_classify_flat.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_apply_classify_sref(const uint32_t *__restrict__ sref, uint64_t n,
                                                               const uint32_t *__restrict__ rep_bits,
                                                               uint32_t *__restrict__ tword,
                                                               unsigned long long *__restrict__ tile_agg) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  static_assert(ITEMS == 8 && TILE <= 2048, "a thread word holds 8 candidate bits and 11-bit counts");
  __shared__ ParAgg s_warp[BLOCK / 32];
  const uint64_t tile = blockIdx.x;
  const uint64_t p0 = tile * TILE + (uint64_t)threadIdx.x * ITEMS;
  uint32_t ref[ITEMS];
  if (p0 + ITEMS <= n && (reinterpret_cast<uintptr_t>(sref) & 15u) == 0) {
    // evict-first: the references stream through once per pass, and L2 is
    // better left to the repeated-slot bitmap
    const uint4 a = __ldcs(reinterpret_cast<const uint4 *>(sref + p0));
    const uint4 b = __ldcs(reinterpret_cast<const uint4 *>(sref + p0 + 4));
    ref[0] = a.x; ref[1] = a.y; ref[2] = a.z; ref[3] = a.w;
    ref[4] = b.x; ref[5] = b.y; ref[6] = b.z; ref[7] = b.w;
  } else {
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) ref[k] = p0 + k < n ? sref[p0 + k] : kNoPair;
  }
  uint32_t word[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) word[k] = ref[k] != kNoPair ? rep_bits[(ref[k] & ~kRevBit) >> 5] : 0u;
  uint32_t cbits = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k)
    cbits |= (uint32_t)(ref[k] != kNoPair && ((word[k] >> (ref[k] & 31)) & 1u)) << k;
  ParAgg total;
  const ParAgg excl = block_par_scan<BLOCK>(par_of_bits(cbits, ITEMS), total, s_warp);
  tword[tile * BLOCK + threadIdx.x] = cbits | ((excl.xo & 3u) << 8) | (excl.c0 << 10) | (excl.c1 << 21);
  if (threadIdx.x == 0) tile_agg[tile] = par_encode(total);
}

// state[t] = the state (x, replaced count) before tile t, encoded x | c << 1.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_tile_states(const unsigned long long *__restrict__ tile_agg,
                                                       uint64_t ntiles, unsigned long long *__restrict__ state,
                                                       unsigned long long *desc, uint32_t *tile_counter,
                                                       DevStatus *status) {
  __shared__ ParAgg s_warp[BLOCK / 32];
  __shared__ uint32_t s_x;
  __shared__ unsigned long long s_c;
  const uint32_t blk = claim_tile(tile_counter);
  const uint64_t i0 = ((uint64_t)blk * BLOCK + threadIdx.x) * ITEMS;
  ParAgg agg[ITEMS];
  ParAgg mine = par_identity();
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    agg[k] = i0 + k < ntiles ? par_decode(tile_agg[i0 + k]) : par_identity();
    mine = par_compose(mine, agg[k]);
  }
  ParAgg total;
  const ParAgg excl = block_par_scan<BLOCK>(mine, total, s_warp);
  if (threadIdx.x < 32) {
    const ParState in = warp_lookback<ParOp>(desc, blk, total, &status->err);
    if (threadIdx.x == 0) {
      s_x = in.x;
      s_c = in.c;
    }
  }
  __syncthreads();
  ParState st = ParOp::apply(excl, ParState{s_x, s_c});
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    if (i0 + k < ntiles) state[i0 + k] = ParOp::encode_incl(st);
    st = ParOp::apply(agg[k], st);
  }
}

// Replays one tile from its carried-in state: replaced positions become
// their temporary rule symbols, consumed ones vanish, and the kept symbols
// are compacted into out; traversal offsets inside the tile are moved to
// their output positions.  v = the thread's ITEMS steps and the next one;
// tw / st / ag = the thread's word, the tile's carried-in state and its
// aggregate; tlo = the tile's first traversal; so / lidx = shared scratch.
// With SREF the rules of the replaced positions come from their slot
// references ref[] (written by the count) instead of a second table lookup,
// and a slot already set in used_bits takes no atomic.
template <int BLOCK, int ITEMS, bool SREF = false>
__device__ __forceinline__ void emit_tile(const int32_t (&v)[ITEMS + 1], uint64_t tile, uint64_t n, uint32_t tw,
                                          unsigned long long st, unsigned long long ag, const uint64_t *s_tlo,
                                          const uint64_t *__restrict__ off, uint64_t ntrav, const PairTable &tab,
                                          int32_t temp_base, int32_t *__restrict__ out, uint64_t out_shift,
                                          uint64_t *__restrict__ new_off, uint32_t *used_bits, DevStatus *status,
                                          int32_t *so, uint16_t *lidx, const uint32_t (&ref)[ITEMS]) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  const uint32_t j0 = threadIdx.x * ITEMS;
  const uint64_t base = tile * TILE;
  const uint32_t len = (uint32_t)min((uint64_t)TILE, n - base);
  const uint32_t cbits = tw & 0xFFu;
  const ParAgg excl{(tw >> 8) & 3u, (tw >> 10) & 0x7FFu, tw >> 21};
  const ParAgg total = par_decode(ag);
  const uint32_t in_x = (uint32_t)(st & 1u);
  const unsigned long long in_c = st >> 1;
  // replay from the carried-in state: kept (not consumed) and replaced bits
  const uint32_t x_init = par_x(excl, in_x);
  const uint32_t c_init = par_c(excl, in_x);  // replaced positions in this tile before j0
  uint32_t keptbits = 0, xbits = 0;
  if (ITEMS == 8) {
    // the replay of all eight positions from one table load; positions past
    // the stream's end (the tile's last thread) are masked off
    const uint32_t t = __ldg(&g_replay8.v[cbits | (x_init << 8)]);
    const uint32_t valid = j0 >= len ? 0u : (len - j0 >= 8u ? 0xFFu : (1u << (len - j0)) - 1u);
    xbits = t & valid;
    keptbits = (t >> 8) & valid;
  } else {
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
  // the rules of the replaced positions
  uint32_t slot[ITEMS], fl[ITEMS], fwdb;
  if (SREF) {
    fwdb = 0;
    uint32_t uw[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      slot[k] = ref[k] & ~kRevBit;
      fwdb |= (uint32_t)((ref[k] & kRevBit) == 0) << k;
      uw[k] = ((xbits >> k) & 1u) ? used_bits[slot[k] >> 5] : 0u;  // all gathers in flight together
    }
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) fl[k] = ((uw[k] >> (slot[k] & 31)) & 1u) ? kFlagUsed : 0u;
  } else {
    lookup_pairs<ITEMS>(v, xbits, tab, slot, fl, fwdb, status);
  }
  // kept positions of the tile before j0: j0 minus the consumed ones (the
  // carried-in position and the partner of every replaced position before
  // j0, except a replaced j0 - 1 whose partner is j0 itself)
  const uint32_t kept_base = j0 - in_x - c_init + x_init;
  const uint64_t out_base = base - in_c + in_x;
  int32_t *dst = out + (out_base - out_shift);  // out holds output positions from out_shift on
  const uint32_t shift = (uint32_t)((reinterpret_cast<uintptr_t>(dst) >> 2) & 3u);
  uint32_t lpk[ITEMS / 2];
  uint32_t need = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t lo = kept_base + __popc(keptbits & ((1u << k) - 1u));
    if ((keptbits >> k) & 1u) {
      int32_t val = v[k];
      if ((xbits >> k) & 1u) {
        const int32_t sym = temp_base + (int32_t)slot[k];
        val = ((fwdb >> k) & 1u) ? sym : neg32(sym);
        if (!(fl[k] & kFlagUsed)) need |= 1u << k;
      }
      so[shift + lo] = val;
    }
    if (k & 1) lpk[k >> 1] |= lo << 16;
    else lpk[k >> 1] = lo & 0xFFFFu;
  }
  *reinterpret_cast<uint4 *>(&lidx[j0]) = make_uint4(lpk[0], lpk[1], lpk[2], lpk[3]);
  // rules chosen here whose slot was not yet flagged used: one flag update
  // per distinct slot per warp (frequent pairs hit one slot from every
  // lane), mirrored into the bitmap of used slots
  if (__any_sync(0xffffffffu, need != 0)) {
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const bool nk = (need >> k) & 1u;
      if (__any_sync(0xffffffffu, nk)) {
        const uint32_t peers = __match_any_sync(0xffffffffu, nk ? slot[k] : 0xFFFFFFFFu);
        if (nk && (peers & lanemask_lt()) == 0) {
          if (!SREF) atomicOr(&tab.slots[slot[k]].flags, kFlagUsed);
          atomicOr(&used_bits[slot[k] >> 5], 1u << (slot[k] & 31));
        }
      }
    }
  }
  __syncthreads();
  // positions consumed inside the tile: the carried-in one (in_x) plus the
  // partner of every replaced position except a replaced last position,
  // whose partner opens the next tile (x_out)
  const uint32_t kept = len - in_x - par_c(total, in_x) + par_x(total, in_x);
  stage_out_phased<BLOCK>(dst, so, shift, kept);
  const bool last_tile = base + len == n;
  for (uint64_t t = *s_tlo + threadIdx.x; t <= ntrav; t += BLOCK) {
    const uint64_t q = off[t];
    if (q < base + len) new_off[t] = out_base + lidx[(uint32_t)(q - base)];
    else if (last_tile && q == n) new_off[t] = out_base + kept;
    else break;
  }
  if (last_tile && threadIdx.x == 0) status->u64[2] = out_base + kept;
}

template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK, 3) k_apply_emit(const int32_t *__restrict__ s, uint64_t n,
                                                      const uint32_t *__restrict__ heads, uint64_t head_words,
                                                      const uint32_t *__restrict__ tword,
                                                      const unsigned long long *__restrict__ tile_agg,
                                                      const unsigned long long *__restrict__ state,
                                                      const uint64_t *__restrict__ off, uint64_t ntrav,
                                                      const uint64_t *__restrict__ tile_trav, PairTable tab,
                                                      int32_t temp_base, int32_t *__restrict__ out,
                                                      uint64_t *__restrict__ new_off, uint32_t *used_bits,
                                                      DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  static_assert(TILE < (1u << 16), "tile must fit 16-bit local indices");
  static_assert(ITEMS == 8, "lidx packs eight 16-bit indices per thread");
  __shared__ __align__(128) TilePipe<TILE> P;
  __shared__ __align__(16) int32_t so[TILE + 4];
  __shared__ __align__(16) uint16_t lidx[TILE];  // output index (in the tile) of each kept position
  __shared__ uint64_t s_tlo;
  const uint64_t ntiles = (n + TILE - 1) / TILE;
  uint64_t tile = blockIdx.x;
  if (tile >= ntiles) return;
  if (threadIdx.x == 0) {
    mbar_init(&P.bar[0], 1);
    mbar_init(&P.bar[1], 1);
    mbar_init_fence();
  }
  __syncthreads();
  uint32_t phases = 0;
  bool bulk_cur = pipe_issue<BLOCK, TILE>(P, 0, tile, s, n, heads, head_words);
  uint32_t tw_cur = tword[tile * BLOCK + threadIdx.x];
  unsigned long long st_cur = state[tile], ag_cur = tile_agg[tile];
  const uint32_t j0 = threadIdx.x * ITEMS;
  for (int b = 0;; b ^= 1) {
    const uint64_t next = tile + gridDim.x;
    const bool has_next = next < ntiles;
    const bool bulk_next = has_next && pipe_issue<BLOCK, TILE>(P, b ^ 1, next, s, n, heads, head_words);
    // the next tile's thread words, aggregate and carried-in state, in flight meanwhile
    const uint32_t tw_next = has_next ? tword[next * BLOCK + threadIdx.x] : 0u;
    const unsigned long long st_next = has_next ? state[next] : 0ull;
    const unsigned long long ag_next = has_next ? tile_agg[next] : 0ull;
    if (threadIdx.x == 0) s_tlo = tile_trav[tile];
    if (!pipe_wait<TILE>(P, b, bulk_cur, phases)) {
      if (threadIdx.x == 0) atomicOr(&status->err, kErrTimeout);
      if (bulk_next) mbar_wait(&P.bar[b ^ 1], (phases >> (b ^ 1)) & 1u);
      return;
    }
    int32_t v[ITEMS + 1];
    thread_steps<ITEMS>(P.sv[b], j0, v);
    const uint32_t no_ref[ITEMS] = {};
    emit_tile<BLOCK, ITEMS>(v, tile, n, tw_cur, st_cur, ag_cur, &s_tlo, off, ntrav, tab, temp_base, out, 0,
                            new_off, used_bits, status, so, lidx, no_ref);
    pipe_release();
    if (!has_next) break;
    tile = next;
    bulk_cur = bulk_next;
    tw_cur = tw_next;
    st_cur = st_next;
    ag_cur = ag_next;
  }
}

// The same replay with one tile per block and the steps read straight from
// global memory (no staging pipeline).
// Chunks of a longer stream: the launch covers tiles tile0 .. tile0 +
// gridDim.x - 1 of the n-step stream, s holds its steps from position
// pos_base on (one past the range when the stream continues), out its output
// from position out_shift on.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) k_apply_emit_flat(const int32_t *__restrict__ s, uint64_t pos_base,
                                                           uint64_t tile0, uint64_t n,
                                                           const uint32_t *__restrict__ tword,
                                                           const unsigned long long *__restrict__ tile_agg,
                                                           const unsigned long long *__restrict__ state,
                                                           const uint64_t *__restrict__ off, uint64_t ntrav,
                                                           const uint64_t *__restrict__ tile_trav, PairTable tab,
                                                           int32_t temp_base, int32_t *__restrict__ out,
                                                           uint64_t out_shift, uint64_t *__restrict__ new_off,
                                                           uint32_t *used_bits, DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  static_assert(TILE < (1u << 16), "tile must fit 16-bit local indices");
  static_assert(ITEMS == 8, "lidx packs eight 16-bit indices per thread");
  __shared__ __align__(16) int32_t so[TILE + 4];
  __shared__ __align__(16) uint16_t lidx[TILE];
  __shared__ uint64_t s_tlo;
  const uint64_t tile = tile0 + blockIdx.x;
  if (threadIdx.x == 0) s_tlo = tile_trav[tile];
  const uint32_t tw = tword[tile * BLOCK + threadIdx.x];
  const unsigned long long st = state[tile], ag = tile_agg[tile];
  const uint64_t p0 = tile * TILE + (uint64_t)threadIdx.x * ITEMS;  // stream position
  const int32_t *sl = s + (p0 - pos_base);
  int32_t v[ITEMS + 1];
  if (p0 + ITEMS < n && (reinterpret_cast<uintptr_t>(sl) & 15u) == 0) {
    const int4 a = *reinterpret_cast<const int4 *>(sl);
    const int4 b = *reinterpret_cast<const int4 *>(sl + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    v[8] = sl[ITEMS];
  } else {
#pragma unroll
    for (int k = 0; k <= ITEMS; ++k) v[k] = p0 + k < n ? sl[k] : 0;
  }
  const uint32_t no_ref[ITEMS] = {};
  emit_tile<BLOCK, ITEMS>(v, tile, n, tw, st, ag, &s_tlo, off, ntrav, tab, temp_base, out, out_shift, new_off,
                          used_bits, status, so, lidx, no_ref);
}

// Emit from slot references: one tile per block (as k_apply_emit_flat on a
// whole resident stream), the replaced positions' rules read from sref.
// Six resident blocks per SM (at most 40 registers): 2.50 against 2.85 ms
// per step at the four blocks its 63 registers would allow.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK, 6) k_apply_emit_sref(const int32_t *__restrict__ s,
                                                           const uint32_t *__restrict__ sref, uint64_t n,
                                                           const uint32_t *__restrict__ tword,
                                                           const unsigned long long *__restrict__ tile_agg,
                                                           const unsigned long long *__restrict__ state,
                                                           const uint64_t *__restrict__ off, uint64_t ntrav,
                                                           const uint64_t *__restrict__ tile_trav, PairTable tab,
                                                           int32_t temp_base, int32_t *__restrict__ out,
                                                           uint64_t *__restrict__ new_off, uint32_t *used_bits,
                                                           DevStatus *status) {
  constexpr uint32_t TILE = BLOCK * ITEMS;
  static_assert(TILE < (1u << 16), "tile must fit 16-bit local indices");
  static_assert(ITEMS == 8, "lidx packs eight 16-bit indices per thread");
  __shared__ __align__(16) int32_t so[TILE + 4];
  __shared__ __align__(16) uint16_t lidx[TILE];
  __shared__ uint64_t s_tlo;
  const uint64_t tile = blockIdx.x;
  if (threadIdx.x == 0) s_tlo = tile_trav[tile];
  const uint32_t tw = tword[tile * BLOCK + threadIdx.x];
  const unsigned long long st = state[tile], ag = tile_agg[tile];
  const uint64_t p0 = tile * TILE + (uint64_t)threadIdx.x * ITEMS;
  int32_t v[ITEMS + 1];
  uint32_t ref[ITEMS];
  if (p0 + ITEMS < n && (reinterpret_cast<uintptr_t>(s) & 15u) == 0 && (reinterpret_cast<uintptr_t>(sref) & 15u) == 0) {
    // evict-first, as in the classification: L2 keeps the used-slot bitmap
    const int4 a = __ldcs(reinterpret_cast<const int4 *>(s + p0));
    const int4 b = __ldcs(reinterpret_cast<const int4 *>(s + p0 + 4));
    const uint4 ra = __ldcs(reinterpret_cast<const uint4 *>(sref + p0));
    const uint4 rb = __ldcs(reinterpret_cast<const uint4 *>(sref + p0 + 4));
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    v[8] = s[p0 + ITEMS];
    ref[0] = ra.x; ref[1] = ra.y; ref[2] = ra.z; ref[3] = ra.w;
    ref[4] = rb.x; ref[5] = rb.y; ref[6] = rb.z; ref[7] = rb.w;
  } else {
#pragma unroll
    for (int k = 0; k <= ITEMS; ++k) v[k] = p0 + k < n ? s[p0 + k] : 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) ref[k] = p0 + k < n ? sref[p0 + k] : kNoPair;
  }
  emit_tile<BLOCK, ITEMS, true>(v, tile, n, tw, st, ag, &s_tlo, off, ntrav, tab, temp_base, out, 0, new_off,
                                used_bits, status, so, lidx, ref);
}

// ---------------------------------------------------------------------------
// Used-rule collection
// ---------------------------------------------------------------------------
// (key with the sign bit flipped, slot) of every slot set in the used
// bitmap, in no particular order; the count lands in status->u64[3], the OR
// and AND of the keys in u64[4] / u64[5] (u64[5] preset to all ones), and
// entries beyond cap_out are dropped with kErrLength.
__global__ void __launch_bounds__(kBlock) k_collect_used(const uint32_t *__restrict__ bits, uint64_t words,
                                                         PairTable tab, unsigned long long *keys_out,
                                                         uint32_t *slots_out, uint64_t cap_out, DevStatus *status) {
  unsigned long long o = 0, a = ~0ull;  // this thread's OR / AND of the keys it wrote
  const int lane = threadIdx.x & 31;
  for (uint64_t wi = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; wi < words;
       wi += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t b = bits[wi];
    const uint32_t act = __activemask();
    const uint32_t cnt = __popc(b);
    // warp-aggregated reservation of this lane's cnt entries
    uint32_t incl = cnt;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t v = __shfl_up_sync(act, incl, d);
      if (lane >= d && ((act >> (lane - d)) & 1u)) incl += v;
    }
    const int last = 31 - __clz(act);
    const uint32_t wsum = __shfl_sync(act, incl, last);
    if (!wsum) continue;
    unsigned long long base = 0;
    if (lane == last) base = atomicAdd(&status->u64[3], (unsigned long long)wsum);
    base = __shfl_sync(act, base, last) + (incl - cnt);
    while (b) {
      const uint32_t j = (uint32_t)__ffs(b) - 1;
      b &= b - 1;
      const uint64_t slot = wi * 32 + j;
      const unsigned long long key = tab.slots[slot].key ^ kSignFlip;
      o |= key;
      a &= key;
      if (base < cap_out) {
        keys_out[base] = key;
        slots_out[base] = (uint32_t)slot;
      } else {
        atomicOr(&status->err, kErrLength);
      }
      ++base;
    }
  }
  // one OR / AND per block
  __shared__ unsigned long long s_o[kBlock / 32], s_a[kBlock / 32];
  for (int d = 16; d > 0; d >>= 1) {
    o |= __shfl_xor_sync(0xffffffffu, o, d);
    a &= __shfl_xor_sync(0xffffffffu, a, d);
  }
  if (lane == 0) {
    s_o[threadIdx.x >> 5] = o;
    s_a[threadIdx.x >> 5] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kBlock / 32; ++w) {
      o |= s_o[w];
      a &= s_a[w];
    }
    if (o) atomicOr(&status->u64[4], o);
    if (~a) atomicAnd(&status->u64[5], a);
  }
}

// ---------------------------------------------------------------------------
// Radix sort of the used rules, id assignment, remap
// ---------------------------------------------------------------------------
// One-sweep LSD radix sort of (u64 key, u32 value) pairs, one kernel per
// byte pass.  Every tile of kSortTile keys ranks its keys stably in shared
// memory, publishes its 256 digit counts, looks back over the earlier tiles
// digit by digit (thread d follows digit d) and scatters; the digit bases
// come from one histogram of all sorted bytes taken before the first pass.
constexpr int kSortItems = 8;
constexpr uint32_t kSortTile = kBlock * kSortItems;

// hist[b * 256 + d] += number of keys whose byte b is d, for the bytes in
// byte_mask (hist zeroed beforehand).
__global__ void __launch_bounds__(kBlock) k_sort_hist(const unsigned long long *__restrict__ keys, uint64_t n,
                                                      uint32_t byte_mask, uint32_t *hist) {
  __shared__ uint32_t cnt[8 * 256];
  for (uint32_t i = threadIdx.x; i < 8 * 256; i += kBlock) cnt[i] = 0;
  __syncthreads();
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = keys[i];
#pragma unroll
    for (int b = 0; b < 8; ++b)
      if ((byte_mask >> b) & 1u) atomicAdd(&cnt[b * 256 + (uint32_t)((k >> (8 * b)) & 0xFF)], 1u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < 8 * 256; i += kBlock)
    if (cnt[i]) atomicAdd(&hist[i], cnt[i]);
}

// One pass on the byte at `shift`; hist_b = that byte's 256 digit counts,
// desc = tiles * 256 zeroed descriptors, counter = zeroed tile counter.
__global__ void __launch_bounds__(kBlock) k_sort_pass(const unsigned long long *__restrict__ keys,
                                                      const uint32_t *__restrict__ vals,
                                                      unsigned long long *__restrict__ keys_out,
                                                      uint32_t *__restrict__ vals_out, uint64_t n, int shift,
                                                      const uint32_t *__restrict__ hist_b, unsigned long long *desc,
                                                      uint32_t *counter, uint32_t *err) {
  static_assert(kBlock == 256, "one thread per digit");
  constexpr int NW = kBlock / 32;
  constexpr uint32_t kWarpKeys = 32 * kSortItems;
  __shared__ uint32_t s_tile;
  __shared__ uint32_t wcnt[NW][256];  // a warp's digit counts, then its offset within the tile
  __shared__ unsigned long long base[256];
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = lane; k < 256; k += 32) wcnt[warp][k] = 0;
  __syncthreads();
  const uint64_t tile = s_tile;
  // warp w ranks the tile's keys [w * kWarpKeys, (w + 1) * kWarpKeys) in
  // order, with counters of its own: no block barrier per key
  const uint64_t w0 = tile * kSortTile + (uint64_t)warp * kWarpKeys;
  unsigned long long key[kSortItems];
  uint32_t val[kSortItems], rank[kSortItems], dig[kSortItems];
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    const uint64_t i = w0 + (uint64_t)it * 32 + lane;
    const bool valid = i < n;
    key[it] = 0;
    val[it] = 0;
    dig[it] = 256;
    if (valid) {
      key[it] = keys[i];
      val[it] = vals[i];
      dig[it] = (uint32_t)((key[it] >> shift) & 0xFF);
    }
    const uint32_t m = __match_any_sync(0xffffffffu, dig[it]);
    const uint32_t lrank = __popc(m & lanemask_lt());
    const uint32_t before = valid ? wcnt[warp][dig[it]] : 0u;
    __syncwarp();
    if (valid && lrank == 0) wcnt[warp][dig[it]] = before + __popc(m);
    __syncwarp();
    rank[it] = before + lrank;
  }
  __syncthreads();
  // digit d: each warp's offset within the tile (exclusive over the warps)
  // and the tile's count
  const uint32_t d = threadIdx.x;
  uint32_t run = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    const uint32_t c = wcnt[w][d];
    wcnt[w][d] = run;
    run += c;
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kSortItems; ++it)
    if (dig[it] < 256) rank[it] += wcnt[warp][dig[it]];
  // digit d: count in this tile, keys of digit d in earlier tiles, base
  const unsigned long long cnt_d = run;
  unsigned long long excl = 0;
  if (tile == 0) {
    st_desc(&desc[d], kDescIncl | cnt_d);
  } else {
    st_desc(&desc[tile * 256 + d], kDescAgg | cnt_d);
    // the predecessors' descriptors kSortWindow at a time, all loads in
    // flight together, summed in order down to the first inclusive one
    // (tile -1 counts as an inclusive zero)
    constexpr int kSortWindow = 8;
    bool found = false;
    for (int64_t j = (int64_t)tile - 1; !found; j -= kSortWindow) {
      unsigned long long v[kSortWindow];
#pragma unroll
      for (int i = 0; i < kSortWindow; ++i) v[i] = j - i >= 0 ? ld_desc(&desc[(uint64_t)(j - i) * 256 + d]) : kDescIncl;
#pragma unroll
      for (int i = 0; i < kSortWindow; ++i) {
        if (found) break;
        unsigned long long x = v[i];
        if ((x & kDescMask) == 0) x = wait_desc(desc + d, (uint64_t)(j - i) * 256, err);
        excl += x & kDescPayload;
        found = (x & kDescMask) == kDescIncl;
      }
    }
    st_desc(&desc[tile * 256 + d], kDescIncl | (excl + cnt_d));
  }
  unsigned long long total;
  const unsigned long long dbase = block_excl_sum<kBlock>(hist_b[d], total);
  base[d] = dbase + excl;
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kSortItems; ++it) {
    if (dig[it] < 256) {
      const unsigned long long dst = base[dig[it]] + rank[it];
      keys_out[dst] = key[it];
      vals_out[dst] = val[it];
    }
  }
}

__global__ void k_assign_ids(const unsigned long long *sorted_keys, const uint32_t *sorted_slots, uint64_t u,
                             uint32_t next_id, PairTable tab, long long *rulebook) {
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < u; r += (uint64_t)gridDim.x * blockDim.x) {
    tab.slots[sorted_slots[r]].val = next_id + (uint32_t)r;
    rulebook[r] = (long long)(sorted_keys[r] ^ kSignFlip);
  }
}

__device__ __forceinline__ int32_t remap_one(int32_t v, int32_t temp_base, const PairSlot *__restrict__ slots) {
  const uint32_t a = abs32(v);
  if (a < (uint32_t)temp_base) return v;
  const int32_t f = (int32_t)slots[a - (uint32_t)temp_base].val;
  return v < 0 ? neg32(f) : f;
}

// 16-byte vectors when s is 16-byte aligned (VEC), single steps otherwise.
template <bool VEC>
__global__ void k_remap(int32_t *s, uint64_t n, int32_t temp_base, const PairSlot *__restrict__ slots) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  uint64_t done = 0;
  if (VEC) {
    int4 *s4 = reinterpret_cast<int4 *>(s);
    for (uint64_t g = t0; g < n / 4; g += stride) {
      int4 x = s4[g];
      x.x = remap_one(x.x, temp_base, slots);
      x.y = remap_one(x.y, temp_base, slots);
      x.z = remap_one(x.z, temp_base, slots);
      x.w = remap_one(x.w, temp_base, slots);
      s4[g] = x;
    }
    done = n & ~3ull;
  }
  for (uint64_t i = done + t0; i < n; i += stride) s[i] = remap_one(s[i], temp_base, slots);
}

// ---------------------------------------------------------------------------
// Append encoder
// ---------------------------------------------------------------------------
// Rule i of [lo, hi) gets id start + i - lo under its key pack(first,
// second).
__global__ void k_build_rule_table(const int32_t *first, const int32_t *second, uint64_t lo, uint64_t hi,
                                   uint32_t start, PairTable tab, DevStatus *status) {
  const uint32_t mask = (uint32_t)(tab.cap - 1);
  for (uint64_t i = lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < hi;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = pack2(first[i], second[i]);
    if (key == kEmptyKey) {
      atomicOr(&status->err, kErrBadSymbol);
      continue;
    }
    uint32_t h = hash_pair(key) & mask;
    for (uint32_t p = 0;; ++p) {
      if (p >= kMaxProbe) {
        atomicOr(&status->err, kErrTableFull);
        break;
      }
      const unsigned long long old = atomicCAS(&tab.slots[h].key, kEmptyKey, key);
      if (old == kEmptyKey || old == key) {
        // the first stored occurrence keeps its id (emplace semantics)
        atomicMin(&tab.slots[h].val, start + (uint32_t)(i - lo));
        break;
      }
      h = (h + 1) & mask;
    }
  }
}

__device__ __forceinline__ bool table_find(const PairTable &tab, unsigned long long key, uint32_t &id) {
  if (key == kEmptyKey) return false;
  const uint32_t mask = (uint32_t)(tab.cap - 1);
  uint32_t h = hash_pair(key) & mask;
  for (uint32_t p = 0; p < kMaxProbe; ++p) {
    const ulonglong2 w = *reinterpret_cast<const ulonglong2 *>(&tab.slots[h]);
    if (w.x == key) {
      id = (uint32_t)(w.y >> 32);
      return true;
    }
    if (w.x == kEmptyKey) return false;
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

// One push of the stack pass with stack top t and pushed symbol x: the
// forward key first, then the reversed key (path_encoder.cpp:40-75).
__device__ __forceinline__ bool stack_match(const PairTable &tab, int32_t t, int32_t x, int32_t &r) {
  const unsigned long long k = pack2(t, x);
  uint32_t id;
  if (table_find(tab, k, id)) {
    r = (int32_t)id;
    return true;
  }
  if (table_find(tab, rev2(k), id)) {
    r = neg32((int32_t)id);
    return true;
  }
  return false;
}

// Chunked stack pass.  The pass only ever looks at the stack top and the
// pushed symbol, so its state is the top alone: after symbol p it is either
// p's own value (p did not pair, and the previous top went to the output)
// or the rule the pair made.  Each chunk runs from its first symbol as if
// the incoming top did not pair with it; top[p] is the top after p and bit 0
// of fl[p] says that p did not pair (it emitted the previous top).  Bit 1
// of fl[p] marks the last symbol of a traversal.  Chunk bounds carry flags
// in bit 63 (kChunkEdge): cs = first chunk of a traversal, ce = last chunk.

__global__ void k_stack_spec(const int32_t *s, const uint64_t *cs, const uint64_t *ce, uint64_t nchunks,
                             PairTable tab, int32_t *top, uint8_t *fl) {
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < nchunks;
       c += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t a = cs[c] & ~kChunkEdge, b = ce[c] & ~kChunkEdge;
    const bool first = cs[c] & kChunkEdge, last = ce[c] & kChunkEdge;
    if (b <= a) continue;
    int32_t cur = s[a];
    top[a] = cur;
    fl[a] = (first ? 0 : 1) | (last && b == a + 1 ? 2 : 0);
    for (uint64_t p = a + 1; p < b; ++p) {
      const int32_t x = s[p];
      int32_t r;
      const bool m = stack_match(tab, cur, x, r);
      cur = m ? r : x;
      top[p] = cur;
      fl[p] = (m ? 0 : 1) | (last && p + 1 == b ? 2 : 0);
    }
  }
}

// A chunk whose first symbol does pair with the true incoming top (the
// previous chunk's last top, final once that chunk converged) runs the pass
// again until its top equals the speculative top; from there on the chunk
// is already right.  A chunk that reaches its end first counts in *nonconv
// and the whole pass must be redone another way.
__global__ void k_stack_fix(const int32_t *s, const uint64_t *cs, const uint64_t *ce, uint64_t nchunks,
                            PairTable tab, int32_t *top, uint8_t *fl, unsigned long long *nonconv) {
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < nchunks;
       c += (uint64_t)gridDim.x * blockDim.x) {
    if (cs[c] & kChunkEdge) continue;
    const uint64_t a = cs[c], b = ce[c] & ~kChunkEdge;
    if (b <= a) continue;
    int32_t cur;
    if (!stack_match(tab, top[a - 1], s[a], cur)) continue;
    fl[a] &= 2;
    if (cur == top[a]) continue;
    top[a] = cur;
    uint64_t p = a + 1;
    for (; p < b; ++p) {
      const int32_t x = s[p];
      int32_t r;
      const bool m = stack_match(tab, cur, x, r);
      const int32_t nxt = m ? r : x;
      fl[p] = (fl[p] & 2) | (m ? 0 : 1);
      if (nxt == top[p]) break;
      top[p] = nxt;
      cur = nxt;
    }
    if (p == b) atomicAdd(nonconv, 1ull);
  }
}

// keep[p] = 1 when top[p] goes to the output: p is the last symbol of its
// traversal, or the next symbol did not pair.
__global__ void k_stack_keep(const uint8_t *fl, uint64_t n, uint32_t *keep) {
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x)
    keep[p] = ((fl[p] & 2) || (p + 1 < n && (fl[p + 1] & 1))) ? 1u : 0u;
}

__global__ void k_stack_scatter(const int32_t *top, const uint32_t *keep, const uint64_t *pos, uint64_t n,
                                int32_t *out) {
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x)
    if (keep[p]) out[pos[p]] = top[p];
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
constexpr int kCountItems = 8;
constexpr int kApplyItems = 8;
static_assert(kBlock * kApplyItems == kApplyTile, "apply tile size");

void launch_delta_encode(const int32_t *in, int32_t *out, uint64_t n, const uint64_t *off, uint64_t ntrav,
                         uint32_t *max_abs, cudaStream_t st) {
  if (!n) return;
  constexpr uint64_t TILE = kBlock * kDeltaItems;
  k_delta_encode<kBlock, kDeltaItems><<<(unsigned)((n + TILE - 1) / TILE), kBlock, 0, st>>>(in, out, n, off, ntrav,
                                                                                            max_abs);
}

void launch_max_abs(const int32_t *in, uint64_t n, uint32_t *max_abs, cudaStream_t st) {
  if (!n) return;
  k_max_abs<kBlock><<<grid_for(n, kBlock), kBlock, 0, st>>>(in, n, max_abs);
}

// Resident blocks of a persistent kernel: SMs x blocks per SM.
template <typename K>
unsigned persistent_grid(K kernel, int block, uint64_t tiles) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
  uint64_t g = (uint64_t)(sms > 0 ? sms : 1) * (uint64_t)(per_sm > 0 ? per_sm : 1);
  if (g > tiles) g = tiles;
  return (unsigned)(g ? g : 1);
}

uint64_t head_words(uint64_t n) { return (n + 1 + 31) / 32 + 8; }

void launch_head_bits(const uint64_t *off, uint64_t ntrav, uint32_t *bits, cudaStream_t st) {
  k_head_bits<<<grid_for(ntrav + 1, kBlock), kBlock, 0, st>>>(off, ntrav, bits);
}

void launch_count_pairs(const int32_t *s, uint64_t n, const uint32_t *heads, PairTable tab, DevStatus *status,
                        CountKernel kind, cudaStream_t st, uint32_t *sref, uint32_t *rep_bits) {
  if (!n) return;
  if (kind == CountKernel::kFlat) {
    k_count_flat<<<grid_for(n, kBlock, 152u * 8u * 16u), kBlock, 0, st>>>(s, n, heads, tab, status, sref, rep_bits);
    return;
  }
  if (kind == CountKernel::kFlat4) {
    k_count_flat4<<<grid_for((n + 3) / 4, kBlock, 152u * 8u * 16u), kBlock, 0, st>>>(s, n, heads, tab, status, sref,
                                                                                        rep_bits);
    return;
  }
  constexpr uint64_t TILE = kBlock * kCountItems;
  const uint64_t tiles = (n + TILE - 1) / TILE;
  const uint64_t hw = head_words(n);
  if (kind == CountKernel::kTiledWarpDedup) {
    auto k = k_count_pairs<kBlock, kCountItems, true>;
    k<<<persistent_grid(k, kBlock, tiles), kBlock, 0, st>>>(s, n, heads, hw, tab, status, nullptr, rep_bits);
  } else {
    auto k = k_count_pairs<kBlock, kCountItems, false>;
    k<<<persistent_grid(k, kBlock, tiles), kBlock, 0, st>>>(s, n, heads, hw, tab, status, sref, rep_bits);
  }
}

void launch_head_bits_range(const uint64_t *off, uint64_t ntrav, uint64_t lo, uint64_t span, uint32_t *bits,
                            cudaStream_t st) {
  k_head_bits_range<<<grid_for(ntrav + 1, kBlock), kBlock, 0, st>>>(off, ntrav, lo, span, bits);
}

void launch_delta_chunk(const int32_t *in, int32_t *out, uint64_t len, const uint32_t *heads, uint32_t *max_abs,
                        cudaStream_t st) {
  if (!len) return;
  k_delta_chunk<<<grid_for(len, kBlock), kBlock, 0, st>>>(in, out, len, heads, max_abs);
}

void launch_classify_chunk(const int32_t *s, uint64_t n_pos, uint64_t n_data, const uint32_t *heads, PairTable tab,
                           uint64_t tile0, const ApplyScratch &w, DevStatus *status, cudaStream_t st) {
  if (!n_pos) return;
  k_apply_classify_flat<kBlock, kApplyItems><<<(unsigned)apply_num_tiles(n_pos), kBlock, 0, st>>>(
      s, n_pos, n_data, heads, tab, w.tword + tile0 * kBlock, w.tile_agg + tile0, status);
}

void launch_emit_chunk(const int32_t *s, uint64_t pos_base, uint64_t tile0, uint64_t tiles, uint64_t n,
                       const uint64_t *off, uint64_t ntrav, const uint64_t *tile_trav, PairTable tab,
                       int32_t temp_base, int32_t *out, uint64_t out_shift, uint64_t *new_off, uint32_t *used_bits,
                       const ApplyScratch &w, DevStatus *status, cudaStream_t st) {
  if (!tiles) return;
  k_apply_emit_flat<kBlock, kApplyItems><<<(unsigned)tiles, kBlock, 0, st>>>(
      s, pos_base, tile0, n, w.tword, w.tile_agg, w.state, off, ntrav, tile_trav, tab, temp_base, out, out_shift,
      new_off, used_bits, status);
}

uint64_t apply_num_tiles(uint64_t n) {
  constexpr uint64_t TILE = kBlock * kApplyItems;
  return (n + TILE - 1) / TILE;
}

void launch_tile_trav(const uint64_t *off, uint64_t ntrav, uint64_t n, uint64_t *tile_trav, cudaStream_t st) {
  const uint64_t tiles = apply_num_tiles(n);
  if (!tiles) return;
  k_tile_trav<<<grid_for(tiles, kBlock), kBlock, 0, st>>>(off, ntrav, tiles, kBlock * kApplyItems, tile_trav);
}

constexpr int kStateItems = 16;
uint64_t apply_state_blocks(uint64_t n) {
  const uint64_t tiles = apply_num_tiles(n);
  constexpr uint64_t PER = kBlock * kStateItems;
  return (tiles + PER - 1) / PER;
}

void launch_apply_classify(const int32_t *s, uint64_t n, const uint32_t *heads, PairTable tab, const ApplyScratch &w,
                           bool flat, DevStatus *status, cudaStream_t st) {
  if (!n) return;
  if (flat) {
    k_apply_classify_flat<kBlock, kApplyItems><<<(unsigned)apply_num_tiles(n), kBlock, 0, st>>>(
        s, n, n, heads, tab, w.tword, w.tile_agg, status);
    return;
  }
  auto k = k_apply_classify<kBlock, kApplyItems>;
  k<<<persistent_grid(k, kBlock, apply_num_tiles(n)), kBlock, 0, st>>>(s, n, heads, head_words(n), tab, w.tword,
                                                                       w.tile_agg, status);
}

void launch_apply_classify_sref(const uint32_t *sref, uint64_t n, const uint32_t *rep_bits, const ApplyScratch &w,
                                cudaStream_t st) {
  if (!n) return;
  k_apply_classify_sref<kBlock, kApplyItems><<<(unsigned)apply_num_tiles(n), kBlock, 0, st>>>(sref, n, rep_bits,
                                                                                               w.tword, w.tile_agg);
}

void launch_apply_emit_sref(const int32_t *s, const uint32_t *sref, uint64_t n, const uint64_t *off, uint64_t ntrav,
                            const uint64_t *tile_trav, PairTable tab, int32_t temp_base, int32_t *out,
                            uint64_t *new_off, uint32_t *used_bits, const ApplyScratch &w, DevStatus *status,
                            cudaStream_t st) {
  if (!n) return;
  k_apply_emit_sref<kBlock, kApplyItems><<<(unsigned)apply_num_tiles(n), kBlock, 0, st>>>(
      s, sref, n, w.tword, w.tile_agg, w.state, off, ntrav, tile_trav, tab, temp_base, out, new_off, used_bits,
      status);
}

void launch_apply_states(uint64_t n, const ApplyScratch &w, DevStatus *status, cudaStream_t st) {
  if (!n) return;
  k_tile_states<kBlock, kStateItems><<<(unsigned)apply_state_blocks(n), kBlock, 0, st>>>(
      w.tile_agg, apply_num_tiles(n), w.state, w.desc, w.counter, status);
}

void launch_apply_emit(const int32_t *s, uint64_t n, const uint32_t *heads, const uint64_t *off, uint64_t ntrav,
                       const uint64_t *tile_trav, PairTable tab, int32_t temp_base, int32_t *out, uint64_t *new_off,
                       uint32_t *used_bits, const ApplyScratch &w, bool flat, DevStatus *status,
                       cudaStream_t st) {
  if (!n) return;
  if (flat) {
    k_apply_emit_flat<kBlock, kApplyItems><<<(unsigned)apply_num_tiles(n), kBlock, 0, st>>>(
        s, 0, 0, n, w.tword, w.tile_agg, w.state, off, ntrav, tile_trav, tab, temp_base, out, 0, new_off, used_bits,
        status);
    return;
  }
  auto k = k_apply_emit<kBlock, kApplyItems>;
  k<<<persistent_grid(k, kBlock, apply_num_tiles(n)), kBlock, 0, st>>>(s, n, heads, head_words(n), w.tword,
                                                                       w.tile_agg, w.state, off, ntrav, tile_trav,
                                                                       tab, temp_base, out, new_off, used_bits, status);
}

void launch_collect_used(const uint32_t *bits, uint64_t cap, PairTable tab, unsigned long long *keys_out,
                         uint32_t *slots_out, uint64_t cap_out, DevStatus *status, cudaStream_t st) {
  const uint64_t words = (cap + 31) / 32;
  k_collect_used<<<grid_for(words, kBlock), kBlock, 0, st>>>(bits, words, tab, keys_out, slots_out, cap_out, status);
}

uint64_t sort_tiles(uint64_t n) { return (n + kSortTile - 1) / kSortTile; }

void launch_sort_hist(const unsigned long long *keys, uint64_t n, uint32_t byte_mask, uint32_t *hist,
                      cudaStream_t st) {
  if (!n) return;
  k_sort_hist<<<grid_for(n, kBlock, 152u * 4u), kBlock, 0, st>>>(keys, n, byte_mask, hist);
}

void launch_sort_pass(const unsigned long long *keys, const uint32_t *vals, unsigned long long *keys_out,
                      uint32_t *vals_out, uint64_t n, int byte, const uint32_t *hist, unsigned long long *desc,
                      uint32_t *counter, uint32_t *err, cudaStream_t st) {
  if (!n) return;
  k_sort_pass<<<(unsigned)sort_tiles(n), kBlock, 0, st>>>(keys, vals, keys_out, vals_out, n, 8 * byte,
                                                           hist + 256 * byte, desc, counter, err);
}

void launch_assign_ids(const unsigned long long *sorted_keys, const uint32_t *sorted_slots, uint64_t u,
                       uint32_t next_id, PairTable tab, long long *rulebook, cudaStream_t st) {
  if (!u) return;
  k_assign_ids<<<grid_for(u, kBlock), kBlock, 0, st>>>(sorted_keys, sorted_slots, u, next_id, tab, rulebook);
}

void launch_remap(int32_t *s, uint64_t n, int32_t temp_base, const PairSlot *slots, cudaStream_t st) {
  if (!n) return;
  if ((reinterpret_cast<uintptr_t>(s) & 15u) == 0)
    k_remap<true><<<grid_for((n + 3) / 4, kBlock), kBlock, 0, st>>>(s, n, temp_base, slots);
  else
    k_remap<false><<<grid_for(n, kBlock), kBlock, 0, st>>>(s, n, temp_base, slots);
}

void launch_copy_bytes(const void *src, void *dst, uint64_t n, cudaStream_t st) {
  if (!n) return;
  k_copy_bytes<<<grid_for((n + 15) / 16, kBlock, 152u * 4u), kBlock, 0, st>>>(static_cast<const char *>(src),
                                                                              static_cast<char *>(dst), n);
}

void launch_zero_bytes(void *dst, uint64_t n, cudaStream_t st) {
  if (!n) return;
  k_zero_bytes<<<grid_for((n + 15) / 16, kBlock, 152u * 8u), kBlock, 0, st>>>(static_cast<char *>(dst), n);
}

void launch_table_clear(PairTable tab, uint32_t val_init, cudaStream_t st, uint32_t *bits_a, uint32_t *bits_b) {
  k_table_clear<<<grid_for(tab.cap, kBlock), kBlock, 0, st>>>(tab, val_init, bits_a, bits_b);
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

void launch_stack_chunks(const int32_t *s, const uint64_t *cs, const uint64_t *ce, uint64_t nchunks, PairTable tab,
                         int32_t *top, uint8_t *fl, unsigned long long *nonconv, cudaStream_t st) {
  if (!nchunks) return;
  k_stack_spec<<<grid_for(nchunks, 64), 64, 0, st>>>(s, cs, ce, nchunks, tab, top, fl);
  k_stack_fix<<<grid_for(nchunks, 64), 64, 0, st>>>(s, cs, ce, nchunks, tab, top, fl, nonconv);
}

void launch_stack_keep(const uint8_t *fl, uint64_t n, uint32_t *keep, cudaStream_t st) {
  if (!n) return;
  k_stack_keep<<<grid_for(n, kBlock), kBlock, 0, st>>>(fl, n, keep);
}

void launch_stack_scatter(const int32_t *top, const uint32_t *keep, const uint64_t *pos, uint64_t n, int32_t *out,
                          cudaStream_t st) {
  if (!n) return;
  k_stack_scatter<<<grid_for(n, kBlock), kBlock, 0, st>>>(top, keep, pos, n, out);
}

void launch_gather_ranges(const int32_t *src, const uint64_t *starts, const uint64_t *dst_off, uint64_t nr,
                          int32_t *dst, cudaStream_t st) {
  if (!nr) return;
  k_gather_ranges<<<(unsigned)(nr < 4096 ? nr : 4096), kBlock, 0, st>>>(src, starts, dst_off, nr, dst);
}

}  // namespace gfz

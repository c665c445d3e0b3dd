// Shared device helpers for the GFAz transform kernels (sm_103a).
//
// 2-mer packing follows the reference's include/grammar/packed_2mer.hpp:15-48:
// pack(a,b) = (int64)a << 32 | (uint32)b, reverse = pack(-b,-a), and the
// canonical key is the SIGNED minimum of the two.  All arithmetic on node
// symbols is int32 with wrap-around, which is what the reference's int32
// arithmetic produces on every supported compiler.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gfz {

// pack(0x01010101, 0x01010101): its reverse pack(-0x01010101, -0x01010101) is
// negative and therefore smaller, so this value is never a canonical key and
// can mark empty hash slots.
constexpr unsigned long long kEmptyKey = 0x0101010101010101ULL;

// Hash-slot flag bits.
constexpr uint32_t kFlagRepeated = 1u;  // canonical pair seen at least twice
constexpr uint32_t kFlagUsed = 2u;      // rule chosen at least once this round

// Error bits reported through the per-context status word.
constexpr uint32_t kErrTableFull = 1u;     // probe sequence exceeded its bound
constexpr uint32_t kErrLookupMiss = 2u;    // a counted pair was not in the table
constexpr uint32_t kErrTimeout = 4u;       // a bounded spin-wait gave up
constexpr uint32_t kErrDepth = 8u;         // rule nesting deeper than the stack
constexpr uint32_t kErrLength = 16u;       // rule/traversal length overflow or mismatch
constexpr uint32_t kErrRuleCycle = 32u;    // rule lengths did not resolve
constexpr uint32_t kErrBadSymbol = 64u;    // symbol outside the valid range

// Spin limit for decoupled look-back; with the nanosleep back-off (up to
// 256 ns per spin) this is several seconds, far beyond any legitimate wait.
constexpr uint32_t kSpinLimit = 1u << 24;

__device__ __forceinline__ int32_t neg32(int32_t x) { return (int32_t)(0u - (uint32_t)x); }
__device__ __forceinline__ uint32_t abs32(int32_t x) {
  return x < 0 ? 0u - (uint32_t)x : (uint32_t)x;
}
__device__ __forceinline__ unsigned long long pack2(int32_t a, int32_t b) {
  return ((unsigned long long)(uint32_t)a << 32) | (unsigned long long)(uint32_t)b;
}
__device__ __forceinline__ int32_t key_first(unsigned long long k) { return (int32_t)(uint32_t)(k >> 32); }
__device__ __forceinline__ int32_t key_second(unsigned long long k) { return (int32_t)(uint32_t)k; }
__device__ __forceinline__ unsigned long long rev2(unsigned long long k) {
  return pack2(neg32(key_second(k)), neg32(key_first(k)));
}
// signed comparison of packed keys
__device__ __forceinline__ bool key_le(unsigned long long a, unsigned long long b) {
  return (long long)a <= (long long)b;
}
__device__ __forceinline__ unsigned long long canon2(unsigned long long k) {
  unsigned long long r = rev2(k);
  return key_le(k, r) ? k : r;
}

// Symbol |x| = a is rule min_id + r for r < nrules; anything else is a step.
__device__ __forceinline__ bool is_rule(uint32_t a, uint32_t min_id, uint64_t nrules) {
  return a >= min_id && (uint64_t)(a - min_id) < nrules;
}

// 32-bit slot hash of a packed key: the halves are combined with an odd
// (golden-ratio) multiplier, then mixed by MurmurHash3's 32-bit finaliser
// (Appleby, public domain).  Cheaper than a 64-bit mix and ample for tables
// of at most 2^31 slots.
__device__ __forceinline__ uint32_t hash_pair(unsigned long long k) {
  uint32_t h = (uint32_t)k * 0x9E3779B1u + (uint32_t)(k >> 32);
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}

// ---- access to decoupled look-back descriptors ------------------------------
// A descriptor carries its status bits and its payload in one 64-bit word and
// no tile reads anything else a predecessor wrote, so gpu-scope relaxed
// accesses suffice: they are coherent in L2, and unlike acquire loads they do
// not hold back a thread's later loads, so a lane keeps all of its look-back
// loads in flight at once.
__device__ __forceinline__ void st_desc(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_desc(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Descriptor status lives in the top two bits.
constexpr unsigned long long kDescAgg = 1ULL << 62;
constexpr unsigned long long kDescIncl = 2ULL << 62;
constexpr unsigned long long kDescMask = 3ULL << 62;
constexpr unsigned long long kDescPayload = ~kDescMask;

// Waits (bounded) until descriptor j is published; on timeout sets
// kErrTimeout and returns an inclusive zero so the caller terminates.
__device__ __forceinline__ unsigned long long wait_desc(const unsigned long long *desc, uint64_t j,
                                                        uint32_t *err) {
  unsigned long long d = ld_desc(desc + j);
  uint32_t spins = 0;
  unsigned ns = 32;
  while ((d & kDescMask) == 0) {
    if (++spins > kSpinLimit) {
      atomicOr(err, kErrTimeout);
      return kDescIncl;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
    d = ld_desc(desc + j);
  }
  return d;
}

// Warp-parallel decoupled look-back, executed by all 32 lanes of one warp.
// Each step inspects a window of 32 * K predecessors, lane l taking tiles
// (base - l*K - i), i < K, with all its loads in flight together; the
// aggregates between the tile and the nearest inclusive descriptor are
// combined with an order-preserving shuffle reduction.  Once a tile turns
// inclusive, every tile within one window of it completes in one more round
// trip, so the inclusive frontier advances 32 * K - 1 tiles per round trip.
// Op supplies the scan monoid:
//   T  aggregate (a function of the incoming state); S concrete state
//   identity(), compose(a, b) = "a then b", apply(f, s), initial()
//   encode_agg/decode_agg, encode_incl/decode_incl (62-bit payloads)
//   shfl_down(T, o), shfl0(T)
// Publishes this tile's aggregate, then its inclusive state, and returns the
// exclusive state (the state before this tile) on every lane.
template <class Op, int K = 4>
__device__ __forceinline__ typename Op::S warp_lookback(unsigned long long *desc, uint64_t tile,
                                                        const typename Op::T &agg, uint32_t *err) {
  using T = typename Op::T;
  using S = typename Op::S;
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    const S s0 = Op::initial();
    if (lane == 0) st_desc(desc, kDescIncl | (Op::encode_incl(Op::apply(agg, s0)) & kDescPayload));
    return s0;
  }
  if (lane == 0) st_desc(desc + tile, kDescAgg | (Op::encode_agg(agg) & kDescPayload));
  const unsigned long long before_first = kDescIncl | (Op::encode_incl(Op::initial()) & kDescPayload);
  T acc = Op::identity();
  int64_t base = (int64_t)tile - 1;
  for (;;) {
    unsigned long long d[K];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int64_t j = base - (int64_t)(lane * K + i);
      d[i] = j >= 0 ? ld_desc(desc + j) : before_first;
    }
#pragma unroll
    for (int i = 0; i < K; ++i)
      if ((d[i] & kDescMask) == 0) d[i] = wait_desc(desc, (uint64_t)(base - (int64_t)(lane * K + i)), err);
    int first = K;  // my nearest inclusive descriptor
#pragma unroll
    for (int i = K - 1; i >= 0; --i)
      if ((d[i] & kDescMask) == kDescIncl) first = i;
    const uint32_t incl = __ballot_sync(0xffffffffu, first < K);
    const int L = incl ? __ffs(incl) - 1 : 32;
    const int limit = lane < L ? K : (lane == L ? first : 0);
    T f = Op::identity();
    unsigned long long mine = before_first;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      if (i < limit) f = Op::compose(Op::decode_agg(d[i] & kDescPayload), f);
      if (i == first) mine = d[i];
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T other = Op::shfl_down(f, o);
      if (lane + o < 32) f = Op::compose(other, f);
    }
    const T window = Op::shfl0(f);
    acc = Op::compose(window, acc);
    if (L < 32) {
      const unsigned long long dl = __shfl_sync(0xffffffffu, mine, L);
      const S excl = Op::apply(acc, Op::decode_incl(dl & kDescPayload));
      if (lane == 0) st_desc(desc + tile, kDescIncl | (Op::encode_incl(Op::apply(agg, excl)) & kDescPayload));
      return excl;
    }
    base -= 32 * K;
  }
}

// Block-wide exclusive sum of a u64 per thread; also returns the total.
// The warps' sums are scanned by warp 0 alone (every thread used to add
// them all up in turn).
template <int BLOCK>
__device__ __forceinline__ unsigned long long block_excl_sum(unsigned long long v, unsigned long long &total) {
  constexpr int NW = BLOCK / 32;
  static_assert(NW >= 1 && NW <= 32, "one lane per warp sum");
  __shared__ unsigned long long s_w[NW];
  __shared__ unsigned long long s_x[NW + 1];  // the warps' exclusive offsets, then the total
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    unsigned long long o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) s_w[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long w = lane < NW ? s_w[lane] : 0ull;
    unsigned long long x = w;
#pragma unroll
    for (int d = 1; d < NW; d <<= 1) {
      const unsigned long long o = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += o;
    }
    if (lane < NW) s_x[lane] = x - w;
    if (lane == NW - 1) s_x[NW] = x;
  }
  __syncthreads();
  total = s_x[NW];
  return s_x[warp] + inc - v;
}

// u64 running sum.
struct SumOp {
  using T = unsigned long long;
  using S = unsigned long long;
  __device__ static T identity() { return 0; }
  __device__ static T compose(T a, T b) { return a + b; }
  __device__ static S apply(T f, S s) { return s + f; }
  __device__ static S initial() { return 0; }
  __device__ static unsigned long long encode_agg(T a) { return a; }
  __device__ static T decode_agg(unsigned long long d) { return d; }
  __device__ static unsigned long long encode_incl(S s) { return s; }
  __device__ static S decode_incl(unsigned long long d) { return d; }
  __device__ static T shfl_down(T a, int o) { return __shfl_down_sync(0xffffffffu, a, o); }
  __device__ static T shfl0(T a) { return __shfl_sync(0xffffffffu, a, 0); }
};

// Dynamic tile index: guarantees that every tile a block waits on has
// already been claimed by a running (or finished) block.
__device__ __forceinline__ uint32_t claim_tile(uint32_t *counter) {
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  return s_tile;
}

// First index t in [0, count] with off[t] >= v (off sorted, off[count] = N).
__device__ __forceinline__ uint64_t lower_bound_u64(const uint64_t *off, uint64_t count, uint64_t v) {
  uint64_t lo = 0, hi = count + 1;
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (off[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Marks, in the shared bitmap `bits`, bit (q - base) for every traversal
// start q = off[t] with base <= q <= base + len (the bit at len flags whether
// the element after the tile starts a traversal; off[T] = N is included so
// that position N counts as a start).  Returns the first such t.  All
// threads of the block must call it; `bits` must hold len + 1 bits and be
// zeroed beforehand; a __syncthreads() must follow before reading.
__device__ __forceinline__ uint64_t mark_heads(const uint64_t *off, uint64_t ntrav, uint64_t base,
                                               uint32_t len, uint32_t *bits, uint64_t *s_tlo) {
  if (threadIdx.x == 0) *s_tlo = lower_bound_u64(off, ntrav, base);
  __syncthreads();
  uint64_t tlo = *s_tlo;
  for (uint64_t t = tlo + threadIdx.x; t <= ntrav; t += blockDim.x) {
    uint64_t q = off[t];
    if (q > base + len) break;
    uint32_t b = (uint32_t)(q - base);
    atomicOr(&bits[b >> 5], 1u << (b & 31));
  }
  return tlo;
}

// Padded shared-memory index: one spare word per 32, so that both striped
// access (consecutive i per lane) and blocked access (lane t reading
// t*ITEMS + k) hit 32 distinct banks.
__device__ __forceinline__ uint32_t padi(uint32_t i) { return i + (i >> 5); }
__host__ __device__ constexpr uint32_t padded_size(uint32_t n) { return n + (n >> 5) + 1; }

// ---- bulk async copies (TMA) with mbarrier completion -----------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// Makes initialised barriers visible to the async proxy.
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Orders this thread's earlier generic-proxy shared accesses before later
// async-proxy (bulk copy) accesses of the same buffer.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global memory into this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for phase `parity` of `bar`; false after kSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i >= 16) __nanosleep(128);
  }
  return false;
}

// ---- tile staging ---------------------------------------------------------
// Copies src[0, cnt) (global) into dst[0, cnt) (shared, 16-byte aligned).  A
// full tile whose source is 16-byte aligned moves as 16-byte vectors, every
// load issued before the first shared store, so a thread keeps TILE/(4*BLOCK)
// loads in flight; anything else is copied element-wise.  All threads call it.
template <int BLOCK, uint32_t TILE>
__device__ __forceinline__ void stage_in(const int32_t *__restrict__ src, uint32_t cnt, int32_t *dst) {
  static_assert(TILE % (4 * BLOCK) == 0, "a tile must be whole 16-byte vectors per thread");
  constexpr int V = TILE / (4 * BLOCK);
  if (cnt == TILE && (reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
    const int4 *s4 = reinterpret_cast<const int4 *>(src);
    int4 r[V];
#pragma unroll
    for (int i = 0; i < V; ++i) r[i] = s4[threadIdx.x + i * BLOCK];
#pragma unroll
    for (int i = 0; i < V; ++i) reinterpret_cast<int4 *>(dst)[threadIdx.x + i * BLOCK] = r[i];
  } else {
    for (uint32_t i = threadIdx.x; i < cnt; i += BLOCK) dst[i] = src[i];
  }
}

// Copies shared src[0, cnt) to global dst[0, cnt): 16-byte vectors for a
// full tile with a 16-byte aligned destination, element-wise otherwise.
template <int BLOCK, uint32_t TILE>
__device__ __forceinline__ void stage_out(int32_t *__restrict__ dst, const int32_t *src, uint32_t cnt) {
  if (cnt == TILE && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
    for (uint32_t i = threadIdx.x; i < TILE / 4; i += BLOCK)
      reinterpret_cast<int4 *>(dst)[i] = reinterpret_cast<const int4 *>(src)[i];
  } else {
    for (uint32_t i = threadIdx.x; i < cnt; i += BLOCK) dst[i] = src[i];
  }
}

// Copies shared src[shift, shift + cnt) to global dst[0, cnt) where `shift`
// is dst's position inside its 16-byte word, in elements (so that staging
// and destination share alignment): whole vectors in the middle, single
// elements in the partial words at both ends.  dst must be 4-byte aligned.
template <int BLOCK>
__device__ __forceinline__ void stage_out_phased(int32_t *dst, const int32_t *src, uint32_t shift, uint32_t cnt) {
  const uint32_t end = shift + cnt;
  const uint32_t nvec = (end + 3) >> 2;
  const uintptr_t gbase = reinterpret_cast<uintptr_t>(dst) - 4u * shift;  // 16-byte aligned
  for (uint32_t v = threadIdx.x; v < nvec; v += BLOCK) {
    const uint32_t e0 = v << 2;
    if (e0 >= shift && e0 + 4 <= end) {
      *reinterpret_cast<int4 *>(gbase + 16u * v) = reinterpret_cast<const int4 *>(src)[v];
    } else {
      const uint32_t lo = e0 > shift ? e0 : shift, hi = e0 + 4 < end ? e0 + 4 : end;
      for (uint32_t e = lo; e < hi; ++e) *reinterpret_cast<int32_t *>(gbase + 4u * e) = src[e];
    }
  }
}

// ---- two-stage tile pipeline -----------------------------------------------
// Stage b holds sv[b][0 .. TILE + 4) = steps base .. base + TILE + 3 of the
// stream (base = tile * TILE; the element after the tile is the lookahead of
// its last pair) and hb[b][0 .. HW) = the traversal-head bitmap words from
// base / 32 on (bit q set <=> a traversal starts at position q; position n
// counts as a start).  While a block works on one stage, the next tile is
// already on its way into the other.
template <uint32_t TILE>
struct TilePipe {
  static constexpr uint32_t HW = TILE / 32 + 4;
  int32_t sv[2][TILE + 4];
  uint32_t hb[2][HW];
  unsigned long long bar[2];
};

// Fills stage b with tile `tile`: two bulk copies issued by thread 0 when
// the tile and its lookahead lie inside the stream and the stream is 16-byte
// aligned, plain loads by all threads otherwise (only the last tiles).
// `heads` holds head_words words.  Returns whether the bulk path was taken;
// all threads call it and get the same answer.
template <int BLOCK, uint32_t TILE>
__device__ __forceinline__ bool pipe_issue(TilePipe<TILE> &P, int b, uint64_t tile, const int32_t *s, uint64_t n,
                                           const uint32_t *heads, uint64_t head_words) {
  constexpr uint32_t HW = TilePipe<TILE>::HW;
  const uint64_t base = tile * TILE;
  const bool bulk = base + TILE + 4 <= n && ((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(heads)) & 15u) == 0 &&
                    base / 32 + HW <= head_words;
  if (bulk) {
    if (threadIdx.x == 0) {
      fence_proxy_async();
      mbar_expect_tx(&P.bar[b], (TILE + 4) * 4 + HW * 4);
      bulk_load(P.sv[b], s + base, (TILE + 4) * 4, &P.bar[b]);
      bulk_load(P.hb[b], heads + base / 32, HW * 4, &P.bar[b]);
    }
  } else {
    const uint32_t cnt = (uint32_t)(n - base < TILE + 4 ? n - base : TILE + 4);
    for (uint32_t j = threadIdx.x; j < cnt; j += BLOCK) P.sv[b][j] = s[base + j];
    for (uint32_t j = threadIdx.x; j < HW; j += BLOCK) P.hb[b][j] = base / 32 + j < head_words ? heads[base / 32 + j] : 0u;
  }
  return bulk;
}

// Waits until stage b is filled.  `phases` holds each stage's barrier phase
// bit.  Returns false (on every thread) if a bulk copy did not complete in
// time; the caller then stops using the pipeline.
template <uint32_t TILE>
__device__ __forceinline__ bool pipe_wait(TilePipe<TILE> &P, int b, bool bulk, uint32_t &phases) {
  bool ok = true;
  if (bulk) {
    ok = mbar_wait(&P.bar[b], (phases >> b) & 1u);
    phases ^= 1u << b;
  }
  return __syncthreads_and(ok) != 0;
}

// Ends the use of a stage: orders this thread's generic accesses of it
// before the bulk copy that refills it, and frees it block-wide.
__device__ __forceinline__ void pipe_release() {
  fence_proxy_async();
  __syncthreads();
}

// Bits [b, b + 32) of a shared bitmap (reads bits[b >> 5] and the word after).
__device__ __forceinline__ uint32_t bits_from(const uint32_t *bits, uint32_t b) {
  const uint32_t w = b >> 5;
  const unsigned long long two = ((unsigned long long)bits[w + 1] << 32) | bits[w];
  return (uint32_t)(two >> (b & 31));
}

__device__ __forceinline__ bool bit_at(const uint32_t *bits, uint32_t b) {
  return (bits[b >> 5] >> (b & 31)) & 1u;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

}  // namespace gfz

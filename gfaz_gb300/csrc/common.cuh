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
// can mark empty hash slots.  Its byte-repeated form lets cudaMemsetAsync
// clear a table.
constexpr unsigned long long kEmptyKey = 0x0101010101010101ULL;
constexpr int kEmptyByte = 0x01;

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

// Spin limit for decoupled look-back; with the nanosleep back-off this is
// well over a second, far beyond any legitimate wait.
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

// 64-bit finaliser (murmur3 fmix64) for slot selection.
__device__ __forceinline__ unsigned long long hash64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

// ---- release/acquire access for decoupled look-back descriptors ----------
__device__ __forceinline__ void st_release(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
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
  unsigned long long d = ld_acquire(desc + j);
  uint32_t spins = 0;
  unsigned ns = 32;
  while ((d & kDescMask) == 0) {
    if (++spins > kSpinLimit) {
      atomicOr(err, kErrTimeout);
      return kDescIncl;
    }
    __nanosleep(ns);
    if (ns < 1024) ns <<= 1;
    d = ld_acquire(desc + j);
  }
  return d;
}

// Sum look-back for a u64 running total (payload limited to 62 bits).
// Called by one thread; returns the exclusive prefix of tile `tile`.
__device__ __forceinline__ unsigned long long lookback_sum(unsigned long long *desc, uint64_t tile,
                                                           unsigned long long agg, uint32_t *err) {
  if (tile == 0) {
    st_release(desc, kDescIncl | (agg & kDescPayload));
    return 0;
  }
  st_release(desc + tile, kDescAgg | (agg & kDescPayload));
  unsigned long long excl = 0;
  uint64_t j = tile;
  while (j > 0) {
    --j;
    unsigned long long d = wait_desc(desc, j, err);
    excl += d & kDescPayload;
    if ((d & kDescMask) == kDescIncl) break;
  }
  st_release(desc + tile, kDescIncl | ((excl + agg) & kDescPayload));
  return excl;
}

// Warp-parallel decoupled look-back, executed by all 32 lanes of one warp.
// Lane l inspects tile (tile - 1 - l - 32k); the aggregates between the tile
// and the nearest inclusive descriptor are combined with an order-preserving
// shuffle reduction.  Op supplies the scan monoid:
//   T  aggregate (a function of the incoming state); S concrete state
//   identity(), compose(a, b) = "a then b", apply(f, s), initial()
//   encode_agg/decode_agg, encode_incl/decode_incl (62-bit payloads)
//   shfl_down(T, o), shfl(S, src)
// Publishes this tile's aggregate, then its inclusive state, and returns the
// exclusive state (the state before this tile) on every lane.
template <class Op>
__device__ __forceinline__ typename Op::S warp_lookback(unsigned long long *desc, uint64_t tile,
                                                        const typename Op::T &agg, uint32_t *err) {
  using T = typename Op::T;
  using S = typename Op::S;
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    const S s0 = Op::initial();
    if (lane == 0) st_release(desc, kDescIncl | (Op::encode_incl(Op::apply(agg, s0)) & kDescPayload));
    return s0;
  }
  if (lane == 0) st_release(desc + tile, kDescAgg | (Op::encode_agg(agg) & kDescPayload));
  T acc = Op::identity();
  int64_t base = (int64_t)tile - 1;
  for (;;) {
    const int64_t j = base - lane;
    unsigned long long d = kDescIncl | (Op::encode_incl(Op::initial()) & kDescPayload);
    if (j >= 0) d = wait_desc(desc, (uint64_t)j, err);
    const uint32_t incl = __ballot_sync(0xffffffffu, (d & kDescMask) == kDescIncl);
    const int L = incl ? __ffs(incl) - 1 : 32;
    T f = lane < L ? Op::decode_agg(d & kDescPayload) : Op::identity();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T other = Op::shfl_down(f, o);
      if (lane + o < 32) f = Op::compose(other, f);
    }
    const T window = Op::shfl0(f);
    acc = Op::compose(window, acc);
    if (L < 32) {
      const unsigned long long dl = __shfl_sync(0xffffffffu, d, L);
      const S excl = Op::apply(acc, Op::decode_incl(dl & kDescPayload));
      if (lane == 0) st_release(desc + tile, kDescIncl | (Op::encode_incl(Op::apply(agg, excl)) & kDescPayload));
      return excl;
    }
    base -= 32;
  }
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

__device__ __forceinline__ bool bit_at(const uint32_t *bits, uint32_t b) {
  return (bits[b >> 5] >> (b & 31)) & 1u;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

}  // namespace gfz

// Pangenome growth on decoded traversals (src/workflows/growth_workflow.cpp:
// 261-503): node coverage = the number of haplotype groups whose traversals
// visit the node, then the histogram of coverage over the nodes.
//
// The reference counts a node once per group with per-thread "last seen"
// stamps over groups processed one at a time.  Here every group owns one
// bit of a per-node row (64 groups per 64-bit word), so all traversals of
// all groups set their bits at once; a node's coverage is the popcount of
// its row.  Rows hold a window of words [w0, w1) so that the bitmap can be
// built in passes when it would not fit at once.
#include "common.cuh"
#include "kernels.h"

namespace gfz {

namespace {

constexpr int kGB = 256;
constexpr int kGItems = 8;

// Largest t with off[t] <= p (off[ntrav] > p).
__device__ __forceinline__ uint64_t trav_at(const uint64_t *off, uint64_t ntrav, uint64_t p) {
  uint64_t lo = 0, hi = ntrav;
  while (hi - lo > 1) {
    const uint64_t mid = (lo + hi) >> 1;
    if (off[mid] <= p) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kGB) k_cover_bits(const int32_t *__restrict__ x, uint64_t n,
                                                    const uint64_t *__restrict__ off, uint64_t ntrav,
                                                    const uint32_t *__restrict__ gid, uint64_t num_nodes,
                                                    uint32_t w0, uint32_t w1, unsigned long long *bits) {
  const uint64_t stride = w1 - w0;
  for (uint64_t p0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) * kGItems; p0 < n;
       p0 += (uint64_t)gridDim.x * blockDim.x * kGItems) {
    uint64_t t = trav_at(off, ntrav, p0), tend = off[t + 1];
    uint32_t g = gid[t];
    // row word and bit of every step (want: bit k = the step needs its bit);
    // a step repeating the previous step's node and group is skipped
    uint64_t idx[kGItems];
    unsigned long long bit[kGItems];
    uint32_t want = 0;
    uint64_t last = ~0ull;
    uint32_t lastg = 0;
#pragma unroll
    for (int k = 0; k < kGItems; ++k) {
      const uint64_t p = p0 + k;
      idx[k] = 0;
      bit[k] = 0;
      if (p < n) {
        while (p >= tend) {
          ++t;
          tend = off[t + 1];
          g = gid[t];
        }
        const uint32_t w = g >> 6;
        const int32_t v = x[p];
        const uint32_t a = v < 0 ? 0u - (uint32_t)v : (uint32_t)v;
        if (w >= w0 && w < w1 && a != 0 && a <= num_nodes) {
          idx[k] = (uint64_t)a * stride + (w - w0);
          bit[k] = 1ull << (g & 63);
          if (!(idx[k] == last && g == lastg)) want |= 1u << k;
          last = idx[k];
          lastg = g;
        }
      }
    }
    // all row loads in flight before any is resolved
    unsigned long long cur[kGItems];
#pragma unroll
    for (int k = 0; k < kGItems; ++k) cur[k] = (want >> k) & 1u ? bits[idx[k]] : ~0ull;
#pragma unroll
    for (int k = 0; k < kGItems; ++k)
      if (!(cur[k] & bit[k])) atomicOr(&bits[idx[k]], bit[k]);
  }
}

// cov[v] += the number of bits set in node v's row.
__global__ void k_cover_count(const unsigned long long *__restrict__ bits, uint64_t num_nodes, uint32_t stride,
                              uint32_t *cov) {
  for (uint64_t v = 1 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v <= num_nodes;
       v += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t c = 0;
    for (uint32_t w = 0; w < stride; ++w) c += __popcll(bits[v * stride + w]);
    cov[v] += c;
  }
}

// hist[c] += nodes 1 .. num_nodes with coverage c (c <= nh); per-block
// shared-memory bins when they fit, else warp-aggregated global atomics.
template <bool SMEM>
__global__ void __launch_bounds__(kGB) k_cover_hist(const uint32_t *__restrict__ cov, uint64_t num_nodes, uint32_t nh,
                                                    unsigned long long *hist) {
  extern __shared__ uint32_t s_bin[];
  if (SMEM) {
    for (uint32_t i = threadIdx.x; i <= nh; i += blockDim.x) s_bin[i] = 0;
    __syncthreads();
  }
  for (uint64_t v0 = blockIdx.x * (uint64_t)blockDim.x; v0 < num_nodes; v0 += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = v0 + threadIdx.x + 1;
    const bool ok = v <= num_nodes && cov[v] <= nh;
    const uint32_t c = ok ? cov[v] : 0xFFFFFFFFu;
    if (SMEM) {
      if (ok) atomicAdd(&s_bin[c], 1u);
    } else {
      const uint32_t peers = __match_any_sync(0xffffffffu, c);
      if (ok && (peers & ((1u << (threadIdx.x & 31)) - 1u)) == 0)
        atomicAdd(&hist[c], (unsigned long long)__popc(peers));
    }
  }
  if (SMEM) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i <= nh; i += blockDim.x)
      if (s_bin[i]) atomicAdd(&hist[i], (unsigned long long)s_bin[i]);
  }
}

inline unsigned grid_for(uint64_t n, int block, unsigned cap = 152u * 16u) {
  uint64_t g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (unsigned)g;
}

}  // namespace

void launch_cover_bits(const int32_t *x, uint64_t n, const uint64_t *off, uint64_t ntrav, const uint32_t *gid,
                       uint64_t num_nodes, uint32_t w0, uint32_t w1, unsigned long long *bits, cudaStream_t st) {
  if (n && ntrav && w1 > w0)
    k_cover_bits<<<grid_for((n + kGItems - 1) / kGItems, kGB, 152u * 32u), kGB, 0, st>>>(x, n, off, ntrav, gid,
                                                                                        num_nodes, w0, w1, bits);
}

void launch_cover_count(const unsigned long long *bits, uint64_t num_nodes, uint32_t stride, uint32_t *cov,
                        cudaStream_t st) {
  if (num_nodes && stride) k_cover_count<<<grid_for(num_nodes, 256), 256, 0, st>>>(bits, num_nodes, stride, cov);
}

void launch_cover_hist(const uint32_t *cov, uint64_t num_nodes, uint32_t nh, unsigned long long *hist,
                       cudaStream_t st) {
  if (!num_nodes) return;
  const unsigned grid = grid_for(num_nodes, kGB, 152u * 4u);
  if ((uint64_t)nh + 1 <= 8192)
    k_cover_hist<true><<<grid, kGB, ((size_t)nh + 1) * sizeof(uint32_t), st>>>(cov, num_nodes, nh, hist);
  else
    k_cover_hist<false><<<grid, kGB, 0, st>>>(cov, num_nodes, nh, hist);
}

}  // namespace gfz

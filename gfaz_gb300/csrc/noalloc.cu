// Allocation-free inverse delta: the per-traversal inverse delta kernel run
// with its look-back scratch taken from a fixed device array instead of the
// stream-ordered pool.
//
// Who needs it: callers that may not allocate device memory at all.  A host
// application whose own pool allocator owns nearly all of HBM leaves no room
// for a second allocator; a plug-in inside such a host is often forbidden to
// allocate; and a latency-bound service loop cannot afford cudaMalloc or
// cudaFree, which can synchronise the whole device and stall its other
// streams.  These callers own their input, output and offset buffers and
// want the decode step to touch nothing else.
//
// The scratch (status word, tile counter, one look-back descriptor per
// 4096-step tile of the inverse-delta kernel) is a file-scope __device__
// array of kScratchBytes.  Every GPU that loads this library holds it until
// the process exits.  All calls on a device share it and it keeps the last
// call's contents, so each call clears what must start at zero; two calls
// whose GPU work overlaps (calls from different host threads, on any streams
// of the same device) race on it and must be serialised by the caller.
#include "noalloc.h"

#include <mutex>
#include <stdexcept>
#include <string>

#include "common.cuh"
#include "kernels.h"
#include "pipeline.h"

namespace gfz {

namespace {

// One look-back descriptor per inverse-delta tile of the largest stream.
constexpr uint64_t kMaxTiles = kNoAllocMaxSteps / kInverseDeltaTile;
static_assert(kMaxTiles * kInverseDeltaTile == kNoAllocMaxSteps, "the step limit is a whole number of tiles");
constexpr size_t kCounterOffset = 128;         // tile counter, after DevStatus
constexpr size_t kDescOffset = 256;            // descriptors, 256-byte aligned
constexpr size_t kScratchBytes = kDescOffset + kMaxTiles * sizeof(unsigned long long);
static_assert(kScratchBytes == 131328, "the documented scratch size");
static_assert(sizeof(DevStatus) <= kCounterOffset, "status must fit before the counter");
constexpr int kMaxDevices = 64;

}  // namespace

// The scratch itself: 131,328 bytes on every device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

std::mutex g_setup_mu;
unsigned char *g_scratch_addr[kMaxDevices];  // device address per ordinal

// One-time set-up per device, run by the first call made with that device
// current: in host code g_noalloc_scratch names a host-side stand-in, not a
// device address, so the address comes from cudaGetSymbolAddress (which may
// also make the runtime load device code on that device).
unsigned char *scratch_for(int dev) {
  if (dev < 0 || dev >= kMaxDevices) throw std::invalid_argument("device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(static scratch)");
    g_scratch_addr[dev] = static_cast<unsigned char *>(p);
  }
  return g_scratch_addr[dev];
}

// The buffers are the caller's and the kernel dereferences them as given:
// only device memory of device `dev` is accepted (managed and mapped host
// memory are refused, since a mapped pointer's device address can differ
// from its host address).
void require_device_memory(const void *p, int dev, const char *what) {
  cudaPointerAttributes a{};
  const cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    throw std::invalid_argument(std::string(what) + ": not a CUDA-visible pointer");
  }
  if (a.type != cudaMemoryTypeDevice || a.device != dev)
    throw std::invalid_argument(std::string(what) + ": not device memory of the current device");
}

// Offsets must run from 0 to n without decreasing; the inverse-delta kernel
// relies on that to stay within its tile.
__global__ void k_check_offsets(const uint64_t *__restrict__ off, uint64_t ntrav, uint64_t n, DevStatus *status) {
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= ntrav; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t v = off[t];
    const bool bad = (t == 0 && v != 0) || (t == ntrav && v != n) || (t < ntrav && off[t + 1] < v);
    if (bad) atomicOr(&status->err, kErrLength);
  }
}

uint32_t read_err(const DevStatus *status, cudaStream_t st) {
  uint32_t e = 0;
  cuda_check(cudaMemcpyAsync(&e, &status->err, sizeof(e), cudaMemcpyDeviceToHost, st), "status read");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
  return e;
}

}  // namespace

void inverse_delta_noalloc(const int32_t *in, int32_t *out, uint64_t n, const uint64_t *offsets, uint64_t ntrav,
                           int delta_round, cudaStream_t st) {
  if (n > kNoAllocMaxSteps)
    throw std::invalid_argument("allocation-free inverse delta: " + std::to_string(n) +
                                " steps exceed the limit of " + std::to_string(kNoAllocMaxSteps) + " steps per call");
  if (delta_round < 0) throw std::invalid_argument("delta_round must be >= 0");
  if (!offsets) throw std::invalid_argument("offsets is NULL");
  if (n && (!in || !out)) throw std::invalid_argument("steps buffer is NULL");
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) % alignof(int32_t) ||
      reinterpret_cast<uintptr_t>(offsets) % alignof(uint64_t))
    throw std::invalid_argument("misaligned buffer");
  if (n && in != out) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(in), b = reinterpret_cast<uintptr_t>(out), bytes = n * 4;
    if (a < b + bytes && b < a + bytes) throw std::invalid_argument("input and output overlap without being equal");
  }
  const uint64_t tiles = inverse_delta_num_tiles(n);
  if (tiles > kMaxTiles) throw std::logic_error("static scratch smaller than the tile count");

  int dev = -1;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  unsigned char *base = scratch_for(dev);
  require_device_memory(offsets, dev, "offsets");
  if (n) {
    require_device_memory(in, dev, "input steps");
    require_device_memory(out, dev, "output steps");
  }
  DevStatus *status = reinterpret_cast<DevStatus *>(base);
  uint32_t *counter = reinterpret_cast<uint32_t *>(base + kCounterOffset);
  unsigned long long *desc = reinterpret_cast<unsigned long long *>(base + kDescOffset);

  cuda_check(cudaMemsetAsync(status, 0, sizeof(DevStatus), st), "status clear");
  {
    uint64_t g = (ntrav + 1 + 255) / 256;
    if (g > 152u * 8u) g = 152u * 8u;
    k_check_offsets<<<(unsigned)g, 256, 0, st>>>(offsets, ntrav, n, status);
    cuda_check(cudaGetLastError(), "offset check launch");
  }
  if (read_err(status, st))
    throw std::invalid_argument("offsets must start at 0, never decrease and end at the step count");
  if (n == 0) return;
  if (in != out) cuda_check(cudaMemcpyAsync(out, in, n * sizeof(int32_t), cudaMemcpyDefault, st), "input copy");
  for (int r = 0; r < delta_round; ++r) {
    cuda_check(cudaMemsetAsync(counter, 0, sizeof(uint32_t), st), "counter clear");
    cuda_check(cudaMemsetAsync(desc, 0, tiles * sizeof(unsigned long long), st), "descriptor clear");
    launch_inverse_delta(out, n, offsets, ntrav, desc, counter, status, st);
    cuda_check(cudaGetLastError(), "inverse delta launch");
  }
  if (const uint32_t e = read_err(status, st)) throw std::runtime_error(describe_device_error("allocation-free inverse delta", e));
}

}  // namespace gfz

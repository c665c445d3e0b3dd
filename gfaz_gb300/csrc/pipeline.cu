// Device pipeline orchestration for the GFAz transform (see pipeline.h).
//
// Compression round loop (src/workflows/compression_workflow.cpp:548-700):
//   count pairs -> stop if no candidate -> greedy replacement with temporary
//   symbols -> collect used rules -> stop if none used -> radix sort by the
//   signed packed key -> final ids next_id + rank -> remap temporaries.
#include "pipeline.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "common.cuh"

namespace gfz {

std::string describe_device_error(const char *stage, uint32_t e) {
  std::string msg = std::string("device error in ") + stage + ":";
  if (e & kErrTableFull) msg += " pair table full;";
  if (e & kErrLookupMiss) msg += " counted pair missing from table;";
  if (e & kErrTimeout) msg += " look-back wait timed out;";
  if (e & kErrDepth) msg += " rule nesting deeper than 64;";
  if (e & kErrLength) msg += " length overflow or mismatch;";
  if (e & kErrRuleCycle) msg += " rule lengths do not resolve (cyclic rulebook);";
  if (e & kErrBadSymbol) msg += " invalid rule key;";
  return msg;
}

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw CudaError(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

namespace {

__global__ void k_split_rules(const long long *rules, uint64_t n, int32_t *first, int32_t *second) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = (unsigned long long)rules[i];
    first[i] = key_first(k);
    second[i] = key_second(k);
  }
}

__global__ void k_gather_pos(const uint64_t *pos, const uint64_t *enc_off, uint64_t ntrav1, uint64_t enc_base,
                             uint64_t *out_off) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < ntrav1; t += (uint64_t)gridDim.x * blockDim.x)
    out_off[t] = pos[enc_off[t] - enc_base];
}

inline unsigned grid_for(uint64_t n, int block, unsigned cap = 152u * 16u) {
  uint64_t g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (unsigned)g;
}

uint64_t next_pow2(uint64_t x) {
  uint64_t c = 1;
  while (c < x) c <<= 1;
  return c;
}

// Steps the tuners time their candidates on: the whole stream up to 2^29
// steps (short runs time unreliably), else its first 2^27 steps;
// GFAZ_TUNE_STEPS sets the prefix for every length.
uint64_t tune_len(const Context &ctx, uint64_t n) {
  if (ctx.tune_steps) return std::min(n, ctx.tune_steps);
  return n <= (1ull << 29) ? n : (1ull << 27);
}

uint64_t ceil_log2(uint64_t x) {
  uint64_t r = 0;
  while ((1ull << r) < x) ++r;
  return r;
}


constexpr uint64_t kMaxTableCap = 1ULL << 31;
constexpr uint64_t kSrefMaxCap = 1ULL << 30;  // largest table whose slots fit a slot reference

// cap scaled down by 2^shift (up by 2^-shift when negative), kept within
// [2^16, the table limit].
uint64_t scale_cap(uint64_t cap, int shift) {
  if (shift >= 0) return std::max<uint64_t>(shift < 63 ? cap >> shift : 0, 1u << 16);
  const int up = std::min(-shift, 40);
  return std::min<uint64_t>(cap << up, kMaxTableCap);
}
constexpr int kPassBatch = 4;  // level passes launched per status read (DevStatus::pass_open slots)
static_assert(kPassBatch <= (int)(sizeof(DevStatus::pass_open) / sizeof(unsigned long long)), "pass slots");


struct Table {
  DevVec<PairSlot> slots;
  explicit Table(cudaStream_t st) : slots(st) {}
  PairTable view(uint64_t cap) { return PairTable{slots.ptr, cap}; }
  // every slot {kEmptyKey, 0, val_init}
  void prepare(uint64_t cap, cudaStream_t st, uint32_t val_init = 0) {
    slots.resize(cap);
    launch_table_clear(view(cap), val_init, st);
  }
};

// Scratch of one greedy replacement pass (per 2048-step tile).
struct ReplaceWork {
  explicit ReplaceWork(cudaStream_t st) : tile_trav(st), tword(st), tile_agg(st), tile_state(st) {}
  DevVec<uint64_t> tile_trav;
  DevVec<uint32_t> tword;
  DevVec<unsigned long long> tile_agg, tile_state;
};

}  // namespace

// GFA_COMPRESSION_DEBUG=1 (the reference's debug switch) prints per-round
// grammar statistics to stderr.
bool debug_enabled() {
  static int on = -1;
  if (on < 0) {
    const char *e = std::getenv("GFA_COMPRESSION_DEBUG");
    on = (e && e[0] && e[0] != '0') ? 1 : 0;
  }
  return on == 1;
}


// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
constexpr unsigned long long kAllOnes = ~0ull;

Context::Context(int device, cudaStream_t stream) : device_(device), desc_(nullptr) {
  cuda_check(cudaSetDevice(device), "cudaSetDevice");
  cudaDeviceProp prop;
  cuda_check(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  sms_ = prop.multiProcessorCount;
  if (stream) {
    stream_ = stream;
  } else {
    // one step above the lowest priority, which the link-bound text of
    // low_stream() takes
    int least = 0, greatest = 0;
    cuda_check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priority range");
    cuda_check(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking, least > greatest ? least - 1 : least),
               "cudaStreamCreate");
    own_stream_ = true;
  }
  // keep freed pool memory cached: repeated calls reuse it without syncs
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  desc_ = DevVec<unsigned long long>(stream_);
  sref_buf = DevVec<uint32_t>(stream_);
  rep_buf = DevVec<uint32_t>(stream_);
  cuda_check(cudaMalloc((void **)&d_status_, sizeof(DevStatus)), "status alloc");
  cuda_check(cudaMallocHost((void **)&h_status_, sizeof(DevStatus)), "status alloc");
  std::memset(h_status_, 0, sizeof(DevStatus));
  cuda_check(cudaMemsetAsync(d_status_, 0, sizeof(DevStatus), stream_), "status clear");
  if (const char *e = std::getenv("GFAZ_TUNE_STEPS")) {
    const long long v = std::atoll(e);
    if (v > 0) tune_steps = (uint64_t)v;
  }
  // earlier tuner decisions: lines "kernel class variant" of GFAZ_TUNE_FILE
  if (const char *f = std::getenv("GFAZ_TUNE_FILE")) {
    if (FILE *fp = std::fopen(f, "r")) {
      int k, c, v;
      while (std::fscanf(fp, "%d %d %d", &k, &c, &v) == 3) tuned[{k, c}] = v;
      std::fclose(fp);
    }
  }
}

void Context::record_tuned(int kernel, int cls, int variant) {
  tuned[{kernel, cls}] = variant;
  if (const char *f = std::getenv("GFAZ_TUNE_FILE")) {
    if (FILE *fp = std::fopen(f, "a")) {
      std::fprintf(fp, "%d %d %d\n", kernel, cls, variant);
      std::fclose(fp);
    }
  }
}

Context::~Context() {
  cudaStreamSynchronize(stream_);
  for (auto &p : pending_) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : event_pool_) cudaEventDestroy(e);
  // every device vector of the context frees on its stream: before the
  // stream is destroyed below
  desc_.release();
  sref_buf.release();
  rep_buf.release();
  cudaStreamSynchronize(stream_);
  cudaFree(d_status_);
  cudaFreeHost(h_status_);
  if (stage_) cudaFreeHost(stage_);
  for (auto &h : host_) {
    if (h.pinned) cudaFreeHost(h.p);
    else std::free(h.p);
  }
  if (low_) {
    cudaStreamSynchronize(low_);
    cudaStreamDestroy(low_);
    for (auto e : order_ev_) cudaEventDestroy(e);
  }
  if (own_stream_) cudaStreamDestroy(stream_);
}

cudaStream_t Context::low_stream() {
  if (!low_) {
    int least = 0, greatest = 0;
    cuda_check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priority range");
    cuda_check(cudaStreamCreateWithPriority(&low_, cudaStreamNonBlocking, least), "low-priority stream");
    for (auto &e : order_ev_) cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
  }
  return low_;
}

void Context::order(cudaStream_t from, cudaStream_t to) {
  cudaEvent_t e = order_ev_[from == stream_ ? 0 : 1];
  cuda_check(cudaEventRecord(e, from), "event record");
  cuda_check(cudaStreamWaitEvent(to, e, 0), "stream wait");
}

int32_t *Context::host_buffer(int i, uint64_t n) {
  HostStage &h = host_[i];
  n = std::max<uint64_t>(n, 1);
  if (h.n >= n) return h.p;
  if (h.pinned) cudaFreeHost(h.p);
  else std::free(h.p);
  h = HostStage{};
  if (cudaHostAlloc(reinterpret_cast<void **>(&h.p), n * sizeof(int32_t), cudaHostAllocDefault) == cudaSuccess) {
    h.pinned = true;
  } else {
    cudaGetLastError();
    h.p = static_cast<int32_t *>(std::malloc(n * sizeof(int32_t)));
    if (!h.p) throw std::bad_alloc();
  }
  h.n = n;
  return h.p;
}

void Context::reset_status() {
  launch_zero_bytes(d_status_, offsetof(DevStatus, sticky_err), stream_);
  count_launch();
}

const DevStatus &Context::read_status() {
  // h_status_ is page-locked: the kernel writes it straight into host memory
  launch_copy_bytes(d_status_, h_status_, sizeof(DevStatus), stream_);
  count_launch();
  sync();
  return *h_status_;
}

char *Context::stage(size_t bytes) {
  const size_t need = (bytes + 15) & ~size_t(15);
  if (stage_used_ + need > stage_cap_) {
    sync();  // every queued transfer through the staging is done
    if (need > stage_cap_) {
      if (stage_) cudaFreeHost(stage_);
      stage_ = nullptr;
      stage_cap_ = 0;
      const size_t cap = std::max<size_t>(need, 4u << 20);
      cuda_check(cudaMallocHost(reinterpret_cast<void **>(&stage_), cap), "staging alloc");
      stage_cap_ = cap;
    }
  }
  char *p = stage_ + stage_used_;
  stage_used_ += need;
  return p;
}

// Page-locked (or device) memory a kernel can address directly.
static bool device_addressable(const void *p) {
  cudaPointerAttributes a{};
  const bool ok = cudaPointerGetAttributes(&a, p) == cudaSuccess &&
                  (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice);
  (void)cudaGetLastError();
  return ok;
}

void Context::upload(void *dst, const void *src, size_t bytes, bool bulk) {
  if (!bytes) return;
  if (bytes > kSmallCopy) {
    if (!bulk && device_addressable(src)) {
      launch_copy_bytes(src, dst, bytes, stream_);
      count_launch();
    } else {
      cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, stream_), "upload");
    }
    return;
  }
  char *p = stage(bytes);
  std::memcpy(p, src, bytes);
  launch_copy_bytes(p, dst, bytes, stream_);
  count_launch();
}

void Context::download(void *dst, const void *src, size_t bytes, bool bulk) {
  if (!bytes) return;
  if (bytes > kSmallCopy) {
    if (!bulk && device_addressable(dst)) {
      launch_copy_bytes(src, dst, bytes, stream_);
      count_launch();
    } else {
      cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, stream_), "download");
    }
    return;
  }
  char *p = stage(bytes);
  launch_copy_bytes(src, p, bytes, stream_);
  count_launch();
  downloads_.push_back(PendingDownload{dst, p, bytes});
}

void Context::zero(void *dst, size_t bytes) {
  if (!bytes) return;
  launch_zero_bytes(dst, bytes, stream_);
  count_launch();
}

void Context::sync() {
  cuda_check(cudaStreamSynchronize(stream_), "stream sync");
  for (const PendingDownload &d : downloads_) std::memcpy(d.dst, d.from, d.bytes);
  downloads_.clear();
  stage_used_ = 0;
}

void Context::check_status(const char *stage) {
  const uint32_t e = h_status_->err | h_status_->sticky_err;
  if (!e) return;
  if (h_status_->sticky_err) {
    h_status_->sticky_err = 0;
    zero(&d_status_->sticky_err, sizeof(uint32_t));
  }
  throw std::runtime_error(describe_device_error(stage, e));
}

unsigned long long *Context::lookback(uint64_t tiles, uint32_t **counter) { return lookback_n(tiles, 1, counter); }

unsigned long long *Context::lookback_n(uint64_t tiles, int n, uint32_t **counters) {
  tiles = std::max<uint64_t>(tiles, 1);
  // the n regions, then the n tile counters (two to a word): one fill
  const uint64_t words = tiles * (uint64_t)n + ((uint64_t)n + 1) / 2;
  desc_.resize(words);
  zero(desc_.ptr, words * sizeof(unsigned long long));
  uint32_t *c = reinterpret_cast<uint32_t *>(desc_.ptr + tiles * (uint64_t)n);
  for (int k = 0; k < n; ++k) counters[k] = c + k;
  return desc_.ptr;
}

float Context::time_launches(const std::function<void()> &launch) {
  cudaEvent_t a = take_event(), b = take_event();
  cuda_check(cudaEventRecord(a, stream_), "event record");
  launch();
  cuda_check(cudaEventRecord(b, stream_), "event record");
  cuda_check(cudaEventSynchronize(b), "event sync");
  float ms = 0;
  cuda_check(cudaEventElapsedTime(&ms, a, b), "event time");
  event_pool_.push_back(a);
  event_pool_.push_back(b);
  return ms;
}

cudaEvent_t Context::take_event() {
  if (!event_pool_.empty()) {
    cudaEvent_t e = event_pool_.back();
    event_pool_.pop_back();
    return e;
  }
  cudaEvent_t e;
  cuda_check(cudaEventCreate(&e), "cudaEventCreate");
  return e;
}

void Context::tbegin(const char *name, double bytes) {
  launches_++;
  if (!timing) return;
  open_name_ = name;
  open_bytes_ = bytes;
  open_a_ = take_event();
  cudaEventRecord(open_a_, stream_);
}

void Context::tend() {
  if (!timing || !open_a_) return;
  cudaEvent_t b = take_event();
  cudaEventRecord(b, stream_);
  pending_.push_back(Pending{open_name_, open_a_, b, open_bytes_});
  open_a_ = nullptr;
}

std::map<std::string, KernelStat> Context::kernel_stats() {
  cudaStreamSynchronize(stream_);
  for (auto &p : pending_) {
    float ms = 0;
    cudaEventElapsedTime(&ms, p.a, p.b);
    auto &s = stats_[p.name];
    s.ms += ms;
    s.launches++;
    s.bytes += p.bytes;
    event_pool_.push_back(p.a);
    event_pool_.push_back(p.b);
  }
  pending_.clear();
  return stats_;
}

void Context::add_bytes(const char *name, double bytes) {
  if (timing) stats_[name].bytes += bytes;
}

void Context::clear_kernel_stats() {
  kernel_stats();
  stats_.clear();
  launches_ = 0;
}

// Launch bracketed by timing events; `bytes` = algorithmic bytes of the
// launch (what it must read and write at minimum).
#define GFZ_TIMED_B(ctx, name, bytes, expr) \
  do {                                      \
    (ctx).tbegin(name, (double)(bytes));    \
    expr;                                   \
    (ctx).tend();                           \
  } while (0)
#define GFZ_TIMED(ctx, name, expr) GFZ_TIMED_B(ctx, name, 0, expr)

// ---------------------------------------------------------------------------
// Compression
// ---------------------------------------------------------------------------
// Used rules of one round: the (key, slot) list and the sort's scratch.
struct SortWork {
  explicit SortWork(cudaStream_t st) : keys(st), keys_tmp(st), slots(st), slots_tmp(st), hist(st) {}
  DevVec<unsigned long long> keys, keys_tmp;
  DevVec<uint32_t> slots, slots_tmp, hist;
};

// Sorts the U used rules of su.keys / su.slots by signed key (on the key
// bytes in byte_mask), gives them ids next_id + rank in the table and
// appends their keys to rules after the first nrules entries.
static void sort_used_rules(Context &ctx, PairTable tab, uint64_t U, uint32_t byte_mask, uint32_t next_id,
                            SortWork &su, DevVec<long long> &rules, uint64_t nrules) {
  cudaStream_t st = ctx.stream();
  DevStatus *ds = ctx.dstatus();
  su.keys_tmp.resize(U);
  su.slots_tmp.resize(U);
  su.hist.resize(8 * 256);
  ctx.zero(su.hist.ptr, 8 * 256 * sizeof(uint32_t));
  ctx.reset_status();
  bool in_tmp = false;
  GFZ_TIMED(ctx, "radix_sort", launch_sort_hist(su.keys.ptr, U, byte_mask, su.hist.ptr, st));
  // the look-back regions of all passes, cleared at once
  const int passes = __builtin_popcount(byte_mask);
  const uint64_t region = sort_tiles(U) * 256;
  uint32_t *counters[8];
  unsigned long long *desc = ctx.lookback_n(region, std::max(passes, 1), counters);
  int pass = 0;
  for (int b = 0; b < 8; ++b) {
    if (!((byte_mask >> b) & 1u)) continue;
    GFZ_TIMED(ctx, "radix_sort",
              launch_sort_pass(in_tmp ? su.keys_tmp.ptr : su.keys.ptr, in_tmp ? su.slots_tmp.ptr : su.slots.ptr,
                               in_tmp ? su.keys.ptr : su.keys_tmp.ptr, in_tmp ? su.slots.ptr : su.slots_tmp.ptr, U, b,
                               su.hist.ptr, desc + region * pass, counters[pass], &ds->err, st));
    ++pass;
    in_tmp = !in_tmp;
  }
  rules.reserve(nrules + U, true);
  rules.size = nrules + U;
  GFZ_TIMED(ctx, "assign_ids",
            launch_assign_ids(in_tmp ? su.keys_tmp.ptr : su.keys.ptr, in_tmp ? su.slots_tmp.ptr : su.slots.ptr, U,
                              next_id, tab, rules.ptr + nrules, st));
}

// Greedy left-to-right replacement of A[0, n) (traversal offsets offA, head
// bitmap heads): inside each traversal, a position whose canonical pair is
// REPEATED in tab and whose predecessor was not replaced becomes
// +-(temp_base + slot).  Writes B and offB and sets the bit of every used
// slot in used_bits (zeroed, tab.cap bits); the output length lands in
// status u64[2] for the caller to read.
// With sref / rep_bits (the count's slot references and repeated-slot
// bitmap) the classification and emit passes read them instead of probing
// the table.
static void replace_pairs(Context &ctx, const int32_t *A, uint64_t n, const uint64_t *offA, uint64_t ntrav,
                          const uint32_t *heads, PairTable tab, int32_t temp_base, int32_t *B, uint64_t *offB,
                          uint32_t *used_bits, int cls, ReplaceWork &w, const uint32_t *sref = nullptr,
                          const uint32_t *rep_bits = nullptr) {
  cudaStream_t st = ctx.stream();
  DevStatus *ds = ctx.dstatus();
  const uint64_t tiles = apply_num_tiles(n);
  uint32_t *counter;
  unsigned long long *desc = ctx.lookback(apply_state_blocks(n), &counter);
  w.tile_trav.resize(std::max<uint64_t>(tiles, 1));
  w.tword.resize(std::max<uint64_t>(tiles * 256, 1));
  w.tile_agg.resize(std::max<uint64_t>(tiles, 1));
  w.tile_state.resize(std::max<uint64_t>(tiles, 1));
  GFZ_TIMED(ctx, "tile_trav", launch_tile_trav(offA, ntrav, n, w.tile_trav.ptr, st));
  const ApplyScratch sc{w.tword.ptr, w.tile_agg.ptr, w.tile_state.ptr, desc, counter};
  if (sref) {
    GFZ_TIMED_B(ctx, "apply_classify", 4.0 * n, launch_apply_classify_sref(sref, n, rep_bits, sc, st));
    GFZ_TIMED(ctx, "apply_states", launch_apply_states(n, sc, ds, st));
    GFZ_TIMED_B(ctx, "apply_emit", 8.0 * n,
                launch_apply_emit_sref(A, sref, n, offA, ntrav, w.tile_trav.ptr, tab, temp_base, B, offB, used_bits, sc,
                                       ds, st));
    return;
  }
  // classify variant: forced by option, else tuned per stream class like
  // the count kernel (both write the same words); emit follows the choice
  // (it flags rules used, so a second timing run would not be alike)
  bool flat = ctx.classify_kernel == 1;
  if (ctx.classify_kernel < 0) {
    const auto it = ctx.tuned.find({Context::kTuneClassify, cls});
    if (it != ctx.tuned.end()) {
      flat = it->second == 1;
    } else {
      // timed on the stream's first steps; the full pass follows
      const uint64_t ns = tune_len(ctx, n);
      const float t_tiled = ctx.time_launches([&] { launch_apply_classify(A, ns, heads, tab, sc, false, ds, st); });
      const float t_flat = ctx.time_launches([&] { launch_apply_classify(A, ns, heads, tab, sc, true, ds, st); });
      flat = t_flat < t_tiled;
      ctx.record_tuned(Context::kTuneClassify, cls, flat ? 1 : 0);
      if (debug_enabled())
        fprintf(stderr, "[gfaz gb300] classify tuner: class %d n=%llu persistent %.3f ms, flat %.3f ms\n", cls,
                (unsigned long long)n, t_tiled, t_flat);
    }
  }
  GFZ_TIMED_B(ctx, "apply_classify", 4.0 * n, launch_apply_classify(A, n, heads, tab, sc, flat, ds, st));
  GFZ_TIMED(ctx, "apply_states", launch_apply_states(n, sc, ds, st));
  GFZ_TIMED_B(ctx, "apply_emit", 4.0 * n,
              launch_apply_emit(A, n, heads, offA, ntrav, w.tile_trav.ptr, tab, temp_base, B, offB, used_bits, sc, flat,
                                ds, st));
}

// Grammar rounds round0 .. rounds - 1 over the device-resident stream A (n
// steps, offsets offA; B / offB the other buffers), continuing from next_id
// and the previous round's distinct pair count.  Used rules are appended to
// rules (g.nrules so far) and g's counters advance; on return A / offA hold
// the result, n its length.
static void run_rounds(Context &ctx, DevVec<int32_t> &A, DevVec<int32_t> &B, DevVec<uint64_t> &offA,
                       DevVec<uint64_t> &offB, uint64_t ntrav, uint64_t &n, uint32_t &next_id, uint64_t &prev_distinct,
                       int round0, int rounds, DevVec<long long> &rules, Grammar &g) {
  cudaStream_t st = ctx.stream();
  DevStatus *ds = ctx.dstatus();
  Table tab(st);
  SortWork su(st);
  DevVec<unsigned long long> &ukeys = su.keys;
  DevVec<uint32_t> &uslots = su.slots;
  DevVec<uint32_t> heads(st), used_bits(st);
  // the count's slot references and repeated-slot bitmap, kept by the context
  DevVec<uint32_t> &sref = ctx.sref_buf, &rep_bits = ctx.rep_buf;
  ReplaceWork rw(st);

  for (int round = round0; round < rounds; ++round) {
    if (n < 2) break;
    const auto round_t0 = std::chrono::steady_clock::now();
    // first round: at most 4M distinct pairs expected (delta-coded
    // traversals repeat few pairs); the table grows when it runs fuller
    // later rounds: distinct pairs grow by up to ~3x per round as rules
    // pair with each other
    uint64_t est = prev_distinct ? prev_distinct * 3 : std::min<uint64_t>(n / 8, 1u << 22);
    est = std::min(est, n);
    uint64_t cap = next_pow2(std::max<uint64_t>(est * 2, 1u << 16));
    const bool forced_cap = round == 0 && ctx.first_table_cap;
    if (forced_cap) cap = ctx.first_table_cap;
    uint64_t distinct = 0, repeated = 0;
    heads.resize(head_words(n));
    ctx.zero(heads.ptr, head_words(n) * sizeof(uint32_t));
    GFZ_TIMED(ctx, "head_bits", launch_head_bits(offA.ptr, ntrav, heads.ptr, st));
    // Count kernel: forced by option, else the faster of the tiled and the
    // flat kernel for this stream class (first round or not, length, and the
    // previous round's distinct pairs per step), timed on the first stream
    // of the class and remembered by the context.  Both fill the table alike.
    const int cls = (round == 0 ? 0 : 1) * 1000 + 4 * (int)ceil_log2(n) +
                    (round == 0 ? 0 : (int)std::min<uint64_t>(3, prev_distinct * 4 / std::max<uint64_t>(n, 1)));
    CountKernel kind = ctx.warp_dedup ? CountKernel::kTiledWarpDedup : CountKernel::kTiled;
    // table size: the estimate's size scaled by the power of two the
    // load-factor tuner kept for this class and round (tuned below, once
    // the distinct pairs are known; negative when the table had to grow)
    const int cap_cls = cls * 16 + std::min(round, 15);
    const uint64_t cap_default = cap;
    bool tune_cap = false;
    if (ctx.table_tuner && !forced_cap) {
      const auto it = ctx.tuned.find({Context::kTuneCap, cap_cls});
      if (it != ctx.tuned.end()) cap = scale_cap(cap, it->second);
      else tune_cap = true;
    }
    bool tune = false;
    if (ctx.count_kernel >= 0) {
      kind = (CountKernel)ctx.count_kernel;
    } else if (!ctx.warp_dedup) {
      const auto it = ctx.tuned.find({Context::kTuneCount, cls});
      if (it != ctx.tuned.end()) kind = (CountKernel)it->second;
      else tune = true;
    }
    // slot references: every count kernel but the warp-folding one records
    // them (the tuner's candidates never include it)
    const bool use_sref = ctx.slot_refs && kind != CountKernel::kTiledWarpDedup;
    uint32_t *d_sref = nullptr, *d_rep = nullptr;
    if (use_sref) {
      sref.resize(n);
      d_sref = sref.ptr;
    }
    // the table cleared for a count, with its repeated-slot bitmap and the
    // replacement's used-slot bitmap (one launch)
    auto prepare = [&](uint64_t c) {
      tab.slots.resize(c);
      used_bits.resize((c + 31) / 32);
      if (use_sref) {
        rep_bits.resize((c + 31) / 32);
        d_rep = rep_bits.ptr;
      }
      launch_table_clear(tab.view(c), 0, st, use_sref ? rep_bits.ptr : nullptr, used_bits.ptr);
      ctx.count_launch();
    };
    for (;;) {
      if (cap > kMaxTableCap) throw std::runtime_error("pair table would exceed 2^31 slots");
      if (tune) {
        // every candidate kernel counts the stream's first tune_len steps
        // into a cleared table; the full count with the fastest follows
        const CountKernel cand[] = {CountKernel::kTiled, CountKernel::kFlat, CountKernel::kFlat4};
        constexpr int kCand = sizeof(cand) / sizeof(cand[0]);
        float best = 0, t[kCand] = {};
        bool refill = false;
        const uint64_t ns = tune_len(ctx, n);
        for (int i = 0; i < kCand; ++i) {
          prepare(cap);
          ctx.reset_status();
          t[i] = ctx.time_launches(
              [&] { launch_count_pairs(A.ptr, ns, heads.ptr, tab.view(cap), ds, cand[i], st, d_sref, d_rep); });
          const DevStatus &s0 = ctx.read_status();
          if ((s0.err & kErrTableFull) || s0.u64[0] * 10 > cap * 8) {
            refill = true;
            break;
          }
          if (i == 0 || t[i] < best) {
            best = t[i];
            kind = cand[i];
          }
        }
        if (refill) {
          cap *= 4;
          continue;
        }
        ctx.record_tuned(Context::kTuneCount, cls, (int)kind);
        if (debug_enabled())
          fprintf(stderr, "[gfaz gb300] count tuner: class %d n=%llu tiled %.3f, flat %.3f, flat4 %.3f ms\n", cls,
                  (unsigned long long)ns, t[0], t[1], t[2]);
        tune = false;
        continue;  // the full count
      } else {
        prepare(cap);
        ctx.reset_status();
        GFZ_TIMED_B(ctx, "count_pairs", (use_sref ? 8.0 : 4.0) * n,
                    launch_count_pairs(A.ptr, n, heads.ptr, tab.view(cap), ds, kind, st, d_sref, d_rep));
      }
      const DevStatus &s = ctx.read_status();
      distinct = s.u64[0];
      repeated = s.u64[1];
      if ((s.err & kErrTableFull) || distinct * 10 > cap * 8) {
        cap *= 4;
        continue;
      }
      ctx.check_status("count_pairs");
      break;
    }
    if (tune_cap) {
      // hash load factor: the count (with its table clear) timed with the
      // estimate's table and with 2, 4 and 8 times smaller ones that keep
      // the load at 1/2 or below for the distinct pairs just counted; the
      // fastest shrink factor is kept for the class and round
      std::vector<uint64_t> caps = {cap};
      for (int sh = 1; sh <= 3; ++sh) {
        const uint64_t c = cap_default >> sh;
        if (c >= 2 * distinct && c >= (1u << 16) && c < cap) caps.push_back(c);
      }
      uint64_t best = cap;
      float tbest = -1;
      const uint64_t ns = tune_len(ctx, n);  // timed on the stream's first steps
      for (const uint64_t c : caps) {
        ctx.reset_status();
        const float t = ctx.time_launches([&] {
          prepare(c);
          launch_count_pairs(A.ptr, ns, heads.ptr, tab.view(c), ds, kind, st, d_sref, d_rep);
        });
        // a probe chain past its limit at this load: not a candidate (the
        // next reset clears the bit)
        if (ctx.read_status().err & kErrTableFull) continue;
        if (tbest < 0 || t < tbest) {
          tbest = t;
          best = c;
        }
      }
      if (debug_enabled())
        fprintf(stderr, "[gfaz gb300] load-factor tuner: class %d distinct=%llu table %llu -> %llu slots\n", cls,
                (unsigned long long)distinct, (unsigned long long)cap, (unsigned long long)best);
      ctx.record_tuned(Context::kTuneCap, cap_cls, (int)ceil_log2(cap_default) - (int)ceil_log2(best));
      cap = best;
      // the timed runs cleared the table: the full count at the kept size
      prepare(cap);
      ctx.reset_status();
      GFZ_TIMED_B(ctx, "count_pairs", (use_sref ? 8.0 : 4.0) * n,
                  launch_count_pairs(A.ptr, n, heads.ptr, tab.view(cap), ds, kind, st, d_sref, d_rep));
      ctx.read_status();
      ctx.check_status("count_pairs");
    }
    prev_distinct = distinct;
    if (repeated == 0) break;  // no candidates: stop all rounds
    if ((uint64_t)next_id + cap >= (1ULL << 31))
      throw std::overflow_error("Compression workflow error: rule id space exhausted");
    const int32_t temp_base = (int32_t)next_id;
    ctx.reset_status();
    ctx.upload(&ds->u64[5], &kAllOnes, sizeof(kAllOnes));
    // slot references hold slots below 2^30 (bit 31 and one value are
    // taken); a larger table is classified and emitted by probing
    const bool by_sref = use_sref && cap <= kSrefMaxCap;
    replace_pairs(ctx, A.ptr, n, offA.ptr, ntrav, heads.ptr, tab.view(cap), temp_base, B.ptr, offB.ptr,
                  used_bits.ptr, cls, rw, by_sref ? d_sref : nullptr, by_sref ? d_rep : nullptr);
    ukeys.resize(std::max<uint64_t>(repeated, 1));
    uslots.resize(std::max<uint64_t>(repeated, 1));
    GFZ_TIMED_B(ctx, "collect_used", cap / 8.0,
                launch_collect_used(used_bits.ptr, cap, tab.view(cap), ukeys.ptr, uslots.ptr,
                                    std::max<uint64_t>(repeated, 1), ds, st));
    const DevStatus &s1 = ctx.read_status();
    ctx.check_status("apply");
    const uint64_t n_out = s1.u64[2];
    const uint64_t U = s1.u64[3];
    // key bytes that differ between the used keys: the only radix passes
    const unsigned long long diff = s1.u64[4] ^ s1.u64[5];
    ctx.add_bytes("collect_used", 12.0 * U);
    ctx.add_bytes("apply_emit", 4.0 * n_out);
    if (U == 0) break;  // no rule used: stop all rounds
    uint32_t byte_mask = 0;
    for (int b = 0; b < 8; ++b)
      if ((diff >> (8 * b)) & 0xFF) byte_mask |= 1u << b;
    sort_used_rules(ctx, tab.view(cap), U, byte_mask, next_id, su, rules, g.nrules);
    GFZ_TIMED_B(ctx, "remap", 8.0 * n_out, launch_remap(B.ptr, n_out, temp_base, tab.slots.ptr, st));
    // the sort's error bits reach the host with the next round's count (or
    // the read after the last round): no wait here
    launch_copy_bytes(&ds->err, &ds->sticky_err, sizeof(uint32_t), st);
    ctx.count_launch();
    if (debug_enabled())
      fprintf(stderr,
              "[gfaz gb300] round %d: n=%llu cap=%llu distinct=%llu candidates=%llu used=%llu n_out=%llu "
              "(host %.2f ms)\n",
              round + 1, (unsigned long long)n, (unsigned long long)cap, (unsigned long long)distinct,
              (unsigned long long)repeated, (unsigned long long)U, (unsigned long long)n_out,
              std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - round_t0).count());
    g.nrules += U;
    g.round_end.push_back(g.nrules);
    next_id += (uint32_t)U;
    n = n_out;
    A.swap(B);
    offA.swap(offB);
    g.rounds_done++;
  }
  ctx.read_status();
  ctx.check_status("rule sort");
  if (ctx.hbm_budget) {
    // under a device-memory budget the round scratch is not kept
    sref.release();
    rep_bits.release();
  }
}

void encode_traversals(Context &ctx, const int32_t *d_steps, const std::vector<uint64_t> &h_off,
                       const EncodeParams &p, Grammar &g) {
  cudaStream_t st = ctx.stream();
  const auto t_start = std::chrono::steady_clock::now();
  if (h_off.empty()) throw std::invalid_argument("offsets must hold ntrav + 1 entries");
  const uint64_t ntrav = h_off.size() - 1;
  const uint64_t N = h_off.back();
  for (uint64_t t = 0; t < ntrav; ++t)
    if (h_off[t + 1] < h_off[t]) throw std::invalid_argument("traversal offsets must be non-decreasing");
  if (h_off[0] != 0) throw std::invalid_argument("offsets must start at 0");
  const int dr = std::max(0, p.delta_round);
  g.ntrav = ntrav;
  g.delta_round = dr;
  g.rounds_done = 0;
  g.nrules = 0;
  g.round_end.clear();

  DevVec<uint64_t> offA(st), offB(st);
  offA.resize(ntrav + 1);
  offB.resize(ntrav + 1);
  ctx.upload(offA.ptr, h_off.data(), (ntrav + 1) * sizeof(uint64_t));
  DevVec<int32_t> A(st), B(st);
  A.resize(std::max<uint64_t>(N, 1));
  B.resize(std::max<uint64_t>(N, 1));

  ctx.reset_status();
  DevStatus *ds = ctx.dstatus();
  if (dr == 0) {
    if (N) cuda_check(cudaMemcpyAsync(A.ptr, d_steps, N * sizeof(int32_t), cudaMemcpyDeviceToDevice, st), "copy");
    GFZ_TIMED_B(ctx, "max_abs", 4.0 * N, launch_max_abs(A.ptr, N, &ds->aux, st));
  } else {
    GFZ_TIMED_B(ctx, "delta_encode", 8.0 * N, launch_delta_encode(d_steps, A.ptr, N, offA.ptr, ntrav, &ds->aux, st));
    for (int r = 1; r < dr; ++r) {
      GFZ_TIMED_B(ctx, "delta_encode", 8.0 * N, launch_delta_encode(A.ptr, B.ptr, N, offA.ptr, ntrav, &ds->aux, st));
      A.swap(B);
    }
  }
  const DevStatus &s0 = ctx.read_status();
  if (debug_enabled())
    fprintf(stderr, "[gfaz gb300] delta transform of %llu steps done (host %.2f ms)\n", (unsigned long long)N,
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count());
  const uint32_t max_abs = s0.aux;
  if (max_abs == UINT32_MAX)
    throw std::overflow_error("Compression workflow error: delta values too large for rule ID assignment");
  uint32_t next_id = max_abs + 1;
  g.layer_start = next_id;

  DevVec<long long> rules(st);
  uint64_t n = N;
  uint64_t prev_distinct = 0;
  run_rounds(ctx, A, B, offA, offB, ntrav, n, next_id, prev_distinct, 0, p.rounds, rules, g);
  g.next_id = next_id;
  A.size = n;
  g.enc = std::move(A);
  g.off = std::move(offA);
  g.h_off.resize(ntrav + 1);
  ctx.download(g.h_off.data(), g.off.ptr, (ntrav + 1) * sizeof(uint64_t));
  rules.size = g.nrules;
  g.rules = std::move(rules);
  ctx.sync();
}

// ---------------------------------------------------------------------------
// Compression of a host-resident stream in HBM-sized chunks
// ---------------------------------------------------------------------------
namespace {

// Device bytes the resident rounds need for an n-step stream: two stream
// buffers, head bitmap, per-tile words and tile arrays, the pair table with
// its used bitmap and sort lists, the rulebook and some slack.
uint64_t resident_bytes(uint64_t n, uint64_t prev_distinct, uint64_t nrules) {
  uint64_t est = prev_distinct ? prev_distinct * 3 : std::min<uint64_t>(n / 8, 1u << 22);
  est = std::min(est, n);
  const uint64_t cap = next_pow2(std::max<uint64_t>(est * 2, 1u << 16));
  // + the count's slot references (4 B per step) and repeated-slot bitmap
  return 12 * n + n / 8 + n / 2 + n / 32 + 16 * cap + cap / 4 + 6 * cap + 8 * (nrules + n / 2) + (64ull << 20);
}

// Copies steps [a, b) of the stream made of segs (back to back) to dst.
void upload_range(const std::vector<HostSeg> &segs, uint64_t a, uint64_t b, int32_t *dst, cudaStream_t st) {
  uint64_t base = 0;
  for (const HostSeg &g : segs) {
    const uint64_t lo = std::max(a, base), hi = std::min(b, base + g.n);
    if (lo < hi)
      cuda_check(cudaMemcpyAsync(dst + (lo - a), g.p + (lo - base), (hi - lo) * sizeof(int32_t), cudaMemcpyDefault, st),
                 "chunk upload");
    base += g.n;
  }
}

}  // namespace

void encode_host_chunked(Context &ctx, const std::vector<HostSeg> &input, const std::vector<uint64_t> &h_off,
                         const EncodeParams &p, uint64_t chunk, uint64_t budget, Grammar &g) {
  cudaStream_t st = ctx.stream();
  if (h_off.empty()) throw std::invalid_argument("offsets must hold ntrav + 1 entries");
  const uint64_t ntrav = h_off.size() - 1;
  const uint64_t N = h_off.back();
  for (uint64_t t = 0; t < ntrav; ++t)
    if (h_off[t + 1] < h_off[t]) throw std::invalid_argument("traversal offsets must be non-decreasing");
  if (h_off[0] != 0) throw std::invalid_argument("offsets must start at 0");
  uint64_t have = 0;
  for (const HostSeg &sg : input) have += sg.n;
  if (have != N) throw std::invalid_argument("input segments do not hold the offsets' steps");
  const uint64_t TILE = kApplyTile;
  const uint64_t C = std::max<uint64_t>(TILE, chunk / TILE * TILE);
  const int dr = std::max(0, p.delta_round);
  g.ntrav = ntrav;
  g.delta_round = dr;
  g.rounds_done = 0;
  g.nrules = 0;
  g.round_end.clear();

  DevVec<uint64_t> offA(st), offB(st);
  offA.resize(ntrav + 1);
  offB.resize(ntrav + 1);
  ctx.upload(offA.ptr, h_off.data(), (ntrav + 1) * sizeof(uint64_t));
  // chunk buffers: steps in (one before / one after the chunk), steps out,
  // chunk-relative head bitmap
  DevVec<int32_t> cin(st), cout(st);
  cin.resize(C + 2);
  cout.resize(C);
  DevVec<uint32_t> hloc(st);
  hloc.resize(head_words(C + 1));
  auto local_heads = [&](const uint64_t *off, uint64_t lo, uint64_t span) {
    ctx.zero(hloc.ptr, head_words(C + 1) * sizeof(uint32_t));
    launch_head_bits_range(off, ntrav, lo, span, hloc.ptr, st);
  };
  // host stream buffers (the context keeps them for later calls)
  int32_t *const X = ctx.host_buffer(0, N);
  int32_t *const Y = ctx.host_buffer(1, N);
  ctx.reset_status();
  DevStatus *ds = ctx.dstatus();
  // delta rounds (or the max |x| of the raw steps), chunk by chunk
  std::vector<HostSeg> cur = input;
  int32_t *nxt = X;
  DevVec<int32_t> A(st), B(st);
  // When round 1 will read its input in place (see the round loop; the
  // same size rule, so it always does), the last delta pass (or the max
  // |x| pass) already leaves the stream in that buffer: round 1 does not
  // upload it again, and the stream never goes back to host memory.
  bool a_ready = false;
  bool a_holds = false;  // A holds the current stream (round 1's input)
  bool dev_next = false;  // the current stream is on the device in B (final ids)
  uint64_t Cr0 = C;
  if (budget && dr <= 1 && resident_bytes(N, 0, 0) > budget) {
    uint64_t cap0 = next_pow2(std::max<uint64_t>(std::min<uint64_t>(N / 8, 1u << 22) * 2, 1u << 16));
    if (ctx.first_table_cap) {
      cap0 = ctx.first_table_cap;
    } else if (ctx.table_tuner) {
      const auto it = ctx.tuned.find({Context::kTuneCap, (4 * (int)ceil_log2(N)) * 16});
      if (it != ctx.tuned.end()) cap0 = scale_cap(cap0, it->second);
    }
    const uint64_t fixed0 = N / 2 + N / 64 + 4 * N / 8 + (64ull << 20) + 17 * cap0;
    if (fixed0 + 4 * (N + 2) + 4 * 8 * TILE <= budget) {
      Cr0 = std::min(C, std::max<uint64_t>(TILE, (budget - fixed0 - 4 * (N + 2)) / 4 / TILE * TILE));
      a_ready = true;
      cin.release();
      cout.release();
      cin.resize(Cr0 + 2);
      A.resize(N + 1);
    }
  }
  if (dr == 0) {
    const uint64_t Cd = a_ready ? Cr0 : C;
    for (uint64_t c0 = 0; c0 < N; c0 += Cd) {
      const uint64_t c1 = std::min(c0 + Cd, N);
      int32_t *dst = a_ready ? A.ptr + c0 : cin.ptr;
      upload_range(cur, c0, c1, dst, st);
      GFZ_TIMED_B(ctx, "max_abs", 4.0 * (c1 - c0), launch_max_abs(dst, c1 - c0, &ds->aux, st));
    }
  }
  for (int r = 0; r < dr; ++r) {
    if (a_ready) {  // dr == 1: the output goes to the round-1 buffer only
      for (uint64_t c0 = 0; c0 < N; c0 += Cr0) {
        const uint64_t c1 = std::min(c0 + Cr0, N);
        if (c0) {
          upload_range(cur, c0 - 1, c1, cin.ptr, st);
        } else {
          ctx.zero(cin.ptr, sizeof(int32_t));
          upload_range(cur, 0, c1, cin.ptr + 1, st);
        }
        local_heads(offA.ptr, c0, c1 - c0);
        GFZ_TIMED_B(ctx, "delta_encode", 8.0 * (c1 - c0),
                    launch_delta_chunk(cin.ptr, A.ptr + c0, c1 - c0, hloc.ptr, &ds->aux, st));
      }
      ctx.sync();
      cur.clear();  // the stream is in A only
      continue;
    }
    for (uint64_t c0 = 0; c0 < N; c0 += C) {
      const uint64_t c1 = std::min(c0 + C, N);
      if (c0) {
        upload_range(cur, c0 - 1, c1, cin.ptr, st);
      } else {
        ctx.zero(cin.ptr, sizeof(int32_t));
        upload_range(cur, 0, c1, cin.ptr + 1, st);
      }
      local_heads(offA.ptr, c0, c1 - c0);
      GFZ_TIMED_B(ctx, "delta_encode", 8.0 * (c1 - c0),
                  launch_delta_chunk(cin.ptr, cout.ptr, c1 - c0, hloc.ptr, &ds->aux, st));
      cuda_check(cudaMemcpyAsync(nxt + c0, cout.ptr, (c1 - c0) * sizeof(int32_t), cudaMemcpyDefault, st),
                 "chunk download");
    }
    ctx.sync();
    cur = {HostSeg{nxt, N}};
    nxt = nxt == X ? Y : X;
  }
  a_holds = a_ready;
  const DevStatus &s0 = ctx.read_status();
  const uint32_t max_abs = s0.aux;
  if (max_abs == UINT32_MAX)
    throw std::overflow_error("Compression workflow error: delta values too large for rule ID assignment");
  uint32_t next_id = max_abs + 1;
  g.layer_start = next_id;
  using clk = std::chrono::steady_clock;
  auto t_phase = clk::now();
  auto phase = [&](const char *what) {
    if (!debug_enabled()) return;
    const auto now = clk::now();
    fprintf(stderr, "[gfaz gb300] chunked %s: %.1f ms\n", what,
            std::chrono::duration<double, std::milli>(now - t_phase).count());
    t_phase = now;
  };
  phase("delta");

  DevVec<long long> rules(st);
  Table tab(st);
  SortWork su(st);
  DevVec<uint32_t> used_bits(st);
  ReplaceWork rw(st);
  std::vector<unsigned long long> h_state;
  uint64_t n = N;
  uint64_t prev_distinct = 0;
  bool resident = false;  // the remaining rounds ran on a device-resident stream
  for (int round = 0; round < p.rounds; ++round) {
    if (n < 2) break;
    if (dev_next || (budget && resident_bytes(n, prev_distinct, g.nrules) <= budget)) {
      // the rest fits the budget: one upload, then the resident rounds
      cin.release();
      cout.release();
      tab.slots.release();
      used_bits.release();
      rw.tword.release();
      rw.tile_agg.release();
      rw.tile_state.release();
      rw.tile_trav.release();
      if (dev_next) {  // the previous round left the stream on the device
        A.swap(B);
        B.resize(std::max<uint64_t>(n, 1));
      } else {
        A.resize(std::max<uint64_t>(n, 1));
        B.resize(std::max<uint64_t>(n, 1));
        upload_range(cur, 0, n, A.ptr, st);
      }
      dev_next = false;
      phase("upload for the resident rounds");
      run_rounds(ctx, A, B, offA, offB, ntrav, n, next_id, prev_distinct, round, p.rounds, rules, g);
      ctx.sync();
      phase("resident rounds");
      resident = true;
      break;
    }
    uint64_t est = prev_distinct ? prev_distinct * 3 : std::min<uint64_t>(n / 8, 1u << 22);
    est = std::min(est, n);
    uint64_t cap = next_pow2(std::max<uint64_t>(est * 2, 1u << 16));
    const bool forced_cap = round == 0 && ctx.first_table_cap;
    if (forced_cap) cap = ctx.first_table_cap;
    // the table size kept for this class and round (the resident rounds'
    // tuner key), so that a table that had to grow does not refill again
    const int cls = (round == 0 ? 0 : 1) * 1000 + 4 * (int)ceil_log2(n) +
                    (round == 0 ? 0 : (int)std::min<uint64_t>(3, prev_distinct * 4 / std::max<uint64_t>(n, 1)));
    const int cap_cls = cls * 16 + std::min(round, 15);
    const uint64_t cap_default = cap;
    bool keep_cap = false;
    if (ctx.table_tuner && !forced_cap) {
      const auto it = ctx.tuned.find({Context::kTuneCap, cap_cls});
      if (it != ctx.tuned.end()) cap = scale_cap(cap, it->second);
      else keep_cap = true;
    }
    // Input resident: when the round's input fits the budget beside the
    // per-tile arrays and the table (with output chunks shrunk to the rest),
    // it is uploaded once and the count, classification and emit passes
    // read it in place instead of uploading every chunk three times.
    uint64_t Cr = C;
    // per-tile words and arrays, the table and its used bitmap, and a margin
    const uint64_t fixed_n = n / 2 + n / 64 + 4 * n / 8 + (64ull << 20) + 17 * cap;
    // (with a_ready, round 1 meets this rule: the same table size and sizes)
    const bool in_res = (a_ready && round == 0) || (budget && fixed_n + 4 * (n + 2) + 4 * 8 * TILE <= budget);
    if (in_res) {
      Cr = std::min(C, std::max<uint64_t>(TILE, (budget - fixed_n - 4 * (n + 2)) / 4 / TILE * TILE));
      cin.release();
      cout.release();
      cout.resize(Cr);
      if (!(a_ready && round == 0)) {
        A.resize(n + 1);
        upload_range(cur, 0, n, A.ptr, st);
      }
    } else {
      cin.resize(C + 2);
      cout.resize(C);
    }
    // the chunk with the step after it (pairs across chunk edges); returns
    // where it starts on the device and how many steps it holds
    const int32_t *chunk_ptr = nullptr;
    auto load_chunk = [&](uint64_t c0, uint64_t c1) {
      const uint64_t e = std::min(c1 + 1, n);
      if (in_res) {
        chunk_ptr = A.ptr + c0;
      } else {
        upload_range(cur, c0, e, cin.ptr, st);
        chunk_ptr = cin.ptr;
      }
      local_heads(offA.ptr, c0, c1 - c0);
      return e - c0;
    };
    const CountKernel kind = round == 0 ? CountKernel::kFlat4 : CountKernel::kFlat;
    uint64_t distinct = 0, repeated = 0;
    for (;;) {
      if (cap > kMaxTableCap) throw std::runtime_error("pair table would exceed 2^31 slots");
      tab.prepare(cap, st);
      ctx.reset_status();
      for (uint64_t c0 = 0; c0 < n; c0 += Cr) {
        const uint64_t c1 = std::min(c0 + Cr, n);
        const uint64_t nd = load_chunk(c0, c1);
        GFZ_TIMED_B(ctx, "count_pairs", 4.0 * (c1 - c0),
                    launch_count_pairs(chunk_ptr, nd, hloc.ptr, tab.view(cap), ds, kind, st));
      }
      const DevStatus &s = ctx.read_status();
      distinct = s.u64[0];
      repeated = s.u64[1];
      if ((s.err & kErrTableFull) || distinct * 10 > cap * 8) {
        cap *= 4;
        continue;
      }
      ctx.check_status("count_pairs");
      break;
    }
    if (keep_cap) ctx.record_tuned(Context::kTuneCap, cap_cls, (int)ceil_log2(cap_default) - (int)ceil_log2(cap));
    prev_distinct = distinct;
    if (repeated == 0) break;
    if ((uint64_t)next_id + cap >= (1ULL << 31))
      throw std::overflow_error("Compression workflow error: rule id space exhausted");
    const int32_t temp_base = (int32_t)next_id;
    // classification of every chunk, then the carried-in state of every tile
    const uint64_t tiles = apply_num_tiles(n);
    rw.tile_trav.resize(tiles);
    rw.tword.resize(tiles * 256);
    rw.tile_agg.resize(tiles);
    rw.tile_state.resize(tiles);
    ctx.reset_status();
    ctx.upload(&ds->u64[5], &kAllOnes, sizeof(kAllOnes));
    used_bits.resize((cap + 31) / 32);
    ctx.zero(used_bits.ptr, (cap + 31) / 32 * sizeof(uint32_t));
    uint32_t *counter;
    unsigned long long *desc = ctx.lookback(apply_state_blocks(n), &counter);
    const ApplyScratch sc{rw.tword.ptr, rw.tile_agg.ptr, rw.tile_state.ptr, desc, counter};
    for (uint64_t c0 = 0; c0 < n; c0 += Cr) {
      const uint64_t c1 = std::min(c0 + Cr, n);
      const uint64_t nd = load_chunk(c0, c1);
      GFZ_TIMED_B(ctx, "apply_classify", 4.0 * (c1 - c0),
                  launch_classify_chunk(chunk_ptr, c1 - c0, nd, hloc.ptr, tab.view(cap), c0 / TILE, sc, ds, st));
    }
    GFZ_TIMED(ctx, "apply_states", launch_apply_states(n, sc, ds, st));
    GFZ_TIMED(ctx, "tile_trav", launch_tile_trav(offA.ptr, ntrav, n, rw.tile_trav.ptr, st));
    h_state.resize(tiles);
    ctx.download(h_state.data(), rw.tile_state.ptr, tiles * sizeof(unsigned long long));
    ctx.read_status();
    ctx.check_status("apply");
    // output position of a chunk's first kept step: tile start minus the
    // steps consumed before it, plus its own carried-in consumption
    auto out_start = [&](uint64_t c0) {
      if (c0 >= n) return (uint64_t)0;
      const unsigned long long stt = h_state[c0 / TILE];
      return c0 - (uint64_t)(stt >> 1) + (uint64_t)(stt & 1u);
    };
    for (uint64_t c0 = 0; c0 < n; c0 += Cr) {
      const uint64_t c1 = std::min(c0 + Cr, n);
      load_chunk(c0, c1);
      const uint64_t o0 = out_start(c0);
      GFZ_TIMED_B(ctx, "apply_emit", 4.0 * (c1 - c0),
                  launch_emit_chunk(chunk_ptr, c0, c0 / TILE, apply_num_tiles(c1 - c0), n, offA.ptr, ntrav,
                                    rw.tile_trav.ptr, tab.view(cap), temp_base, cout.ptr, o0, offB.ptr,
                                    used_bits.ptr, sc, ds, st));
      if (c1 < n) {
        const uint64_t o1 = out_start(c1);
        if (o1 > o0)
          cuda_check(cudaMemcpyAsync(nxt + o0, cout.ptr, (o1 - o0) * sizeof(int32_t), cudaMemcpyDefault, st),
                     "chunk download");
      } else {
        const DevStatus &se = ctx.read_status();
        const uint64_t n_end = se.u64[2];
        if (n_end > o0)
          cuda_check(cudaMemcpyAsync(nxt + o0, cout.ptr, (n_end - o0) * sizeof(int32_t), cudaMemcpyDefault, st),
                     "chunk download");
      }
    }
    su.keys.resize(std::max<uint64_t>(repeated, 1));
    su.slots.resize(std::max<uint64_t>(repeated, 1));
    GFZ_TIMED_B(ctx, "collect_used", cap / 8.0,
                launch_collect_used(used_bits.ptr, cap, tab.view(cap), su.keys.ptr, su.slots.ptr,
                                    std::max<uint64_t>(repeated, 1), ds, st));
    const DevStatus &s1 = ctx.read_status();
    ctx.check_status("apply");
    const uint64_t n_out = s1.u64[2];
    const uint64_t U = s1.u64[3];
    const unsigned long long diff = s1.u64[4] ^ s1.u64[5];
    if (U == 0) break;
    uint32_t byte_mask = 0;
    for (int b = 0; b < 8; ++b)
      if ((diff >> (8 * b)) & 0xFF) byte_mask |= 1u << b;
    sort_used_rules(ctx, tab.view(cap), U, byte_mask, next_id, su, rules, g.nrules);
    if (in_res) A.release();
    a_holds = false;
    // final ids into the round's output: when the next round runs resident,
    // the output goes up once and is remapped in place for it; otherwise
    // chunk by chunk through host memory
    dev_next = budget && resident_bytes(n_out, distinct, g.nrules + U) <= budget;
    if (dev_next) {
      cin.release();
      cout.release();
      used_bits.release();
      B.resize(std::max<uint64_t>(n_out, 1));
      if (n_out)
        cuda_check(cudaMemcpyAsync(B.ptr, nxt, n_out * sizeof(int32_t), cudaMemcpyDefault, st), "stream upload");
      GFZ_TIMED_B(ctx, "remap", 8.0 * n_out, launch_remap(B.ptr, n_out, temp_base, tab.slots.ptr, st));
    } else {
      for (uint64_t o0 = 0; o0 < n_out; o0 += Cr) {
        const uint64_t o1 = std::min(o0 + Cr, n_out);
        cuda_check(cudaMemcpyAsync(cout.ptr, nxt + o0, (o1 - o0) * sizeof(int32_t), cudaMemcpyDefault, st),
                   "chunk upload");
        GFZ_TIMED_B(ctx, "remap", 8.0 * (o1 - o0), launch_remap(cout.ptr, o1 - o0, temp_base, tab.slots.ptr, st));
        cuda_check(cudaMemcpyAsync(nxt + o0, cout.ptr, (o1 - o0) * sizeof(int32_t), cudaMemcpyDefault, st),
                   "chunk download");
      }
    }
    ctx.read_status();
    ctx.check_status("rule sort");
    if (debug_enabled())
      fprintf(stderr, "[gfaz gb300] chunked round %d%s: n=%llu chunk=%llu cap=%llu distinct=%llu used=%llu n_out=%llu\n",
              round + 1, in_res ? " (input resident)" : "", (unsigned long long)n, (unsigned long long)Cr,
              (unsigned long long)cap,
              (unsigned long long)distinct, (unsigned long long)U, (unsigned long long)n_out);
    g.nrules += U;
    g.round_end.push_back(g.nrules);
    next_id += (uint32_t)U;
    n = n_out;
    phase("round");
    cur = {HostSeg{nxt, n}};
    nxt = nxt == X ? Y : X;
    offA.swap(offB);
    g.rounds_done++;
  }
  g.next_id = next_id;
  if (resident) {
    A.size = n;
    g.enc = std::move(A);
  } else if (dev_next) {  // the last round's output, remapped on the device
    B.size = n;
    g.enc = std::move(B);
  } else if (a_holds) {  // round 1 stopped before any output: its input
    A.size = n;
    g.enc = std::move(A);
  } else {
    g.enc.resize(std::max<uint64_t>(n, 1));
    g.enc.size = n;
    upload_range(cur, 0, n, g.enc.ptr, st);
  }
  g.off = std::move(offA);
  g.h_off.resize(ntrav + 1);
  ctx.download(g.h_off.data(), g.off.ptr, (ntrav + 1) * sizeof(uint64_t));
  rules.size = g.nrules;
  g.rules = std::move(rules);
  ctx.sync();
}

void exclusive_scan(Context &ctx, const uint32_t *in, uint64_t n, uint64_t *out, const char *timer) {
  uint32_t *counter = nullptr;
  unsigned long long *desc = ctx.lookback(excl_scan_tiles(n), &counter);
  GFZ_TIMED_B(ctx, timer, 12.0 * n, launch_excl_scan_u32(in, n, out, desc, counter, ctx.dstatus(), ctx.stream()));
}

void exclusive_scan(Context &ctx, const uint64_t *in, uint64_t n, uint64_t *out, const char *timer) {
  uint32_t *counter = nullptr;
  unsigned long long *desc = ctx.lookback(excl_scan_tiles(n), &counter);
  GFZ_TIMED_B(ctx, timer, 16.0 * n, launch_excl_scan_u64(in, n, out, desc, counter, ctx.dstatus(), ctx.stream()));
}

bool resident_fits(const Context &ctx, uint64_t n) {
  if (ctx.encode_chunk) return false;
  // input, two stream buffers, the count's slot references, per-tile words,
  // a pair table
  return !ctx.hbm_budget ||
         16 * n + n / 2 + (64ull << 20) + 16 * std::min<uint64_t>(n, 1ull << 23) <= ctx.hbm_budget;
}

void encode_host(Context &ctx, const std::vector<HostSeg> &input, const std::vector<uint64_t> &h_off,
                 const EncodeParams &p, Grammar &g) {
  const uint64_t N = h_off.empty() ? 0 : h_off.back();
  uint64_t chunk = ctx.encode_chunk;
  if (!chunk && ctx.hbm_budget) {
    if (!resident_fits(ctx, N)) {
      // chunked: per-tile words and tile arrays of the whole stream, the
      // first round's pair table and used bitmap, the final stream; chunk
      // buffers of 12 bytes per step
      const uint64_t cap0 = next_pow2(std::max<uint64_t>(std::min<uint64_t>(N / 8, 1u << 22) * 2, 1u << 16));
      const uint64_t fixed = N / 2 + N / 64 + 4 * N / 8 + (64ull << 20) + 17 * cap0;
      if (ctx.hbm_budget <= fixed + 12 * kApplyTile)
        throw std::runtime_error("HBM budget too small for " + std::to_string(N) + " steps");
      chunk = (ctx.hbm_budget - fixed) / 12;
    }
  }
  if (chunk) {
    // with a budget the rounds turn resident once the stream fits it
    encode_host_chunked(ctx, input, h_off, p, chunk, ctx.encode_chunk ? 0 : ctx.hbm_budget, g);
    return;
  }
  cudaStream_t st = ctx.stream();
  DevVec<int32_t> d(st);
  d.resize(std::max<uint64_t>(N, 1));
  uint64_t at = 0;
  for (const HostSeg &sg : input) {
    if (sg.n) ctx.upload(d.ptr + at, sg.p, sg.n * sizeof(int32_t), true);
    at += sg.n;
  }
  if (at != N) throw std::invalid_argument("input segments do not hold the offsets' steps");
  encode_traversals(ctx, d.ptr, h_off, p, g);
}

void rule_columns_delta(Context &ctx, const Grammar &g, DevVec<int32_t> &first, DevVec<int32_t> &second) {
  cudaStream_t st = ctx.stream();
  const uint64_t R = g.nrules;
  first.resize(std::max<uint64_t>(R, 1));
  second.resize(std::max<uint64_t>(R, 1));
  first.size = second.size = R;
  if (!R) return;
  DevVec<int32_t> tf(st), ts(st);
  tf.resize(R);
  ts.resize(R);
  DevVec<uint64_t> off(st);
  off.resize(2);
  const uint64_t h[2] = {0, R};
  ctx.upload(off.ptr, h, sizeof(h));
  GFZ_TIMED(ctx, "split_rules", (k_split_rules<<<grid_for(R, 256), 256, 0, st>>>(g.rules.ptr, R, tf.ptr, ts.ptr)));
  ctx.reset_status();
  GFZ_TIMED(ctx, "delta_encode", launch_delta_encode(tf.ptr, first.ptr, R, off.ptr, 1, &ctx.dstatus()->aux, st));
  GFZ_TIMED(ctx, "delta_encode", launch_delta_encode(ts.ptr, second.ptr, R, off.ptr, 1, &ctx.dstatus()->aux, st));
  ctx.sync();
}

// ---------------------------------------------------------------------------
// Decompression
// ---------------------------------------------------------------------------
void load_rules(Context &ctx, Grammar &g, const int32_t *first, const int32_t *second, uint64_t nrules,
                uint32_t min_id) {
  cudaStream_t st = ctx.stream();
  g.nrules = nrules;
  g.layer_start = min_id;
  g.next_id = min_id + (uint32_t)nrules;
  g.first.resize(std::max<uint64_t>(nrules, 1));
  g.second.resize(std::max<uint64_t>(nrules, 1));
  g.first.size = g.second.size = nrules;
  g.rlen_ready = false;
  g.rpre_state = 0;
  if (!nrules) return;
  ctx.upload(g.first.ptr, first, nrules * 4);
  ctx.upload(g.second.ptr, second, nrules * 4);
  // stored columns are delta coded (codec.cpp:88-95): prefix sums on device
  DevVec<uint64_t> off(st);
  off.resize(2);
  const uint64_t h[2] = {0, nrules};
  ctx.upload(off.ptr, h, sizeof(h));
  ctx.reset_status();
  uint32_t *counter;
  unsigned long long *desc = ctx.lookback(inverse_delta_num_tiles(nrules), &counter);
  GFZ_TIMED(ctx, "inverse_delta",
            launch_inverse_delta(g.first.ptr, nrules, off.ptr, 1, desc, counter, ctx.dstatus(), st));
  desc = ctx.lookback(inverse_delta_num_tiles(nrules), &counter);
  GFZ_TIMED(ctx, "inverse_delta",
            launch_inverse_delta(g.second.ptr, nrules, off.ptr, 1, desc, counter, ctx.dstatus(), st));
  ctx.read_status();
  ctx.check_status("rule decode");
}

void load_encoded(Context &ctx, Grammar &g, const int32_t *enc, const std::vector<uint64_t> &off) {
  cudaStream_t st = ctx.stream();
  if (off.empty() || off[0] != 0) throw std::invalid_argument("encoded offsets must start at 0");
  const uint64_t nt = off.size() - 1, m = off.back();
  g.ntrav = nt;
  g.h_off = off;
  g.off.resize(nt + 1);
  ctx.upload(g.off.ptr, off.data(), (nt + 1) * 8);
  g.enc.resize(std::max<uint64_t>(m, 1));
  g.enc.size = m;
  if (m) ctx.upload(g.enc.ptr, enc, m * 4);
}

// The grammar's rules are known round by round (see Grammar::round_end).
static bool layered(const Grammar &g) { return !g.round_end.empty() && g.round_end.back() == g.nrules; }

static void ensure_rule_lengths(Context &ctx, Grammar &g) {
  if (g.rlen_ready) return;
  cudaStream_t st = ctx.stream();
  const uint64_t R = g.nrules;
  g.rlen.resize(std::max<uint64_t>(R, 1));
  if (R) {
    // the compressor's rulebook (or a compression-side Grammar) provides the
    // columns: derive them when only packed rules exist
    if (g.first.size != R) {
      g.first.resize(R);
      g.second.resize(R);
      g.first.size = g.second.size = R;
      GFZ_TIMED(ctx, "split_rules",
                (k_split_rules<<<grid_for(R, 256), 256, 0, st>>>(g.rules.ptr, R, g.first.ptr, g.second.ptr)));
    }
    ctx.zero(g.rlen.ptr, R * sizeof(uint32_t));
    bool done = false;
    if (layered(g)) {
      // one launch per grammar round over that round's rules: their parts
      // are steps or rules of earlier rounds, whose lengths are known by then
      ctx.reset_status();
      uint64_t lo = 0;
      for (const uint64_t hi : g.round_end) {
        GFZ_TIMED(ctx, "rule_len", launch_rule_len_pass(g.first.ptr, g.second.ptr, R, g.layer_start, g.rlen.ptr,
                                                        ctx.dstatus(), 0, st, lo, hi));
        lo = hi;
      }
      const DevStatus &s = ctx.read_status();
      ctx.check_status("rule lengths");
      done = s.pass_open[0] == 0;  // else the level passes below finish the job
    }
    // level passes in batches, one status read per batch (extra passes
    // after the last level find nothing to do)
    uint64_t prev_open = UINT64_MAX;
    while (!done) {
      ctx.reset_status();
      for (int k = 0; k < kPassBatch; ++k)
        GFZ_TIMED(ctx, "rule_len", launch_rule_len_pass(g.first.ptr, g.second.ptr, R, g.layer_start, g.rlen.ptr,
                                                        ctx.dstatus(), k, st));
      const DevStatus &s = ctx.read_status();
      ctx.check_status("rule lengths");
      const uint64_t open = s.pass_open[kPassBatch - 1];
      if (open == 0) break;
      if (open >= prev_open)
        throw std::runtime_error("rule lengths do not resolve: the rulebook references itself");
      prev_open = open;
    }
  }
  g.rlen_ready = true;
}

// Rule prefix buffers larger than this (in steps) are not built; decoding
// then expands symbol by symbol.
constexpr uint64_t kMaxPrefixSteps = 1ull << 31;

// Builds g.roff / g.rpre once per grammar (see expand_kernels.cu); false when
// the buffer would exceed kMaxPrefixSteps.
static bool ensure_rule_prefix(Context &ctx, Grammar &g) {
  if (g.rpre_state) return g.rpre_state > 0;
  ensure_rule_lengths(ctx, g);
  cudaStream_t st = ctx.stream();
  const uint64_t R = g.nrules;
  g.roff.resize(R + 1);
  ctx.reset_status();
  uint32_t *counter;
  unsigned long long *desc = ctx.lookback(excl_scan_tiles(R), &counter);
  GFZ_TIMED(ctx, "rule_prefix", launch_excl_scan_u32(g.rlen.ptr, R, g.roff.ptr, desc, counter, ctx.dstatus(), st));
  uint64_t steps = 0;
  ctx.download(&steps, g.roff.ptr + R, sizeof(steps));
  ctx.read_status();
  ctx.check_status("rule prefix offsets");
  if (steps > kMaxPrefixSteps) {
    g.rpre_state = -1;
    return false;
  }
  g.rpre.resize(std::max<uint64_t>(steps, 1));
  g.rstat.resize(std::max<uint64_t>(R, 1));
  if (R) {
    DevVec<uint32_t> built(st);
    built.resize(R);
    ctx.zero(built.ptr, R * sizeof(uint32_t));
    const RulePrefixView rv{g.rlen.ptr, g.roff.ptr, g.rpre.ptr, g.rstat.ptr, g.layer_start, R};
    uint32_t first_pass = 1;
    bool done = false;
    if (layered(g)) {
      // one launch per grammar round over that round's rules (their parts'
      // buffers were built by the earlier launches)
      ctx.reset_status();
      uint64_t lo = 0;
      for (const uint64_t hi : g.round_end) {
        GFZ_TIMED_B(ctx, "rule_prefix", 0,
                    launch_rule_prefix_pass(g.first.ptr, g.second.ptr, rv, g.rpre.ptr, g.rstat.ptr,
                                            g.delta_round == 1 ? 1 : 0, built.ptr, first_pass, ctx.dstatus(), 0, st,
                                            lo, hi));
        lo = hi;
        ++first_pass;
      }
      const DevStatus &s = ctx.read_status();
      ctx.check_status("rule prefix");
      done = s.pass_open[0] == 0;  // else the level passes below finish the job
    }
    uint64_t prev_open = UINT64_MAX;
    for (uint32_t pass = first_pass; !done; pass += kPassBatch) {
      ctx.reset_status();
      for (int k = 0; k < kPassBatch; ++k)
        GFZ_TIMED_B(ctx, "rule_prefix", 0,
                    launch_rule_prefix_pass(g.first.ptr, g.second.ptr, rv, g.rpre.ptr, g.rstat.ptr,
                                            g.delta_round == 1 ? 1 : 0, built.ptr, pass + k, ctx.dstatus(), k, st));
      const DevStatus &s = ctx.read_status();
      ctx.check_status("rule prefix");
      const uint64_t open = s.pass_open[kPassBatch - 1];
      if (open == 0) break;
      if (open >= prev_open) throw std::runtime_error("rule expansions do not resolve: the rulebook references itself");
      prev_open = open;
    }
  }
  g.rpre_state = 1;
  return true;
}

// Device data of one expansion: symbol positions, output offsets, symbol
// sums (delta_round 1) and the symbol at each output tile.
struct ExpandPlan {
  explicit ExpandPlan(cudaStream_t st) : pos(st), out_off(st), tile_sym(st), rec(st) {}
  DevVec<uint64_t> pos, out_off, tile_sym;
  DevVec<int4> rec;
  std::vector<uint64_t> h_out_off;
  uint64_t m = 0, total = 0;
  ExpandSource source(const Grammar &g) const {
    return ExpandSource{rec.ptr, pos.ptr, tile_sym.ptr, m, total,
                        RulePrefixView{g.rlen.ptr, g.roff.ptr, g.rpre.ptr, g.rstat.ptr, g.layer_start, g.nrules}};
  }
};

// The prefix decoder applies to delta_round 0 and 1 with a buildable
// prefix buffer; other streams expand symbol by symbol.
static bool prefix_decodable(Context &ctx, Grammar &g, uint64_t t0, uint64_t t1) {
  if (g.delta_round > 1) return false;
  if (g.h_off[t1] == g.h_off[t0]) return false;  // no symbols: nothing to expand
  return ensure_rule_prefix(ctx, g);
}

static void plan_expansion(Context &ctx, Grammar &g, uint64_t t0, uint64_t t1, ExpandPlan &P) {
  cudaStream_t st = ctx.stream();
  const uint64_t e0 = g.h_off[t0], e1 = g.h_off[t1];
  const uint64_t m = e1 - e0, nt = t1 - t0;
  P.m = m;
  P.pos.resize(m + 1);
  P.out_off.resize(nt + 1);
  ctx.reset_status();
  uint32_t *counter;
  unsigned long long *desc = ctx.lookback(scan_num_tiles(m), &counter);
  GFZ_TIMED_B(ctx, "symbol_positions", 12.0 * m, launch_symbol_positions(g.enc.ptr + e0, m, g.layer_start, g.nrules,
                                                             g.rlen.ptr, P.pos.ptr, desc, counter, ctx.dstatus(), st));
  GFZ_TIMED(ctx, "gather_pos", (k_gather_pos<<<grid_for(nt + 1, 256), 256, 0, st>>>(
                                   P.pos.ptr, g.off.ptr + t0, nt + 1, e0, P.out_off.ptr)));
  P.h_out_off.resize(nt + 1);
  ctx.download(P.h_out_off.data(), P.out_off.ptr, (nt + 1) * sizeof(uint64_t));
  ctx.read_status();
  ctx.check_status("expansion offsets");
  P.total = P.h_out_off[nt];
  const RulePrefixView rv{g.rlen.ptr, g.roff.ptr, g.rpre.ptr, g.rstat.ptr, g.layer_start, g.nrules};
  P.rec.resize(m);
  if (g.delta_round == 1) {
    // S_i: segmented (per traversal) exclusive sums of the symbol totals
    DevVec<int32_t> sums(st);
    sums.resize(m);
    DevVec<uint64_t> loc(st);
    std::vector<uint64_t> h_loc(nt + 1);
    for (uint64_t t = 0; t <= nt; ++t) h_loc[t] = g.h_off[t0 + t] - e0;
    loc.resize(nt + 1);
    ctx.upload(loc.ptr, h_loc.data(), (nt + 1) * sizeof(uint64_t));
    GFZ_TIMED_B(ctx, "symbol_sums", 24.0 * m, launch_symbol_records(g.enc.ptr + e0, m, rv, P.rec.ptr, sums.ptr, st));
    desc = ctx.lookback(inverse_delta_num_tiles(m), &counter);
    GFZ_TIMED_B(ctx, "symbol_sums", 8.0 * m,
                launch_inverse_delta(sums.ptr, m, loc.ptr, nt, desc, counter, ctx.dstatus(), st));
    GFZ_TIMED_B(ctx, "symbol_sums", 36.0 * m, launch_symbol_exclusive(P.rec.ptr, sums.ptr, m, st));
  } else {
    GFZ_TIMED_B(ctx, "symbol_sums", 20.0 * m, launch_symbol_records(g.enc.ptr + e0, m, rv, P.rec.ptr, nullptr, st));
  }
  P.tile_sym.resize(expand_num_tiles(P.total) + 1);
  GFZ_TIMED(ctx, "tile_symbols", launch_tile_symbols(P.pos.ptr, m, P.total, P.tile_sym.ptr, st));
}

void prepare_decode(Context &ctx, Grammar &g) {
  ensure_rule_lengths(ctx, g);
  if (g.delta_round <= 1) ensure_rule_prefix(ctx, g);
}

void decode_traversals(Context &ctx, Grammar &g, uint64_t t0, uint64_t t1, DevVec<int32_t> &out,
                       std::vector<uint64_t> &out_off) {
  cudaStream_t st = ctx.stream();
  if (t1 < t0 || t1 > g.ntrav) throw std::out_of_range("traversal range out of bounds");
  ensure_rule_lengths(ctx, g);
  if (prefix_decodable(ctx, g, t0, t1)) {
    ExpandPlan P(st);
    plan_expansion(ctx, g, t0, t1, P);
    out.resize(std::max<uint64_t>(P.total, 1));
    out.size = P.total;
    const ExpandSource E = P.source(g);
    GFZ_TIMED_B(ctx, "expand_steps", 8.0 * P.total, launch_expand_steps(E, g.delta_round, out.ptr, st));
    ctx.read_status();
    ctx.check_status("expansion");
    out_off = std::move(P.h_out_off);
    return;
  }
  const uint64_t e0 = g.h_off[t0], e1 = g.h_off[t1];
  const uint64_t m = e1 - e0;
  const uint64_t nt = t1 - t0;
  DevVec<uint64_t> pos(st), d_out_off(st);
  pos.resize(m + 1);
  d_out_off.resize(nt + 1);
  uint64_t total = 0;
  if (m) {
    ctx.reset_status();
    uint32_t *counter;
    unsigned long long *desc = ctx.lookback(scan_num_tiles(m), &counter);
    GFZ_TIMED_B(ctx, "symbol_positions", 12.0 * m, launch_symbol_positions(g.enc.ptr + e0, m, g.layer_start, g.nrules,
                                                               g.rlen.ptr, pos.ptr, desc, counter, ctx.dstatus(), st));
  } else {
    ctx.zero(pos.ptr, sizeof(uint64_t));
  }
  GFZ_TIMED(ctx, "gather_pos", (k_gather_pos<<<grid_for(nt + 1, 256), 256, 0, st>>>(
                                   pos.ptr, g.off.ptr + t0, nt + 1, e0, d_out_off.ptr)));
  out_off.resize(nt + 1);
  ctx.download(out_off.data(), d_out_off.ptr, (nt + 1) * sizeof(uint64_t));
  const DevStatus &s = ctx.read_status();
  ctx.check_status("expansion offsets");
  (void)s;
  total = out_off[nt];
  out.resize(std::max<uint64_t>(total, 1));
  out.size = total;
  if (m) {
    GFZ_TIMED_B(ctx, "expand", 12.0 * m + 4.0 * total, launch_expand(g.enc.ptr + e0, m, pos.ptr, g.first.ptr, g.second.ptr, g.nrules,
                                           g.layer_start, out.ptr, ctx.dstatus(), st));
  }
  for (int r = 0; r < g.delta_round && total; ++r) {
    uint32_t *counter;
    unsigned long long *desc = ctx.lookback(inverse_delta_num_tiles(total), &counter);
    GFZ_TIMED_B(ctx, "inverse_delta", 8.0 * total,
              launch_inverse_delta(out.ptr, total, d_out_off.ptr, nt, desc, counter, ctx.dstatus(), st));
  }
  ctx.read_status();
  ctx.check_status("expansion");
}

uint64_t emit_text(Context &ctx, const DevVec<int32_t> &x, const std::vector<uint64_t> &off,
                   const TextPieces &pieces, int mode, DevVec<char> &text) {
  cudaStream_t st = ctx.stream();
  const uint64_t nt = off.size() - 1;
  const uint64_t n = off.back();
  if (n == 0) {
    // no steps at all: every line is fixed text (all prefixes + tail)
    std::string all;
    for (uint64_t t = 0; t < nt; ++t) {
      all.append(pieces.blob, pieces.pre_off[t], pieces.pre_off[t + 1] - pieces.pre_off[t]);
      all.append(pieces.blob, pieces.suf_off[t], pieces.suf_off[t + 1] - pieces.suf_off[t]);
    }
    all += pieces.tail;
    text.resize(std::max<uint64_t>(all.size(), 1));
    text.size = all.size();
    if (!all.empty())
      ctx.upload(text.ptr, all.data(), all.size());
    ctx.sync();
    return all.size();
  }
  DevVec<uint64_t> d_off(st), d_pre(st), d_suf(st);
  DevVec<char> d_blob(st), d_tail(st);
  d_off.resize(nt + 1);
  d_pre.resize(nt + 1);
  d_suf.resize(nt + 1);
  d_blob.resize(std::max<size_t>(pieces.blob.size(), 1));
  d_tail.resize(std::max<size_t>(pieces.tail.size(), 1));
  ctx.upload(d_off.ptr, off.data(), (nt + 1) * 8);
  ctx.upload(d_pre.ptr, pieces.pre_off.data(), (nt + 1) * 8);
  ctx.upload(d_suf.ptr, pieces.suf_off.data(), (nt + 1) * 8);
  if (!pieces.blob.empty())
    ctx.upload(d_blob.ptr, pieces.blob.data(), pieces.blob.size());
  if (!pieces.tail.empty())
    ctx.upload(d_tail.ptr, pieces.tail.data(), pieces.tail.size());
  const uint64_t bound = n * 12 + pieces.blob.size() + pieces.tail.size() + 64;
  text.resize(bound);
  TextMeta meta{d_blob.ptr, d_pre.ptr, d_suf.ptr, d_tail.ptr, (uint64_t)pieces.tail.size(), mode};
  ctx.reset_status();
  uint32_t *counter;
  unsigned long long *desc = ctx.lookback(text_num_tiles(n), &counter);
  GFZ_TIMED_B(ctx, "emit_text", 4.0 * n,
            launch_emit_text(x.ptr, n, d_off.ptr, nt, meta, text.ptr, desc, counter, ctx.dstatus(), st));
  const DevStatus &s = ctx.read_status();
  ctx.check_status("text emission");
  text.size = s.u64[7];
  ctx.add_bytes("emit_text", (double)text.size);
  return text.size;
}

// Text pieces on the device.
struct DevPieces {
  explicit DevPieces(cudaStream_t st) : pre(st), suf(st), blob(st), tail(st) {}
  DevVec<uint64_t> pre, suf;
  DevVec<char> blob, tail;
  void upload(Context &ctx, const TextPieces &p) {
    const uint64_t n1 = p.pre_off.size();
    pre.resize(n1);
    suf.resize(n1);
    blob.resize(std::max<size_t>(p.blob.size(), 1));
    tail.resize(std::max<size_t>(p.tail.size(), 1));
    ctx.upload(pre.ptr, p.pre_off.data(), n1 * 8);
    ctx.upload(suf.ptr, p.suf_off.data(), n1 * 8);
    if (!p.blob.empty())
      ctx.upload(blob.ptr, p.blob.data(), p.blob.size());
    if (!p.tail.empty())
      ctx.upload(tail.ptr, p.tail.data(), p.tail.size());
  }
};

// Pieces of the staged host text (each copied while the next is written).
constexpr uint64_t kStagedTextPieces = 8;

uint64_t decode_text(Context &ctx, Grammar &g, uint64_t t0, uint64_t t1,
                     const std::function<TextPieces(const std::vector<uint64_t> &)> &make_pieces, int mode,
                     DevVec<char> &text, char *direct, uint64_t direct_cap) {
  cudaStream_t st = ctx.stream();
  if (t1 < t0 || t1 > g.ntrav) throw std::out_of_range("traversal range out of bounds");
  ensure_rule_lengths(ctx, g);
  if (!prefix_decodable(ctx, g, t0, t1)) {
    DevVec<int32_t> x(st);
    std::vector<uint64_t> off;
    decode_traversals(ctx, g, t0, t1, x, off);
    const uint64_t n = emit_text(ctx, x, off, make_pieces(off), mode, text);
    if (direct) {
      if (direct_cap < n) throw std::length_error("output buffer too small");
      if (n) cuda_check(cudaMemcpyAsync(direct, text.ptr, n, cudaMemcpyDefault, st), "text copy");
      ctx.sync();
    }
    return n;
  }
  ExpandPlan P(st);
  plan_expansion(ctx, g, t0, t1, P);
  const uint64_t nt = t1 - t0;
  const TextPieces pieces = make_pieces(P.h_out_off);
  DevPieces dp(st);
  dp.upload(ctx, pieces);
  DevVec<uint32_t> heads(st);
  heads.resize(head_words(P.total));
  ctx.zero(heads.ptr, head_words(P.total) * sizeof(uint32_t));
  GFZ_TIMED(ctx, "head_bits", launch_head_bits(P.out_off.ptr, nt, heads.ptr, st));
  const TextMeta meta{dp.blob.ptr, dp.pre.ptr, dp.suf.ptr, dp.tail.ptr, (uint64_t)pieces.tail.size(), mode};
  TextSource T{P.out_off.ptr, nt, heads.ptr, meta, 0, &ctx.dstatus()->err};
  const ExpandSource E = P.source(g);
  // text bytes per symbol, their offsets, then the text of every output tile
  DevVec<uint64_t> slen(st), soff(st);
  DevVec<uint8_t> sdig(st);
  slen.resize(P.m);
  soff.resize(P.m + 1);
  sdig.resize(P.m);
  ctx.reset_status();
  GFZ_TIMED_B(ctx, "symbol_text", 24.0 * P.m, launch_symbol_text(E, T, g.delta_round, slen.ptr, sdig.ptr, st));
  uint32_t *counter;
  unsigned long long *desc = ctx.lookback(excl_scan_tiles(P.m), &counter);
  GFZ_TIMED_B(ctx, "symbol_text", 16.0 * P.m,
              launch_excl_scan_u64(slen.ptr, P.m, soff.ptr, desc, counter, ctx.dstatus(), st));
  uint64_t body = 0;
  ctx.download(&body, soff.ptr + P.m, sizeof(body));
  ctx.read_status();
  ctx.check_status("text lengths");
  const uint64_t size = body + pieces.tail.size();
  char *dst;
  bool to_host = false, staged = false;
  if (direct) {
    if (direct_cap < size) throw std::length_error("output buffer too small");
    dst = direct;
    cudaPointerAttributes a{};
    to_host = cudaPointerGetAttributes(&a, direct) == cudaSuccess && a.type == cudaMemoryTypeHost;
    (void)cudaGetLastError();
    if (to_host && ctx.host_text == 1) {
      // staged: the kernel writes HBM, a copy engine moves the bytes
      staged = true;
      text.resize(std::max<uint64_t>(size, 1));
      text.size = size;
      dst = text.ptr;
    }
  } else {
    text.resize(std::max<uint64_t>(size, 1));
    text.size = size;
    dst = text.ptr;
  }
  T.cap = body;
  DevVec<uint64_t> toff(st);
  toff.resize(std::max<uint64_t>(expand_num_tiles(P.total), 1));
  GFZ_TIMED(ctx, "symbol_text", launch_tile_text_off(E, T, g.delta_round, soff.ptr, sdig.ptr, toff.ptr, st));
  if (to_host && !staged) {
    // bound by the chip-to-chip link: on the low-priority stream
    cudaStream_t low = ctx.low_stream();
    ctx.order(st, low);
    GFZ_TIMED_B(ctx, "text_write", 4.0 * P.total + (double)body,
                launch_text_write(E, T, g.delta_round, toff.ptr, dst, low);
                ctx.order(low, st));
  } else if (staged) {
    // in pieces of output tiles: a copy engine moves piece k into host
    // memory (on the low-priority stream) while the kernel writes piece k + 1
    const uint64_t nt = expand_num_tiles(P.total);
    const uint64_t np = std::max<uint64_t>(1, std::min<uint64_t>(nt, kStagedTextPieces));
    std::vector<uint64_t> cut(np + 1), at(np + 1);
    for (uint64_t k = 0; k <= np; ++k) cut[k] = nt * k / np;
    for (uint64_t k = 0; k < np; ++k) ctx.download(&at[k], toff.ptr + cut[k], sizeof(uint64_t));
    ctx.sync();
    at[np] = body;
    cudaStream_t low = ctx.low_stream();
    for (uint64_t k = 0; k < np; ++k) {
      GFZ_TIMED_B(ctx, "text_write", k ? 0.0 : 4.0 * P.total + (double)body,
                  launch_text_write(E, T, g.delta_round, toff.ptr, dst, st, cut[k], cut[k + 1]));
      ctx.order(st, low);
      if (at[k + 1] > at[k])
        cuda_check(cudaMemcpyAsync(direct + at[k], dst + at[k], at[k + 1] - at[k], cudaMemcpyDeviceToHost, low),
                   "text download");
    }
    ctx.order(low, st);
  } else {
    GFZ_TIMED_B(ctx, "text_write", 4.0 * P.total + (double)body,
                launch_text_write(E, T, g.delta_round, toff.ptr, dst, st));
  }
  // the tail (the last line's end) after the body: bytes the text kernel
  // does not write
  if (!pieces.tail.empty()) {
    if (to_host) std::memcpy(direct + body, pieces.tail.data(), pieces.tail.size());
    else ctx.upload(dst + body, pieces.tail.data(), pieces.tail.size());
  }
  ctx.read_status();
  ctx.check_status("text emission");
  return size;
}

// ---------------------------------------------------------------------------
// Append encoding
// ---------------------------------------------------------------------------
void append_encode(Context &ctx, const int32_t *d_first, const int32_t *d_second, uint64_t nrules,
                   const std::vector<Layer> &layers, int delta_round, std::vector<int32_t> &steps,
                   const std::vector<uint64_t> &off, std::vector<uint64_t> &lens, uint32_t &max_abs) {
  cudaStream_t st = ctx.stream();
  const uint64_t nt = off.size() - 1;
  const uint64_t N = off.back();
  DevVec<int32_t> A(st), B(st);
  A.resize(std::max<uint64_t>(N, 1));
  B.resize(std::max<uint64_t>(N, 1));
  DevVec<uint64_t> offA(st), offB(st), d_len(st);
  offA.resize(nt + 1);
  offB.resize(nt + 1);
  ctx.upload(offA.ptr, off.data(), (nt + 1) * 8);
  if (N) ctx.upload(B.ptr, steps.data(), N * 4);
  ctx.reset_status();
  for (int r = 0; r < delta_round; ++r) {
    GFZ_TIMED(ctx, "delta_encode", launch_delta_encode(B.ptr, A.ptr, N, offA.ptr, nt, &ctx.dstatus()->aux, st));
    A.swap(B);
  }
  A.swap(B);  // the stream to encode is in A
  const DevStatus &s = ctx.read_status();
  max_abs = s.aux;
  std::vector<uint64_t> h_off = off;  // offsets of A
  uint64_t n = N;
  if (nrules && nt) {
    Table tab(st);
    DevVec<uint64_t> d_cs(st), d_ce(st), pos(st);
    DevVec<int32_t> top(st);
    DevVec<uint8_t> fl(st);
    DevVec<uint32_t> keep(st);
    for (const Layer &L : layers) {
      const uint64_t count = (uint64_t)(L.end - L.start);
      const uint64_t lo = L.k == 0 ? 0 : L.flat_off / (uint64_t)L.k;
      if (lo + count > nrules) throw std::runtime_error("Add-haplotypes workflow error: rule column is truncated");
      if (!count || !n) continue;
      const uint64_t cap = next_pow2(std::max<uint64_t>(2 * count + 1024, 1u << 12));
      tab.prepare(cap, st, 0xFFFFFFFFu);
      ctx.reset_status();
      GFZ_TIMED(ctx, "build_rule_table",
                launch_build_rule_table(d_first, d_second, lo, lo + count, L.start, tab.view(cap), ctx.dstatus(), st));
      // chunked stack pass; a chunk whose fix-up does not settle within
      // the chunk voids the pass, which is redone with longer chunks and
      // finally one thread per traversal
      bool done = false;
      const std::vector<uint64_t> ladder =
          ctx.append_chunk ? std::vector<uint64_t>{ctx.append_chunk} : std::vector<uint64_t>{256, 2048, 16384};
      for (uint64_t C : ladder) {
        std::vector<uint64_t> cs, ce;
        for (uint64_t t = 0; t < nt; ++t)
          for (uint64_t a = h_off[t]; a < h_off[t + 1]; a += C) {
            const uint64_t b = std::min(a + C, h_off[t + 1]);
            cs.push_back(a | (a == h_off[t] ? kChunkEdge : 0));
            ce.push_back(b | (b == h_off[t + 1] ? kChunkEdge : 0));
          }
        const uint64_t nc = cs.size();
        d_cs.resize(std::max<uint64_t>(nc, 1));
        d_ce.resize(std::max<uint64_t>(nc, 1));
        ctx.upload(d_cs.ptr, cs.data(), nc * 8);
        ctx.upload(d_ce.ptr, ce.data(), nc * 8);
        top.resize(n);
        fl.resize(n);
        ctx.reset_status();
        GFZ_TIMED(ctx, "stack_chunks", launch_stack_chunks(A.ptr, d_cs.ptr, d_ce.ptr, nc, tab.view(cap), top.ptr,
                                                           fl.ptr, &ctx.dstatus()->u64[7], st));
        const DevStatus &sc = ctx.read_status();
        ctx.check_status("append encoding");
        if (sc.u64[7]) continue;
        keep.resize(n);
        pos.resize(n + 1);
        GFZ_TIMED(ctx, "stack_pack", launch_stack_keep(fl.ptr, n, keep.ptr, st));
        uint32_t *counter;
        unsigned long long *desc = ctx.lookback(excl_scan_tiles(n), &counter);
        GFZ_TIMED(ctx, "stack_pack", launch_excl_scan_u32(keep.ptr, n, pos.ptr, desc, counter, ctx.dstatus(), st));
        GFZ_TIMED(ctx, "stack_pack", launch_stack_scatter(top.ptr, keep.ptr, pos.ptr, n, B.ptr, st));
        GFZ_TIMED(ctx, "stack_pack", (k_gather_pos<<<grid_for(nt + 1, 256), 256, 0, st>>>(pos.ptr, offA.ptr, nt + 1,
                                                                                            0, offB.ptr)));
        A.swap(B);
        offA.swap(offB);
        ctx.download(h_off.data(), offA.ptr, (nt + 1) * 8);
        ctx.read_status();
        ctx.check_status("append encoding");
        n = h_off[nt];
        done = true;
        break;
      }
      if (!done) {
        // the reference's stack pass, one thread per traversal, in place;
        // then the traversals are packed back to back again
        std::vector<uint64_t> len(nt);
        for (uint64_t t = 0; t < nt; ++t) len[t] = h_off[t + 1] - h_off[t];
        d_len.resize(nt);
        ctx.upload(d_len.ptr, len.data(), nt * 8);
        GFZ_TIMED(ctx, "stack_encode", launch_stack_encode(A.ptr, offA.ptr, d_len.ptr, nt, tab.view(cap),
                                                           ctx.dstatus(), st));
        ctx.download(len.data(), d_len.ptr, nt * 8);
        ctx.read_status();
        ctx.check_status("append encoding");
        std::vector<uint64_t> packed(nt + 1, 0);
        for (uint64_t t = 0; t < nt; ++t) packed[t + 1] = packed[t] + len[t];
        ctx.upload(offB.ptr, packed.data(), (nt + 1) * 8);
        launch_gather_ranges(A.ptr, offA.ptr, offB.ptr, nt, B.ptr, st);
        A.swap(B);
        offA.swap(offB);
        h_off = packed;
        n = packed[nt];
      }
    }
  }
  lens.resize(nt);
  for (uint64_t t = 0; t < nt; ++t) lens[t] = h_off[t + 1] - h_off[t];
  steps.resize(n);
  if (n) ctx.download(steps.data(), A.ptr, n * 4);
  ctx.sync();
}

}  // namespace gfz

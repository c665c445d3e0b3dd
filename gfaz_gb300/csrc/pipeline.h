// Device pipeline of the GFAz transform: compression (delta + grammar
// rounds) and decompression (expansion + inverse delta + P/W text) on one
// GPU stream.  Host code above this layer (container, parser, workflows,
// C ABI) never touches kernels directly.
#pragma once

#include <cstdint>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.h"

namespace gfz {

// GFA_COMPRESSION_DEBUG set (and not "0"): diagnostics on stderr.
bool debug_enabled();

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
void cuda_check(cudaError_t e, const char *what);
// "device error in <stage>:" followed by one phrase per kErr* bit set in e.
std::string describe_device_error(const char *stage, uint32_t e);

// Growable device array allocated from the stream-ordered pool.
template <typename T>
struct DevVec {
  T *ptr = nullptr;
  uint64_t size = 0, cap = 0;
  cudaStream_t st = nullptr;
  bool owned = true;  // false: a view of another vector's memory (borrow)
  DevVec() = default;
  explicit DevVec(cudaStream_t s) : st(s) {}
  DevVec(const DevVec &) = delete;
  DevVec &operator=(const DevVec &) = delete;
  DevVec(DevVec &&o) noexcept { swap(o); }
  DevVec &operator=(DevVec &&o) noexcept {
    if (this != &o) {
      release();
      swap(o);
    }
    return *this;
  }
  ~DevVec() { release(); }
  void swap(DevVec &o) noexcept {
    std::swap(ptr, o.ptr);
    std::swap(size, o.size);
    std::swap(cap, o.cap);
    std::swap(st, o.st);
    std::swap(owned, o.owned);
  }
  void release() {
    if (ptr && owned) cudaFreeAsync(ptr, st);
    ptr = nullptr;
    size = cap = 0;
    owned = true;
  }
  // Views n elements at p without owning them; the owner must outlive the view.
  void borrow(T *p, uint64_t n) {
    release();
    ptr = p;
    size = cap = n;
    owned = false;
  }
  // Ensures capacity >= n (contents are kept when keep = true).
  void reserve(uint64_t n, bool keep = false) {
    if (n <= cap) return;
    T *np = nullptr;
    cuda_check(cudaMallocAsync((void **)&np, (n ? n : 1) * sizeof(T), st), "device allocation");
    if (keep && ptr && size)
      cuda_check(cudaMemcpyAsync(np, ptr, size * sizeof(T), cudaMemcpyDeviceToDevice, st), "device copy");
    if (ptr && owned) cudaFreeAsync(ptr, st);
    ptr = np;
    cap = n;
    owned = true;
  }
  void resize(uint64_t n, bool keep = false) {
    reserve(n, keep);
    size = n;
  }
};

struct KernelStat {
  double ms = 0;
  uint64_t launches = 0;
  double bytes = 0;  // algorithmic bytes (input read + output written)
};

// One context per (device, stream).  Not thread-safe; calls are
// stream-ordered and synchronous at the C-ABI boundary.
class Context {
 public:
  Context(int device, cudaStream_t stream);
  ~Context();
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;

  int device() const { return device_; }
  cudaStream_t stream() const { return stream_; }
  int sm_count() const { return sms_; }

  DevStatus *dstatus() { return d_status_; }
  // Clears the status block (err and result slots) on the stream.
  void reset_status();
  // Synchronises the stream and returns the host copy of the status block.
  const DevStatus &read_status();
  // Throws when the last read status carries an error bit.
  void check_status(const char *stage);

  // Zeroed look-back descriptors (n tiles) + tile counter.
  unsigned long long *lookback(uint64_t tiles, uint32_t **counter);
  // n zeroed regions of `tiles` descriptors (region k at the result +
  // k * tiles) and their n tile counters, cleared by one launch.
  unsigned long long *lookback_n(uint64_t tiles, int n, uint32_t **counters);

  // Transfers between host memory and this context's device buffers, moved
  // by kernels rather than by copy engines: a copy engine serves its
  // transfers in order, so a few bytes of offsets or status, or a grammar's
  // megabytes, would otherwise wait behind another stream's gigabyte
  // transfer (tens of ms each).  Up to kSmallCopy bytes go through
  // page-locked staging; larger ones are read from or written into
  // page-locked host memory by the kernel directly.  Larger ones with
  // pageable host memory, and bulk ones (a long one-way stream such as the
  // input steps, left to a copy engine so that it holds no SMs), use
  // cudaMemcpyAsync.  upload: src may be reused on return when it is
  // pageable.  download: dst holds the bytes after the next sync() or
  // read_status().
  static constexpr size_t kSmallCopy = 1u << 20;
  void upload(void *dst, const void *src, size_t bytes, bool bulk = false);
  void download(void *dst, const void *src, size_t bytes, bool bulk = false);
  // Zero-fills device memory with a kernel (see upload).
  void zero(void *dst, size_t bytes);
  // Waits for the stream and completes the pending downloads.
  void sync();

  // Kernel timing (CUDA events on the context stream).
  bool timing = false;
  void tbegin(const char *name, double bytes = 0);
  void tend();
  // Adds algorithmic bytes known only after a launch (e.g. output length).
  void add_bytes(const char *name, double bytes);
  std::map<std::string, KernelStat> kernel_stats();  // flushes pending events
  void clear_kernel_stats();
  uint64_t launches() const { return launches_; }
  void count_launch(uint64_t n = 1) { launches_ += n; }

  // tuning knobs
  bool warp_dedup = false;
  uint64_t first_table_cap = 0;  // pair-table slots of the first round (0 = automatic)
  uint64_t append_chunk = 0;     // steps per chunk of the chunked stack pass (0 = the automatic ladder)
  uint64_t hbm_budget = 0;       // device bytes host-input compression may use (0 = no limit)
  uint64_t encode_chunk = 0;     // steps per chunk of host-input compression (0 = from the budget)
  uint64_t decode_chunk = 0;     // expanded steps per device text pass of the full-file writer (0 = all)
  bool slot_refs = true;         // resident rounds: the count records slot references for classify / emit
  int count_kernel = -1;         // CountKernel forced by option; -1 = chosen by the tuner
  int classify_kernel = -1;      // 0 = persistent, 1 = flat; -1 = chosen by the tuner
  int front_end = 1;             // GFA parse: 1 = device front end, 0 = host parser
  int static_text = 1;           // S/L text of the full-file writer: 1 = device, 0 = host
  // P/W text for page-locked host memory: 1 (default) = the kernel writes
  // HBM and a copy engine moves it, piece by piece; 0 = the text kernel
  // writes host memory itself (its stores then starve concurrent uploads
  // of other contexts, whose read requests travel the same way)
  int host_text = 1;
  // Tuner: (kernel, stream class) -> the variant that was faster the first
  // time the class came up (see encode_traversals).  With GFAZ_TUNE_FILE
  // set, decisions are loaded from that file when the context is made and
  // appended to it when taken, so later processes (a profiler's replay of
  // the same command) run the same variants.
  // kTuneCap: the pair table's shrink factor (log2) against the size the
  // distinct-pair estimate gives, per class and round
  enum TunedKernel { kTuneCount = 0, kTuneClassify = 1, kTuneCap = 2 };
  bool table_tuner = true;  // pair-table size (hash load factor) tuned per stream class
  uint64_t tune_steps = 0;  // tuners' timing prefix (GFAZ_TUNE_STEPS); 0 = by stream length
  std::map<std::pair<int, int>, int> tuned;
  void record_tuned(int kernel, int cls, int variant);
  // Launches on this context's stream and returns their device time (ms).
  float time_launches(const std::function<void()> &launch);
  // Page-locked host buffer i (0 or 1) of at least n int32, kept for later
  // calls (chunked compression's host stream buffers); pageable memory when
  // page-locking fails.
  int32_t *host_buffer(int i, uint64_t n);
  // A stream of the lowest priority, made on first use: the P/W text that
  // gfz_decode_text writes into host memory runs there, bound by the
  // chip-to-chip link for tens of ms, so that kernels of streams of higher
  // priority (another context's compression) take SMs as its blocks retire
  // instead of waiting for the whole text kernel.
  cudaStream_t low_stream();
  // Makes `to` wait for the work queued so far on `from` (this context's
  // stream and its low-priority stream).
  void order(cudaStream_t from, cudaStream_t to);
  // Scratch of the grammar rounds kept for later calls, so that repeated
  // compressions do not return gigabytes to the pool and take them back
  // (the pool then spends milliseconds mapping memory for the next call):
  // the count's slot references and its repeated-slot bitmap.
  DevVec<uint32_t> sref_buf, rep_buf;

 private:
  int device_ = 0, sms_ = 152;
  cudaStream_t stream_ = nullptr;
  bool own_stream_ = false;
  cudaStream_t low_ = nullptr;
  cudaEvent_t order_ev_[2] = {nullptr, nullptr};
  DevStatus *d_status_ = nullptr;
  DevStatus *h_status_ = nullptr;
  // page-locked staging of upload / download: bytes [0, stage_used_) belong
  // to transfers queued since the last sync()
  char *stage_ = nullptr;
  size_t stage_cap_ = 0, stage_used_ = 0;
  struct PendingDownload {
    void *dst;
    const char *from;
    size_t bytes;
  };
  std::vector<PendingDownload> downloads_;
  char *stage(size_t bytes);
  DevVec<unsigned long long> desc_;
  struct Pending {
    std::string name;
    cudaEvent_t a, b;
    double bytes;
  };
  std::vector<Pending> pending_;
  std::vector<cudaEvent_t> event_pool_;
  std::string open_name_;
  double open_bytes_ = 0;
  cudaEvent_t open_a_ = nullptr;
  std::map<std::string, KernelStat> stats_;
  struct HostStage {
    int32_t *p = nullptr;
    uint64_t n = 0;
    bool pinned = false;
  } host_[2];
  uint64_t launches_ = 0;
  cudaEvent_t take_event();
};

// Device-resident grammar: the result of compression, or a rulebook + encoded
// streams loaded from a container for decompression.
struct Grammar {
  explicit Grammar(cudaStream_t st)
      : enc(st), off(st), rules(st), first(st), second(st), rlen(st), roff(st), rpre(st), rstat(st) {}
  DevVec<int32_t> enc;         // encoded traversals back to back
  DevVec<uint64_t> off;        // ntrav + 1 offsets into enc
  std::vector<uint64_t> h_off; // host copy of off
  uint64_t ntrav = 0;
  DevVec<long long> rules;     // packed rulebook (index = id - layer_start)
  DevVec<int32_t> first, second;  // decoded rule columns (decode side)
  DevVec<uint32_t> rlen;       // rule expansion lengths (decode side)
  DevVec<uint64_t> roff;       // rule prefix buffer: offsets (nrules + 1)
  DevVec<int32_t> rpre;        // inclusive prefix sums of every rule's expansion
  DevVec<int4> rstat;          // per-rule value ranges (text lengths)
  uint64_t nrules = 0;
  // rules made by each grammar round: round r's are [round_end[r - 1],
  // round_end[r]) and use only earlier rounds' (known for a grammar this
  // library compressed; empty for a loaded one)
  std::vector<uint64_t> round_end;
  uint32_t layer_start = 0, next_id = 0;
  int delta_round = 1;
  int rounds_done = 0;
  bool rlen_ready = false;
  int rpre_state = 0;          // 0 not built, 1 built, -1 too large (per-symbol expansion instead)
};

struct EncodeParams {
  int rounds = 8;
  int delta_round = 1;
};

// Compresses traversals steps[off[t] .. off[t+1]) (device pointer; ntrav + 1
// host offsets).  The input is not modified.
void encode_traversals(Context &ctx, const int32_t *d_steps, const std::vector<uint64_t> &h_off,
                       const EncodeParams &p, Grammar &g);

// A piece of a host-resident stream.
struct HostSeg {
  const int32_t *p;
  uint64_t n;
};
// The same compression for a stream in host memory (the segments back to
// back), moved through HBM in chunks of `chunk` steps (rounded down to whole
// apply tiles): only the pair table, per-tile words and chunk buffers live
// on the device, and the result is identical to encode_traversals'.  With
// budget > 0, the rounds continue resident once a round's stream fits the
// budget (rounds shrink the stream).
void encode_host_chunked(Context &ctx, const std::vector<HostSeg> &input, const std::vector<uint64_t> &h_off,
                         const EncodeParams &p, uint64_t chunk, uint64_t budget, Grammar &g);

// out[0 .. n] = exclusive scan of in[0 .. n) (out[n] = the total) on ctx's
// stream; the launch is timed under `timer`.
void exclusive_scan(Context &ctx, const uint32_t *in, uint64_t n, uint64_t *out, const char *timer);
void exclusive_scan(Context &ctx, const uint64_t *in, uint64_t n, uint64_t *out, const char *timer);

// Whether compression of n steps runs resident in HBM under ctx's budget
// and chunk options (working set about 16.5 bytes per step).
bool resident_fits(const Context &ctx, uint64_t n);

// Compression of host-resident input: resident in HBM when its working set
// (about 16.5 bytes per step) fits ctx.hbm_budget, else in chunks
// (encode_host_chunked) sized from the budget or ctx.encode_chunk.
void encode_host(Context &ctx, const std::vector<HostSeg> &input, const std::vector<uint64_t> &h_off,
                 const EncodeParams &p, Grammar &g);

// Splits the packed rulebook into first/second columns on the device and
// delta-codes each column (compression_utils.cpp:165-193).
void rule_columns_delta(Context &ctx, const Grammar &g, DevVec<int32_t> &first, DevVec<int32_t> &second);

// Loads decoded rule columns (host) into g.first/second.
void load_rules(Context &ctx, Grammar &g, const int32_t *first, const int32_t *second, uint64_t nrules,
                uint32_t min_id);

// Uploads encoded traversals (host data, ntrav + 1 offsets) into g.
void load_encoded(Context &ctx, Grammar &g, const int32_t *enc, const std::vector<uint64_t> &off);

// Expands traversals [t0, t1) of g (with inverse delta) into out (device),
// returning expanded offsets (host, t1 - t0 + 1 entries, relative).
void decode_traversals(Context &ctx, Grammar &g, uint64_t t0, uint64_t t1, DevVec<int32_t> &out,
                       std::vector<uint64_t> &out_off);

// Per-traversal text pieces (host) for the text kernel.
struct TextPieces {
  std::string blob;
  std::vector<uint64_t> pre_off, suf_off;  // ntrav + 1
  std::string tail;
};

// Emits P (mode 0) or W (mode 1) lines for decoded traversals x/off (device
// data, host offsets) into a device text buffer; returns the size.
uint64_t emit_text(Context &ctx, const DevVec<int32_t> &x, const std::vector<uint64_t> &off,
                   const TextPieces &pieces, int mode, DevVec<char> &text);

// Builds g's decode-side tables (rule lengths, rule prefix buffers) now
// instead of on first use.
void prepare_decode(Context &ctx, Grammar &g);

// Decode + text for traversals [t0, t1) of g.  `pieces` builds the text
// pieces from the decoded traversal offsets (t1 - t0 + 1 entries, from 0).
// direct (optional, direct_cap bytes): device memory or page-locked host
// memory the kernels write the text into, in place of `text`.
uint64_t decode_text(Context &ctx, Grammar &g, uint64_t t0, uint64_t t1,
                     const std::function<TextPieces(const std::vector<uint64_t> &)> &pieces, int mode,
                     DevVec<char> &text, char *direct = nullptr, uint64_t direct_cap = 0);

// Append encoding with a stored rulebook (one stack-encoder pass per layer).
struct Layer {
  int k;
  uint32_t start, end;
  uint64_t flat_off, count;
};
// Encodes appended traversals with a stored rulebook, layer by layer
// (add_haplotypes_workflow.cpp:336-465 with path_encoder.cpp:31-79).
// d_first/d_second: the decoded rule columns on the device.  steps: the raw
// traversals (host, offsets `off`); on return the encoded traversals back
// to back, lens[t] steps each.  max_abs: max |delta| (collision check).
void append_encode(Context &ctx, const int32_t *d_first, const int32_t *d_second, uint64_t nrules,
                   const std::vector<Layer> &layers, int delta_round, std::vector<int32_t> &steps,
                   const std::vector<uint64_t> &off, std::vector<uint64_t> &lens, uint32_t &max_abs);

}  // namespace gfz

// Resident extraction server: the rulebook, its prefix buffers and every
// encoded traversal of one container stay in HBM, and extract-path /
// extract-walk / append requests are served with continuous batching.
//
// The reference answers each extraction with a fresh full-file decode
// (src/workflows/extraction_workflow.cpp:207-357) and each append with a
// container rewrite (src/workflows/add_haplotypes_workflow.cpp:579); the
// lines returned here are byte-identical to those calls.
//
// Requests wait in one FIFO queue.  Each worker thread owns a CUDA stream;
// a free worker takes the longest run of queued extractions of one kind
// (paths or walks) whose expanded output fits the free part of the HBM
// budget and decodes them in one expansion launch, so batches of different
// workers overlap on the device and requests arriving meanwhile join the
// next batch.  An append waits until no batch is in flight, updates the
// container and the resident streams, and is seen by every later request.
#pragma once

#include <chrono>
#include <cstdlib>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../pipeline.h"
#include "model.h"
#include "workflows.h"

namespace gfz {

class Server {
 public:
  // Loads c onto `device`.  hbm_budget bounds the expanded output of the
  // batches in flight (bytes); workers = concurrent batches (streams).
  Server(int device, const Compressed &c, uint64_t hbm_budget, int workers);
  ~Server();
  Server(const Server &) = delete;
  Server &operator=(const Server &) = delete;

  // Queue a request; returns its ticket.  Unknown names fail at submission
  // with the reference's extraction messages.
  uint64_t submit_path(const std::string &name);
  uint64_t submit_walk(const WalkKey &key);
  uint64_t submit_append(const std::string &gfa_text);
  // Blocks until the request is done and returns its line (empty for an
  // append): a pointer into the server's pinned host memory, valid until
  // release(ticket), with its length in *len; latency_ms = submission to
  // completion.  A failed request rethrows its error and needs no release.
  const char *wait(uint64_t ticket, size_t *len, double *latency_ms);
  // For a finished request that is not yet released: time queued (submission
  // to the start of its batch), time in service (batch start to completion)
  // and the number of requests in its batch.
  void times(uint64_t ticket, double *queue_ms, double *service_ms, uint32_t *batch_size);
  void release(uint64_t ticket);

  struct Stats {
    uint64_t batches = 0, requests = 0, max_batch = 0, appends = 0;
    uint64_t pageable = 0;  // batches whose text went to pageable memory (pinned pool exhausted)
    // host wall time summed over batches: gather + expansion + text, text
    // download, splitting into lines
    double decode_ms = 0, copy_ms = 0, split_ms = 0;
  };
  Stats stats();

 private:
  enum Kind { kPath = 0, kWalk = 1, kAppend = 2 };
  struct Request {
    Kind kind;
    uint64_t trav = 0;       // traversal index (paths, then walks)
    std::string pre, suf;    // line pieces
    std::string append_text;
    uint64_t need = 0;       // admission bytes
    std::chrono::steady_clock::time_point t0, ts, t1;  // submitted, batch started, done
    uint32_t batch_size = 0;
    const char *result = nullptr;  // the line, inside `buf`
    size_t result_len = 0;
    int buf = -1;                  // pinned buffer holding the line
    std::string error;
    bool done = false;
  };
  // Pinned host chunks that batch text lands in.  Batches take 64-byte
  // aligned ranges of the open chunk one after another; a chunk is reused
  // once every range in it was released, so a few slow readers pin only the
  // chunks holding their own lines.
  struct Pinned {
    char *p = nullptr;
    size_t cap = 0, used = 0;  // used: bump offset while the chunk is open
    int refs = 0;              // ranges (lines, or a batch in flight) not yet released
    bool pooled = true;        // false: pageable one-off memory (pool exhausted, or larger than a chunk)
  };
  // A range of n bytes holding one reference: the buffer index and the address.
  int take_pinned(size_t n, char **dst);  // mu_ held
  void drop_pinned(int b);                // mu_ held: one reference fewer
  void add_pinned_chunk();

  void load_resident();                 // (re)build the resident grammar from c_
  void worker(int w);
  void run_batch(Context &ctx, Kind kind, const std::vector<uint64_t> &tickets);
  // An append: encoded with the stored rulebook alongside running batches,
  // then spliced into the resident stream once no batch is in flight.
  struct Prepared {
    AppendInput in;
    std::vector<int32_t> add;    // encoded appended traversals, back to back
    std::vector<uint64_t> lens;  // their encoded lengths
  };
  Prepared prepare_append(Context &ctx, uint64_t ticket);
  void check_append_names(const AppendInput &in);  // mu_ held
  void splice_append(const Prepared &p);             // mu_ held, no batch in flight
  uint64_t admission_bytes(uint64_t trav) const;

  int device_;
  uint64_t budget_;
  Compressed c_;
  std::unique_ptr<Context> setup_;      // loads the resident state
  std::unique_ptr<Grammar> g_;          // resident grammar (decode side)
  uint64_t np_ = 0, nw_ = 0;
  std::vector<uint64_t> steps_;         // decoded steps per traversal
  std::vector<Layer> layers_;
  std::unordered_map<std::string, uint64_t> path_index_;
  std::vector<std::string> overlaps_;
  std::map<std::string, uint64_t> walk_index_;  // full walk identity -> index

  static constexpr size_t kMaxBatch = 64;  // requests per expansion launch: keeps results flowing
  // pinned result chunks: a batch's admission bytes (>= its text) fit one
  static constexpr size_t kChunk = 128ull << 20;

  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::deque<uint64_t> queue_;
  std::unordered_map<uint64_t, Request> reqs_;
  uint64_t next_ticket_ = 1, in_use_ = 0;
  int in_flight_ = 0;      // extraction batches running
  int splicing_ = 0;       // appends waiting to splice: no new batch starts
  bool stop_ = false;
  Stats stats_;
  std::vector<Pinned> pinned_;
  std::vector<int> free_pinned_;  // pooled chunks holding no range
  int open_pinned_ = -1;          // the chunk ranges are taken from
  std::vector<std::thread> threads_;
};

}  // namespace gfz

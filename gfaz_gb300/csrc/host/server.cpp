// Resident extraction server (see server.h).
#include "server.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

#include "codec.h"

namespace gfz {

namespace {

constexpr const char *kExtractErr = "Extraction workflow error: ";

std::string walk_key_id(const std::string &s, uint32_t h, const std::string &q, int64_t a, int64_t b) {
  return s + '\x1f' + std::to_string(h) + '\x1f' + q + '\x1f' + std::to_string(a) + '\x1f' + std::to_string(b);
}

std::string coord(int64_t v) { return v >= 0 ? std::to_string(v) : std::string("*"); }

}  // namespace

Server::Server(int device, const Compressed &c, uint64_t hbm_budget, int workers)
    : device_(device), budget_(hbm_budget), c_(c) {
  if (workers < 1) throw std::invalid_argument("a server needs at least one worker");
  setup_ = std::make_unique<Context>(device, nullptr);
  load_resident();
  // four result chunks per worker, pinned up front (pinning is slow)
  for (int k = 0; k < 4 * workers; ++k) add_pinned_chunk();
  for (int w = 0; w < workers; ++w) threads_.emplace_back(&Server::worker, this, w);
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_work_.notify_all();
  for (auto &t : threads_) t.join();
  if (debug_enabled())
    fprintf(stderr, "[gfaz gb300] server: %llu batches, %llu requests, %llu appends, %llu pageable; host ms: decode %.1f, "
            "copy %.1f, split %.1f\n",
            (unsigned long long)stats_.batches, (unsigned long long)stats_.requests,
            (unsigned long long)stats_.appends, (unsigned long long)stats_.pageable, stats_.decode_ms, stats_.copy_ms,
            stats_.split_ms);
  for (auto &b : pinned_) {
    if (!b.p) continue;
    if (b.pooled) cudaFreeHost(b.p);
    else std::free(b.p);
  }
}

// A range of the open pinned chunk; when it is full, the next free chunk
// opens.  With no free chunk (or n above a chunk), ordinary pageable memory:
// pinning memory on the request path would stall the worker far longer than
// a pageable copy.
int Server::take_pinned(size_t n, char **dst) {
  const size_t need = (n + 63) & ~size_t(63);
  if (need <= kChunk) {
    if (open_pinned_ < 0 || pinned_[open_pinned_].cap - pinned_[open_pinned_].used < need) {
      if (!free_pinned_.empty()) {
        const int prev = open_pinned_;
        open_pinned_ = free_pinned_.back();
        free_pinned_.pop_back();
        pinned_[open_pinned_].used = 0;
        if (prev >= 0 && pinned_[prev].refs == 0) free_pinned_.push_back(prev);
      }
    }
    if (open_pinned_ >= 0 && pinned_[open_pinned_].cap - pinned_[open_pinned_].used >= need) {
      Pinned &c = pinned_[open_pinned_];
      *dst = c.p + c.used;
      c.used += need;
      c.refs++;
      return open_pinned_;
    }
  }
  stats_.pageable++;
  Pinned b;
  b.cap = std::max<size_t>(n, 1);
  b.pooled = false;
  b.refs = 1;
  b.p = static_cast<char *>(std::malloc(b.cap));
  if (!b.p) throw std::bad_alloc();
  pinned_.push_back(b);
  *dst = b.p;
  return (int)pinned_.size() - 1;
}

void Server::drop_pinned(int b) {
  Pinned &c = pinned_[b];
  if (--c.refs > 0) return;
  if (!c.pooled) {
    std::free(c.p);
    c.p = nullptr;
    c.cap = 0;
  } else if (b == open_pinned_) {
    c.used = 0;  // nothing in it is live: refill from the start
  } else {
    free_pinned_.push_back(b);
  }
}

void Server::add_pinned_chunk() {
  Pinned b;
  b.cap = kChunk;
  cuda_check(cudaMallocHost(reinterpret_cast<void **>(&b.p), b.cap), "pinned result buffer");
  pinned_.push_back(b);
  free_pinned_.push_back((int)pinned_.size() - 1);
}

void Server::load_resident() {
  auto g = std::make_unique<Grammar>(setup_->stream());
  load_traversals(*setup_, c_, *g, np_, nw_);
  prepare_decode(*setup_, *g);
  cuda_check(cudaStreamSynchronize(setup_->stream()), "stream sync");
  layers_.clear();
  for (const auto &l : c_.layers) layers_.push_back(Layer{l.k, l.start_id, l.end_id, l.flattened_offset, l.element_count});
  g_ = std::move(g);
  steps_.assign(c_.original_path_lengths.begin(), c_.original_path_lengths.end());
  steps_.insert(steps_.end(), c_.original_walk_lengths.begin(), c_.original_walk_lengths.end());
  steps_.resize(np_ + nw_, 0);

  path_index_.clear();
  const auto names = split_strings(unzstd_str(c_.names), unzstd_u32(c_.name_lengths), true, kExtractErr);
  for (uint64_t i = 0; i < names.size() && i < np_; ++i)
    if (!path_index_.emplace(names[i], i).second) path_index_[names[i]] = UINT64_MAX;  // ambiguous
  overlaps_ = split_strings(unzstd_str(c_.overlaps), unzstd_u32(c_.overlap_lengths), true, kExtractErr);

  walk_index_.clear();
  const auto samples =
      split_strings(unzstd_str(c_.walk_sample_ids), unzstd_u32(c_.walk_sample_id_lengths), true, kExtractErr);
  const auto haps = unzstd_u32(c_.walk_hap_indices);
  const auto seqids = split_strings(unzstd_str(c_.walk_seq_ids), unzstd_u32(c_.walk_seq_id_lengths), true, kExtractErr);
  const auto starts = unvarint_i64(c_.walk_seq_starts, c_.walk_lengths.size());
  const auto ends = unvarint_i64(c_.walk_seq_ends, c_.walk_lengths.size());
  for (uint64_t i = 0; i < nw_; ++i)
    if (i < samples.size() && i < haps.size() && i < seqids.size() && i < starts.size() && i < ends.size())
      walk_index_.emplace(walk_key_id(samples[i], haps[i], seqids[i], starts[i], ends[i]), i);  // first match wins
}

uint64_t Server::admission_bytes(uint64_t trav) const {
  // text (at most 10 digits, a mark and a comma per step), the per-symbol
  // decoding scratch and the line pieces
  const uint64_t symbols = g_->h_off[trav + 1] - g_->h_off[trav];
  return 12 * steps_[trav] + 48 * symbols + 4096;
}

uint64_t Server::submit_path(const std::string &name) {
  std::lock_guard<std::mutex> lk(mu_);
  const auto it = path_index_.find(name);
  if (it == path_index_.end()) throw std::runtime_error(std::string(kExtractErr) + "path not found: " + name);
  if (it->second == UINT64_MAX) throw std::runtime_error(std::string(kExtractErr) + "path name is ambiguous: " + name);
  Request r;
  r.kind = kPath;
  r.trav = it->second;
  const std::string ov = it->second < overlaps_.size() ? overlaps_[it->second] : std::string();
  r.pre = "P\t" + name + "\t";
  r.suf = "\t" + (ov.empty() ? std::string("*") : ov) + "\n";
  r.need = admission_bytes(r.trav);
  if (r.need > budget_) throw std::length_error("request exceeds the server's HBM budget");
  r.t0 = std::chrono::steady_clock::now();
  const uint64_t ticket = next_ticket_++;
  reqs_.emplace(ticket, std::move(r));
  queue_.push_back(ticket);
  cv_work_.notify_one();
  return ticket;
}

uint64_t Server::submit_walk(const WalkKey &k) {
  std::lock_guard<std::mutex> lk(mu_);
  const auto it = walk_index_.find(walk_key_id(k.sample_id, k.hap_index, k.seq_id, k.seq_start, k.seq_end));
  if (it == walk_index_.end())
    throw std::runtime_error(std::string(kExtractErr) + "walk not found for the provided identifier: " + k.sample_id +
                             "\t" + std::to_string(k.hap_index) + "\t" + k.seq_id + "\t" +
                             std::to_string(k.seq_start) + "\t" + std::to_string(k.seq_end));
  Request r;
  r.kind = kWalk;
  r.trav = np_ + it->second;
  r.pre = "W\t" + k.sample_id + "\t" + std::to_string(k.hap_index) + "\t" + k.seq_id + "\t" + coord(k.seq_start) +
          "\t" + coord(k.seq_end) + "\t";
  r.suf = "\n";
  r.need = admission_bytes(r.trav);
  if (r.need > budget_) throw std::length_error("request exceeds the server's HBM budget");
  r.t0 = std::chrono::steady_clock::now();
  const uint64_t ticket = next_ticket_++;
  reqs_.emplace(ticket, std::move(r));
  queue_.push_back(ticket);
  cv_work_.notify_one();
  return ticket;
}

uint64_t Server::submit_append(const std::string &gfa_text) {
  std::lock_guard<std::mutex> lk(mu_);
  Request r;
  r.kind = kAppend;
  r.append_text = gfa_text;
  r.t0 = std::chrono::steady_clock::now();
  const uint64_t ticket = next_ticket_++;
  reqs_.emplace(ticket, std::move(r));
  queue_.push_back(ticket);
  cv_work_.notify_one();
  return ticket;
}

const char *Server::wait(uint64_t ticket, size_t *len, double *latency_ms) {
  std::unique_lock<std::mutex> lk(mu_);
  cv_done_.wait(lk, [&] {
    const auto it = reqs_.find(ticket);
    return it == reqs_.end() || it->second.done;
  });
  const auto it = reqs_.find(ticket);
  if (it == reqs_.end()) throw std::invalid_argument("unknown request ticket");
  Request &r = it->second;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r.t1 - r.t0).count();
  if (!r.error.empty()) {
    const std::string e = r.error;
    reqs_.erase(it);
    throw std::runtime_error(e);
  }
  *len = r.result_len;
  return r.result ? r.result : "";
}

void Server::times(uint64_t ticket, double *queue_ms, double *service_ms, uint32_t *batch_size) {
  std::lock_guard<std::mutex> lk(mu_);
  const auto it = reqs_.find(ticket);
  if (it == reqs_.end() || !it->second.done) throw std::invalid_argument("unknown or unfinished request ticket");
  const Request &r = it->second;
  using ms = std::chrono::duration<double, std::milli>;
  if (queue_ms) *queue_ms = ms(r.ts - r.t0).count();
  if (service_ms) *service_ms = ms(r.t1 - r.ts).count();
  if (batch_size) *batch_size = r.batch_size;
}

void Server::release(uint64_t ticket) {
  std::lock_guard<std::mutex> lk(mu_);
  const auto it = reqs_.find(ticket);
  if (it == reqs_.end() || !it->second.done) throw std::invalid_argument("unknown or unfinished request ticket");
  const int b = it->second.buf;
  reqs_.erase(it);
  if (b >= 0) drop_pinned(b);
}

Server::Stats Server::stats() {
  std::lock_guard<std::mutex> lk(mu_);
  return stats_;
}

void Server::worker(int) {
  Context ctx(device_, nullptr);
  std::unique_lock<std::mutex> lk(mu_);
  // the queue head can start: an append at once (it is encoded alongside
  // the batches in flight), an extraction once no append is splicing and
  // its bytes fit the free budget
  auto ready = [&] {
    if (stop_) return true;
    if (queue_.empty()) return false;
    const Request &r = reqs_.at(queue_.front());
    if (r.kind == kAppend) return true;
    return splicing_ == 0 && in_use_ + r.need <= budget_;
  };
  for (;;) {
    cv_work_.wait(lk, ready);
    if (stop_) break;
    const uint64_t head = queue_.front();
    const Kind kind = reqs_.at(head).kind;
    if (kind == kAppend) {
      queue_.pop_front();
      reqs_.at(head).ts = std::chrono::steady_clock::now();
      reqs_.at(head).batch_size = 1;
      lk.unlock();
      std::string err;
      Prepared prep;
      try {
        prep = prepare_append(ctx, head);
      } catch (const std::exception &e) {
        err = e.what();
      }
      lk.lock();
      if (err.empty()) {
        ++splicing_;
        cv_work_.wait(lk, [&] { return in_flight_ == 0; });
        try {
          check_append_names(prep.in);
          splice_append(prep);
        } catch (const std::exception &e) {
          err = e.what();
        }
        --splicing_;
      }
      Request &r = reqs_.at(head);
      r.error = err;
      r.done = true;
      r.t1 = std::chrono::steady_clock::now();
      stats_.appends++;
      cv_done_.notify_all();
      cv_work_.notify_all();
      continue;
    }
    // the longest run of queued extractions of this kind that fits
    std::vector<uint64_t> batch;
    uint64_t bytes = 0;
    while (!queue_.empty()) {
      const Request &q = reqs_.at(queue_.front());
      if (q.kind != kind || in_use_ + bytes + q.need > budget_ || batch.size() == kMaxBatch) break;
      if (!batch.empty() && bytes + q.need > kChunk) break;  // the batch's text fits one pinned chunk
      bytes += q.need;
      batch.push_back(queue_.front());
      queue_.pop_front();
    }
    const auto started = std::chrono::steady_clock::now();
    for (uint64_t t : batch) {
      Request &r = reqs_.at(t);
      r.ts = started;
      r.batch_size = (uint32_t)batch.size();
    }
    in_use_ += bytes;
    ++in_flight_;
    stats_.batches++;
    stats_.requests += batch.size();
    if (batch.size() > stats_.max_batch) stats_.max_batch = batch.size();
    lk.unlock();
    std::string err;
    try {
      run_batch(ctx, kind, batch);
    } catch (const std::exception &e) {
      err = e.what();
    }
    lk.lock();
    in_use_ -= bytes;
    --in_flight_;
    const auto now = std::chrono::steady_clock::now();
    for (uint64_t t : batch) {
      Request &r = reqs_.at(t);
      if (!err.empty()) r.error = err;
      r.done = true;
      r.t1 = now;
    }
    cv_done_.notify_all();
    cv_work_.notify_all();
  }
  // stopping: fail what is still queued
  for (uint64_t t : queue_) {
    Request &r = reqs_.at(t);
    r.error = "server stopped";
    r.done = true;
  }
  queue_.clear();
  cv_done_.notify_all();
}

void Server::run_batch(Context &ctx, Kind kind, const std::vector<uint64_t> &tickets) {
  using clock = std::chrono::steady_clock;
  const auto t_start = clock::now();
  cudaStream_t st = ctx.stream();
  const Grammar &R = *g_;
  std::vector<uint64_t> trav;
  std::vector<std::string> pre, suf;
  {
    std::lock_guard<std::mutex> lk(mu_);
    for (uint64_t t : tickets) {
      const Request &r = reqs_.at(t);
      trav.push_back(r.trav);
      pre.push_back(r.pre);
      suf.push_back(r.suf);
    }
  }
  const uint64_t nb = trav.size();
  // a grammar view: the resident rules, the selected traversals gathered
  // into one encoded stream
  Grammar gb(st);
  gb.first.borrow(R.first.ptr, R.first.size);
  gb.second.borrow(R.second.ptr, R.second.size);
  gb.rlen.borrow(R.rlen.ptr, R.rlen.size);
  gb.roff.borrow(R.roff.ptr, R.roff.size);
  gb.rpre.borrow(R.rpre.ptr, R.rpre.size);
  gb.rstat.borrow(R.rstat.ptr, R.rstat.size);
  gb.nrules = R.nrules;
  gb.layer_start = R.layer_start;
  gb.next_id = R.next_id;
  gb.delta_round = R.delta_round;
  gb.rlen_ready = true;
  gb.rpre_state = R.rpre_state;
  std::vector<uint64_t> starts(nb), off(nb + 1, 0);
  for (uint64_t k = 0; k < nb; ++k) {
    starts[k] = R.h_off[trav[k]];
    off[k + 1] = off[k] + (R.h_off[trav[k] + 1] - R.h_off[trav[k]]);
  }
  gb.ntrav = nb;
  gb.h_off = off;
  gb.off.resize(nb + 1);
  gb.enc.resize(std::max<uint64_t>(off[nb], 1));
  gb.enc.size = off[nb];
  DevVec<uint64_t> d_starts(st);
  d_starts.resize(nb);
  cuda_check(cudaMemcpyAsync(gb.off.ptr, off.data(), (nb + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st),
             "batch offsets");
  cuda_check(cudaMemcpyAsync(d_starts.ptr, starts.data(), nb * sizeof(uint64_t), cudaMemcpyHostToDevice, st),
             "batch starts");
  launch_gather_ranges(R.enc.ptr, d_starts.ptr, gb.off.ptr, nb, gb.enc.ptr, st);
  DevVec<char> text(st);
  const uint64_t n = decode_text(
      ctx, gb, 0, nb, [&](const std::vector<uint64_t> &xoff) { return make_pieces(pre, suf, xoff); },
      kind == kPath ? 0 : 1, text);
  // line ends: every line is one request and ends in its only '\n'
  DevVec<unsigned long long> d_nl(st);
  d_nl.resize(nb + 1);
  cuda_check(cudaMemsetAsync(d_nl.ptr, 0, sizeof(unsigned long long), st), "line ends");
  launch_find_newlines(text.ptr, n, d_nl.ptr, nb, st);
  std::vector<unsigned long long> nl(nb + 1);
  const auto t_decoded = clock::now();
  int b;
  char *dst;
  {
    std::lock_guard<std::mutex> lk(mu_);
    b = take_pinned(n + 1, &dst);
  }
  try {
    if (n) cuda_check(cudaMemcpyAsync(dst, text.ptr, n, cudaMemcpyDeviceToHost, st), "text download");
    cuda_check(cudaMemcpyAsync(nl.data(), d_nl.ptr, (nb + 1) * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               st),
               "line ends");
    cuda_check(cudaStreamSynchronize(st), "stream sync");
    if (nl[0] != nb) throw std::runtime_error("extraction text does not hold one line per request");
  } catch (...) {
    std::lock_guard<std::mutex> lk(mu_);
    drop_pinned(b);
    throw;
  }
  const auto t_copied = clock::now();
  std::sort(nl.begin() + 1, nl.end());
  std::vector<size_t> ends(nb);
  for (uint64_t k = 0; k < nb; ++k) ends[k] = (size_t)nl[k + 1] + 1;
  const auto t_split = clock::now();
  // each line is a view into the buffer holding one reference to it (the
  // batch's own reference passes to the first)
  std::lock_guard<std::mutex> lk(mu_);
  pinned_[b].refs += (int)nb - 1;
  for (uint64_t k = 0; k < nb; ++k) {
    Request &r = reqs_.at(tickets[k]);
    const size_t begin = k ? ends[k - 1] : 0;
    r.result = dst + begin;
    r.result_len = ends[k] - begin;
    r.buf = b;
  }
  using ms = std::chrono::duration<double, std::milli>;
  stats_.decode_ms += ms(t_decoded - t_start).count();
  stats_.copy_ms += ms(t_copied - t_decoded).count();
  stats_.split_ms += ms(t_split - t_copied).count();
}

// Appends encode with the stored rulebook exactly as add_haplotypes does
// (add_haplotypes_workflow.cpp:336-465: same checks and messages) and are
// spliced into the resident stream: the rules do not change, so nothing
// else is rebuilt, and extractions of the existing traversals keep running
// while an append is encoded.  The server's container copy is not rewritten.
static const char *kAddErr = "Add-haplotypes workflow error: ";

void Server::check_append_names(const AppendInput &in) {
  if (in.has_paths) {
    std::unordered_map<std::string, int> seen;
    for (const auto &n : in.names)
      if (path_index_.count(n) || seen[n]++)
        throw std::runtime_error(std::string(kAddErr) + "path name already exists or is duplicated: " + n);
  } else {
    std::unordered_map<std::string, int> seen;
    for (uint64_t i = 0; i < in.walks.size(); ++i) {
      const std::string id = walk_key_id(in.samples[i], in.haps[i], in.seqids[i], in.starts[i], in.ends[i]);
      if (walk_index_.count(id) || seen[id]++)
        throw std::runtime_error(std::string(kAddErr) + "walk identifier already exists or is duplicated: " +
                                 in.samples[i] + "\t" + std::to_string(in.haps[i]) + "\t" + in.seqids[i] + "\t" +
                                 std::to_string(in.starts[i]) + "\t" + std::to_string(in.ends[i]));
    }
  }
}

Server::Prepared Server::prepare_append(Context &ctx, uint64_t ticket) {
  Prepared p;
  std::string text;
  {
    std::lock_guard<std::mutex> lk(mu_);
    text = reqs_.at(ticket).append_text;
  }
  p.in = parse_append_text(text);
  {
    std::lock_guard<std::mutex> lk(mu_);
    check_append_names(p.in);
  }
  const Traversals &tv = p.in.has_paths ? p.in.paths : p.in.walks;
  std::vector<int32_t> steps = tv.steps;
  uint32_t max_abs = 0;
  append_encode(ctx, g_->first.ptr, g_->second.ptr, g_->nrules, layers_, c_.delta_round, steps, tv.offsets, p.lens,
                max_abs);
  if (!c_.layers.empty() && max_abs >= c_.min_rule_id())
    throw std::runtime_error(std::string(kAddErr) + "delta-encoded appended sequence reaches ID " +
                             std::to_string(max_abs) + ", which collides with the stored rule region starting at " +
                             std::to_string(c_.min_rule_id()));
  p.add = std::move(steps);
  return p;
}

void Server::splice_append(const Prepared &p) {
  const AppendInput &in = p.in;
  const Traversals &tv = in.has_paths ? in.paths : in.walks;
  const uint64_t m = tv.size();
  // paths, [new paths], walks, [new walks]
  Grammar &g = *g_;
  cudaStream_t st = setup_->stream();
  const uint64_t P = g.h_off[np_], E = g.h_off[np_ + nw_];
  const uint64_t at = in.has_paths ? P : E;
  DevVec<int32_t> enc(st);
  enc.resize(std::max<uint64_t>(E + p.add.size(), 1));
  enc.size = E + p.add.size();
  if (at) cuda_check(cudaMemcpyAsync(enc.ptr, g.enc.ptr, at * 4, cudaMemcpyDeviceToDevice, st), "splice");
  if (!p.add.empty())
    cuda_check(cudaMemcpyAsync(enc.ptr + at, p.add.data(), p.add.size() * 4, cudaMemcpyHostToDevice, st), "splice");
  if (E > at)
    cuda_check(cudaMemcpyAsync(enc.ptr + at + p.add.size(), g.enc.ptr + at, (E - at) * 4, cudaMemcpyDeviceToDevice, st),
               "splice");
  const uint64_t pos = in.has_paths ? np_ : np_ + nw_;  // first new traversal index
  std::vector<uint64_t> h_off(g.h_off.begin(), g.h_off.begin() + (ptrdiff_t)pos + 1);
  for (uint64_t t = 0; t < m; ++t) h_off.push_back(h_off.back() + p.lens[t]);
  for (uint64_t t = pos; t < np_ + nw_; ++t) h_off.push_back(h_off.back() + (g.h_off[t + 1] - g.h_off[t]));
  DevVec<uint64_t> off(st);
  off.resize(h_off.size());
  cuda_check(cudaMemcpyAsync(off.ptr, h_off.data(), h_off.size() * 8, cudaMemcpyHostToDevice, st), "offsets");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
  g.enc = std::move(enc);
  g.off = std::move(off);
  g.h_off = std::move(h_off);
  g.ntrav += m;
  std::vector<uint64_t> orig(m);
  for (uint64_t t = 0; t < m; ++t) orig[t] = tv.offsets[t + 1] - tv.offsets[t];
  steps_.insert(steps_.begin() + (ptrdiff_t)pos, orig.begin(), orig.end());
  if (in.has_paths) {
    overlaps_.resize(np_);
    for (uint64_t t = 0; t < m; ++t) {
      path_index_.emplace(in.names[t], np_ + t);
      overlaps_.push_back(t < in.overlaps.size() ? in.overlaps[t] : std::string());
    }
    np_ += m;
  } else {
    for (uint64_t t = 0; t < m; ++t)
      walk_index_.emplace(walk_key_id(in.samples[t], in.haps[t], in.seqids[t], in.starts[t], in.ends[t]), nw_ + t);
    nw_ += m;
  }
}

}  // namespace gfz

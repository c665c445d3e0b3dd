// Pangenome growth (src/workflows/growth_workflow.cpp:261-503): haplotype
// groups from the traversal names, node coverage on the GPU from the
// decoded traversals (growth_kernels.cu), then the Panacus-style curve
// growth[k] = sum_c hist[c] * P(a node covered by c of N groups is in a
// random k-subset) on the host.
#include <algorithm>
#include <cctype>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "codec.h"
#include "workflows.h"

namespace gfz {

namespace {

// Drops a trailing ":<digits>-<digits>" (PanSN coordinates), when the colon
// is not the first byte and both numbers are present.
void strip_coords(std::string &s) {
  const size_t colon = s.rfind(':');
  if (colon == std::string::npos || colon == 0) return;
  const size_t dash = s.find('-', colon + 1);
  if (dash == std::string::npos || dash == colon + 1 || dash + 1 == s.size()) return;
  auto digits = [&](size_t a, size_t b) {
    for (size_t i = a; i < b; ++i)
      if (!std::isdigit((unsigned char)s[i])) return false;
    return true;
  };
  if (digits(colon + 1, dash) && digits(dash + 1, s.size())) s.erase(colon);
}

// A P-line name read as PanSN sample[#hap[#seq]] (the pattern
// ^([^#]+)(#[^#]+)?(#[^#].*)?$, coordinates cleared from the last field).
struct PanSN {
  std::string sample, hap, seq;
  bool has_hap = false, has_seq = false;
};

PanSN parse_pansn(const std::string &name) {
  PanSN p;
  const size_t a = name.find('#');
  if (a == std::string::npos) {
    p.sample = name;
    strip_coords(p.sample);
    return p;
  }
  p.sample = name.substr(0, a);
  auto two_fields = [&](std::string hap) {
    if (hap.empty()) return;  // "sample#": the sample alone
    p.hap = std::move(hap);
    p.has_hap = true;
    strip_coords(p.hap);
  };
  const size_t b = name.find('#', a + 1);
  if (b == std::string::npos) {
    two_fields(name.substr(a + 1));
    return p;
  }
  if (b == a + 1) return p;  // "sample##...": the sample alone
  std::string seq = name.substr(b + 1);
  if (seq.empty() || seq[0] == '#') {  // no third field: the first two
    two_fields(name.substr(a + 1, b - a - 1));
    return p;
  }
  p.hap = name.substr(a + 1, b - a - 1);
  p.has_hap = true;
  p.seq = std::move(seq);
  p.has_seq = true;
  strip_coords(p.seq);
  return p;
}

std::string path_key(const PanSN &p, GroupMode m) {
  switch (m) {
    case GroupMode::kSample: return p.sample;
    case GroupMode::kSampleHap: return p.sample + "#" + (p.has_hap ? p.hap : std::string());
    default:
      if (p.has_hap) return p.has_seq ? p.sample + "#" + p.hap + "#" + p.seq : p.sample + "#" + p.hap;
      return p.has_seq ? p.sample + "#*#" + p.seq : p.sample;
  }
}

std::string walk_key(const std::string &sample, uint32_t hap, const std::string &seq, GroupMode m) {
  switch (m) {
    case GroupMode::kSample: return sample;
    case GroupMode::kSampleHap: return sample + "#" + std::to_string(hap);
    default: return sample + "#" + std::to_string(hap) + "#" + seq;
  }
}

// Names of the slices' strings; entries past the column are empty.
std::vector<std::string> cut(const std::string &cat, const std::vector<uint32_t> &lens) {
  std::vector<std::string> out(lens.size());
  size_t o = 0;
  for (size_t i = 0; i < lens.size(); ++i) {
    if (o + lens[i] <= cat.size()) out[i] = cat.substr(o, lens[i]);
    o += lens[i];
  }
  return out;
}

}  // namespace

// Group id of every traversal (paths, then walks) in first-seen key order.
std::vector<uint32_t> growth_groups(const Compressed &c, GroupMode mode, uint32_t &ngroups) {
  const size_t np = c.sequence_lengths.size(), nw = c.walk_lengths.size();
  std::vector<uint32_t> gid(np + nw);
  if (mode == GroupMode::kPerPathWalk) {
    for (size_t i = 0; i < gid.size(); ++i) gid[i] = (uint32_t)i;
    ngroups = (uint32_t)gid.size();
    return gid;
  }
  std::vector<std::string> keys;
  keys.reserve(np + nw);
  if (np) {
    const std::vector<uint32_t> lens = unzstd_u32(c.name_lengths);
    if (lens.size() != np) throw std::runtime_error("growth: path name count does not match number of paths");
    for (const std::string &n : cut(unzstd_str(c.names), lens)) keys.push_back(path_key(parse_pansn(n), mode));
  }
  if (nw) {
    const std::vector<uint32_t> sl = unzstd_u32(c.walk_sample_id_lengths), ql = unzstd_u32(c.walk_seq_id_lengths);
    const std::vector<uint32_t> haps = unzstd_u32(c.walk_hap_indices);
    if (sl.size() != nw || ql.size() != nw || haps.size() != nw)
      throw std::runtime_error("growth: walk metadata column count does not match number of walks");
    const std::vector<std::string> s = cut(unzstd_str(c.walk_sample_ids), sl), q = cut(unzstd_str(c.walk_seq_ids), ql);
    for (size_t i = 0; i < nw; ++i) keys.push_back(walk_key(s[i], haps[i], q[i], mode));
  }
  std::unordered_map<std::string, uint32_t> seen;
  seen.reserve(keys.size() * 2);
  ngroups = 0;
  for (size_t i = 0; i < keys.size(); ++i) {
    auto it = seen.emplace(std::move(keys[i]), ngroups);
    if (it.second) ++ngroups;
    gid[i] = it.first->second;
  }
  return gid;
}

// growth[k] for k = 1 .. N (growth[0] = 0).  P(covered) = 1 - prod_{i<c}
// (N-k-i)/(N-i), 0 for c == 0, 1 when c >= N or N - c < k; the product for
// c extends the one for c - 1 by one factor, so the same products are
// formed, in the same order, as by evaluating each c from scratch.
std::vector<double> growth_curve(const std::vector<uint64_t> &hist, uint32_t N, int threads) {
  std::vector<double> growth((size_t)N + 1, 0.0);
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
  for (int64_t k = 1; k <= (int64_t)N; ++k) {
    double sum = 0.0, ratio = 1.0;
    for (uint32_t c = 1; c <= N; ++c) {
      double frac;
      if (c >= N || N - c < (uint32_t)k) {
        frac = 1.0;
      } else {
        ratio *= (double)(N - (uint32_t)k - (c - 1)) / (double)(N - (c - 1));
        frac = 1.0 - ratio;
      }
      if (hist[c]) sum += (double)hist[c] * frac;
    }
    growth[(size_t)k] = sum;
  }
  return growth;
}

GrowthResult compute_growth(Context &ctx, const Compressed &c, int threads, GroupMode mode) {
  GrowthResult r;
  const uint64_t num_nodes = unzstd_u32(c.segment_seq_lengths).size();
  r.num_nodes = (uint32_t)num_nodes;
  const uint64_t ntrav = c.sequence_lengths.size() + c.walk_lengths.size();
  if (!ntrav) return r;
  uint32_t N = 0;
  const std::vector<uint32_t> gid = growth_groups(c, mode, N);
  if (!N) return r;
  r.num_haplotypes = N;
  const int nth = resolve_threads(threads);
  set_zstd_threads(nth);

  cudaStream_t st = ctx.stream();
  Grammar g(st);
  uint64_t np = 0, nw = 0;
  load_traversals(ctx, c, g, np, nw);
  // traversal chunks of at most 2^28 decoded steps (a longer one alone)
  std::vector<uint64_t> olen(ntrav);
  for (uint64_t t = 0; t < np; ++t) olen[t] = t < c.original_path_lengths.size() ? c.original_path_lengths[t] : 0;
  for (uint64_t t = 0; t < nw; ++t)
    olen[np + t] = t < c.original_walk_lengths.size() ? c.original_walk_lengths[t] : 0;
  std::vector<uint64_t> cuts{0};
  for (uint64_t t = 0, acc = 0; t < ntrav; ++t) {
    if (acc && acc + olen[t] > (1ull << 28)) {
      cuts.push_back(t);
      acc = 0;
    }
    acc += olen[t];
  }
  cuts.push_back(ntrav);
  // bitmap rows of W words per node, built in windows of words when the
  // whole bitmap would take more than half the HBM budget
  const uint32_t W = (N + 63) / 64;
  const uint64_t row_bytes = (num_nodes + 1) * 8;
  uint32_t per_pass = W;
  if (ctx.hbm_budget && row_bytes * W > ctx.hbm_budget / 2)
    per_pass = (uint32_t)std::max<uint64_t>(1, (ctx.hbm_budget / 2) / row_bytes);
  DevVec<unsigned long long> bits(st);
  DevVec<uint32_t> cov(st), dgid(st);
  DevVec<uint64_t> doff(st);
  DevVec<unsigned long long> hist(st);
  bits.resize((num_nodes + 1) * per_pass);
  cov.resize(num_nodes + 1);
  cuda_check(cudaMemsetAsync(cov.ptr, 0, (num_nodes + 1) * 4, st), "memset");
  DevVec<int32_t> x(st);
  std::vector<uint64_t> xoff;
  for (uint32_t w0 = 0; w0 < W; w0 += per_pass) {
    const uint32_t w1 = std::min(W, w0 + per_pass);
    cuda_check(cudaMemsetAsync(bits.ptr, 0, (num_nodes + 1) * (w1 - w0) * 8, st), "memset");
    for (size_t k = 0; k + 1 < cuts.size(); ++k) {
      const uint64_t t0 = cuts[k], t1 = cuts[k + 1];
      decode_traversals(ctx, g, t0, t1, x, xoff);
      doff.resize(xoff.size());
      dgid.resize(t1 - t0);
      cuda_check(cudaMemcpyAsync(doff.ptr, xoff.data(), xoff.size() * 8, cudaMemcpyHostToDevice, st), "upload");
      cuda_check(cudaMemcpyAsync(dgid.ptr, gid.data() + t0, (t1 - t0) * 4, cudaMemcpyHostToDevice, st), "upload");
      ctx.tbegin("growth_cover", 4.0 * xoff.back());
      launch_cover_bits(x.ptr, xoff.back(), doff.ptr, t1 - t0, dgid.ptr, num_nodes, w0, w1, bits.ptr, st);
      ctx.tend();
      cuda_check(cudaStreamSynchronize(st), "stream sync");  // xoff / the chunk's buffers are reused
    }
    ctx.tbegin("growth_count", (double)(num_nodes + 1) * (8.0 * (w1 - w0) + 4));
    launch_cover_count(bits.ptr, num_nodes, w1 - w0, cov.ptr, st);
    ctx.tend();
  }
  hist.resize((uint64_t)N + 1);
  cuda_check(cudaMemsetAsync(hist.ptr, 0, ((uint64_t)N + 1) * 8, st), "memset");
  ctx.tbegin("growth_hist", 4.0 * num_nodes);
  launch_cover_hist(cov.ptr, num_nodes, N, hist.ptr, st);
  ctx.tend();
  r.hist.resize((size_t)N + 1);
  cuda_check(cudaMemcpyAsync(r.hist.data(), hist.ptr, ((uint64_t)N + 1) * 8, cudaMemcpyDeviceToHost, st), "download");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
  r.growth = growth_curve(r.hist, N, nth);
  return r;
}

}  // namespace gfz

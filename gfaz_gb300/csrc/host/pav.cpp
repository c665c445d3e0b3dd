// Presence/absence (PAV) ratios over BED ranges
// (src/workflows/pav_workflow.cpp:475-759, `gfaz pav`): for a range on a
// reference traversal, the denominator is the summed length of the unique
// nodes the range overlaps along that traversal, and a group's numerator
// the summed length of those nodes the group's traversals visit.
//
// The GPU decodes every traversal and sets, per node, one bit per group
// visiting it (growth_kernels.cu's membership rows); the reference
// traversals are decoded alone and swept against their ranges on the host.
#include <algorithm>
#include <cctype>
#include <fstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "codec.h"
#include "workflows.h"

namespace gfz {

namespace {

// Whitespace-separated fields of one BED line, read left to right the way
// formatted stream extraction reads them: a word is a run of non-blank
// bytes; a number is an optional sign and decimal digits directly at the
// cursor (a '-' wraps, as strtoull does), and whatever follows the digits is
// left for the next field.
struct BedFields {
  const std::string &s;
  size_t i = 0;
  explicit BedFields(const std::string &line) : s(line) {}
  void skip_blanks() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
  }
  bool word(std::string &out) {
    skip_blanks();
    const size_t b = i;
    while (i < s.size() && !std::isspace((unsigned char)s[i])) ++i;
    out.assign(s, b, i - b);
    return i > b;
  }
  bool number(uint64_t &out) {
    skip_blanks();
    bool neg = false;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) neg = s[i++] == '-';
    uint64_t v = 0;
    const size_t b = i;
    for (; i < s.size() && s[i] >= '0' && s[i] <= '9'; ++i) {
      const uint64_t d = (uint64_t)(s[i] - '0');
      if (v > (UINT64_MAX - d) / 10) return false;
      v = v * 10 + d;
    }
    if (i == b) return false;
    out = neg ? 0 - v : v;
    return true;
  }
};

// BED ranges (chrom start end [name]); '#' lines and empty lines are
// skipped.  The messages are the reference CLI's (pav_workflow.cpp:225-251).
std::vector<PavRange> read_bed(const std::string &path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error("pav: failed to open BED file: " + path);
  std::vector<PavRange> ranges;
  for (std::string line; std::getline(in, line);) {
    if (line.empty() || line[0] == '#') continue;
    BedFields f(line);
    PavRange r;
    if (!f.word(r.chrom) || !f.number(r.start) || !f.number(r.end))
      throw std::runtime_error("pav: malformed BED line: " + line);
    if (!f.word(r.name)) r.name = r.chrom + ":" + std::to_string(r.start) + "-" + std::to_string(r.end);
    if (r.end < r.start) throw std::runtime_error("pav: BED end before start: " + line);
    ranges.push_back(std::move(r));
  }
  if (ranges.empty()) throw std::runtime_error("pav: BED file contains no ranges");
  return ranges;
}

std::vector<std::string> strings_strict(const Block &cat, const Block &lens, const char *label) {
  const std::string s = unzstd_str(cat);
  const std::vector<uint32_t> l = unzstd_u32(lens);
  std::vector<std::string> out;
  out.reserve(l.size());
  size_t o = 0;
  for (uint32_t n : l) {
    if (o + n > s.size()) throw std::runtime_error(std::string("pav: truncated ") + label + " string column");
    out.push_back(s.substr(o, n));
    o += n;
  }
  return out;
}

// ":<digits>-<digits>" at the end of s (colon not first) is dropped.
void clear_coords(std::string &s) {
  const size_t colon = s.rfind(':');
  if (colon == std::string::npos || colon == 0) return;
  const size_t dash = s.find('-', colon + 1);
  if (dash == std::string::npos || dash == colon + 1 || dash + 1 == s.size()) return;
  for (size_t i = colon + 1; i < s.size(); ++i)
    if (i != dash && !std::isdigit((unsigned char)s[i])) return;
  s.erase(colon);
}

// The group key of a P line under PAV's reading of sample#hap#seq: the
// first two '#' split the name (later ones stay in seq), empty parts count
// as absent, coordinates are cleared from the hap (two parts) or the seq.
std::string pav_path_key(const std::string &name, GroupMode m) {
  if (m == GroupMode::kPerPathWalk) return name;
  const size_t a = name.find('#');
  std::string sample = a == std::string::npos ? name : name.substr(0, a), hap, seq;
  if (a == std::string::npos) {
    clear_coords(sample);
  } else {
    const size_t b = name.find('#', a + 1);
    if (b == std::string::npos) {
      hap = name.substr(a + 1);
      clear_coords(hap);
    } else {
      hap = name.substr(a + 1, b - a - 1);
      seq = name.substr(b + 1);
      clear_coords(seq);
    }
  }
  const bool has_hap = !hap.empty(), has_seq = !seq.empty();
  if (m == GroupMode::kSample) return sample;
  if (m == GroupMode::kSampleHap) return has_hap ? sample + "#" + hap : sample;
  if (has_hap && has_seq) return sample + "#" + hap + "#" + seq;
  return has_hap ? sample + "#" + hap : sample;
}

std::string pav_walk_key(const std::string &sample, uint32_t hap, const std::string &seq, GroupMode m) {
  if (m == GroupMode::kSample) return sample;
  if (m == GroupMode::kSampleHap) return sample + "#" + std::to_string(hap);
  return sample + "#" + std::to_string(hap) + "#" + seq;
}

}  // namespace

PavResult compute_pav(Context &ctx, const Compressed &c, const std::string &bed_path, int threads, GroupMode mode) {
  PavResult r;
  r.ranges = read_bed(bed_path);
  const std::vector<uint32_t> seg_len = unzstd_u32(c.segment_seq_lengths);
  const uint64_t num_nodes = seg_len.size();
  const int nth = resolve_threads(threads);
  set_zstd_threads(nth);

  // traversal names and groups (pav_workflow.cpp:379-443)
  const size_t np = c.sequence_lengths.size(), nw = c.walk_lengths.size(), ntrav = np + nw;
  std::vector<std::string> names;  // reference names: paths, then walks
  std::vector<std::string> keys;
  if (np) {
    names = strings_strict(c.names, c.name_lengths, "path name");
    if (names.size() != np) throw std::runtime_error("pav: path name count mismatch");
    for (const std::string &n : names) keys.push_back(pav_path_key(n, mode));
  }
  if (nw) {
    const std::vector<std::string> samples = strings_strict(c.walk_sample_ids, c.walk_sample_id_lengths, "walk sample");
    const std::vector<std::string> seqs = strings_strict(c.walk_seq_ids, c.walk_seq_id_lengths, "walk seq");
    const std::vector<uint32_t> haps = unzstd_u32(c.walk_hap_indices);
    const std::vector<int64_t> starts = unvarint_i64(c.walk_seq_starts, nw), ends = unvarint_i64(c.walk_seq_ends, nw);
    if (samples.size() != nw || seqs.size() != nw || haps.size() != nw || starts.size() != nw || ends.size() != nw)
      throw std::runtime_error("pav: walk metadata count mismatch");
    for (size_t i = 0; i < nw; ++i) {
      std::string n = samples[i] + "#" + std::to_string(haps[i]) + "#" + seqs[i];
      if (starts[i] != -1 || ends[i] != -1) n += ":" + std::to_string(starts[i]) + "-" + std::to_string(ends[i]);
      names.push_back(std::move(n));
      keys.push_back(pav_walk_key(samples[i], haps[i], seqs[i], mode));
    }
  }
  std::vector<uint32_t> gid(ntrav);
  {
    std::unordered_map<std::string, uint32_t> seen;
    for (size_t i = 0; i < ntrav; ++i) {
      auto it = seen.emplace(keys[i], (uint32_t)r.group_names.size());
      if (it.second) r.group_names.push_back(keys[i]);
      gid[i] = it.first->second;
    }
  }
  if (r.group_names.empty()) return r;
  const uint64_t G = r.group_names.size(), nr = r.ranges.size();
  r.denominators.assign(nr, 0);
  r.numerators.assign(nr * G, 0);

  // BED chroms -> reference traversals (first name wins), in BED order
  std::unordered_map<std::string, uint32_t> by_name;
  for (uint32_t t = 0; t < (uint32_t)ntrav; ++t) by_name.emplace(names[t], t);
  std::vector<std::string> chroms;
  std::unordered_map<std::string, std::vector<uint32_t>> ranges_of;
  for (uint32_t i = 0; i < (uint32_t)nr; ++i) {
    auto &v = ranges_of[r.ranges[i].chrom];
    if (v.empty()) chroms.push_back(r.ranges[i].chrom);
    v.push_back(i);
  }
  std::vector<uint32_t> ref_of(chroms.size());
  for (size_t k = 0; k < chroms.size(); ++k) {
    auto it = by_name.find(chroms[k]);
    if (it == by_name.end()) throw std::runtime_error("pav: BED reference path not found: " + chroms[k]);
    ref_of[k] = it->second;
  }

  // membership rows on the GPU: bit g of node v's row when group g visits v
  cudaStream_t st = ctx.stream();
  Grammar g(st);
  uint64_t lp = 0, lw = 0;
  load_traversals(ctx, c, g, lp, lw);
  const uint32_t W = (uint32_t)((G + 63) / 64);
  DevVec<unsigned long long> bits(st);
  DevVec<uint32_t> dgid(st);
  DevVec<uint64_t> doff(st);
  DevVec<int32_t> x(st);
  std::vector<uint64_t> xoff;
  bits.resize((num_nodes + 1) * W);
  cuda_check(cudaMemsetAsync(bits.ptr, 0, (num_nodes + 1) * W * 8, st), "memset");
  std::vector<uint64_t> olen(ntrav);
  for (size_t t = 0; t < np; ++t) olen[t] = t < c.original_path_lengths.size() ? c.original_path_lengths[t] : 0;
  for (size_t t = 0; t < nw; ++t) olen[np + t] = t < c.original_walk_lengths.size() ? c.original_walk_lengths[t] : 0;
  for (uint64_t t0 = 0; t0 < ntrav;) {
    uint64_t t1 = t0, acc = 0;
    while (t1 < ntrav && (t1 == t0 || acc + olen[t1] <= (1ull << 28))) acc += olen[t1++];
    decode_traversals(ctx, g, t0, t1, x, xoff);
    doff.resize(xoff.size());
    dgid.resize(t1 - t0);
    cuda_check(cudaMemcpyAsync(doff.ptr, xoff.data(), xoff.size() * 8, cudaMemcpyHostToDevice, st), "upload");
    cuda_check(cudaMemcpyAsync(dgid.ptr, gid.data() + t0, (t1 - t0) * 4, cudaMemcpyHostToDevice, st), "upload");
    ctx.tbegin("pav_cover", 4.0 * xoff.back());
    launch_cover_bits(x.ptr, xoff.back(), doff.ptr, t1 - t0, dgid.ptr, num_nodes, 0, W, bits.ptr, st);
    ctx.tend();
    cuda_check(cudaStreamSynchronize(st), "stream sync");
    t0 = t1;
  }
  std::vector<unsigned long long> hbits((num_nodes + 1) * W);
  cuda_check(cudaMemcpyAsync(hbits.data(), bits.ptr, hbits.size() * 8, cudaMemcpyDeviceToHost, st), "download");
  // reference traversals, decoded alone
  std::vector<std::vector<int32_t>> ref(chroms.size());
  for (size_t k = 0; k < chroms.size(); ++k) {
    decode_traversals(ctx, g, ref_of[k], ref_of[k] + 1, x, xoff);
    ref[k].resize(xoff.back());
    if (xoff.back())
      cuda_check(cudaMemcpyAsync(ref[k].data(), x.ptr, xoff.back() * 4, cudaMemcpyDeviceToHost, st), "download");
    cuda_check(cudaStreamSynchronize(st), "stream sync");
  }

  // sweep every reference traversal against its ranges (pav_workflow.cpp:676-757)
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
  for (int64_t k = 0; k < (int64_t)chroms.size(); ++k) {
    std::vector<uint32_t> ids = ranges_of[chroms[k]];
    std::sort(ids.begin(), ids.end(), [&](uint32_t a, uint32_t b) {
      return std::tie(r.ranges[a].start, r.ranges[a].end, a) < std::tie(r.ranges[b].start, r.ranges[b].end, b);
    });
    std::vector<std::pair<uint32_t, uint32_t>> hit;  // (range, node)
    size_t next = 0;
    uint64_t pos = 0;
    for (const int32_t s : ref[k]) {
      const uint32_t v = s < 0 ? 0u - (uint32_t)s : (uint32_t)s;
      if (v == 0 || v > num_nodes) continue;
      const uint64_t a = pos, b = pos + seg_len[v - 1];
      while (next < ids.size() && r.ranges[ids[next]].end <= a) ++next;
      for (size_t j = next; j < ids.size(); ++j) {
        const PavRange &q = r.ranges[ids[j]];
        if (q.start >= b) break;
        if (q.end > a && q.start < b) hit.emplace_back(ids[j], v);
      }
      pos = b;
    }
    std::sort(hit.begin(), hit.end());
    hit.erase(std::unique(hit.begin(), hit.end()), hit.end());
    for (const auto &h : hit) {
      const uint64_t len = seg_len[h.second - 1];
      r.denominators[h.first] += len;
      const unsigned long long *row = &hbits[(uint64_t)h.second * W];
      for (uint32_t w = 0; w < W; ++w)
        for (unsigned long long m = row[w]; m; m &= m - 1)
          r.numerators[(uint64_t)h.first * G + w * 64 + (uint32_t)__builtin_ctzll(m)] += len;
    }
  }
  return r;
}

}  // namespace gfz

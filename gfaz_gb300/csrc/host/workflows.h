// Host workflows of the GB300 GFAz build: the reference's public operations
// (compress, streaming decompress, in-memory decompress, extraction,
// add-haplotypes) with the traversal transform running on the GPU through
// the device pipeline.
#pragma once

#include <chrono>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../pipeline.h"
#include "model.h"

namespace gfz {

// Wall-clock phases on stderr ("[label] phase: ms") when
// GFA_COMPRESSION_DEBUG is set.
struct PhaseClock {
  explicit PhaseClock(const char *label) : label_(label) {}
  void mark(const char *what) {
    if (!on_) return;
    const auto now = std::chrono::steady_clock::now();
    std::cerr << "[" << label_ << "] " << what << ": "
              << std::chrono::duration<double, std::milli>(now - t_).count() << " ms" << std::endl;
    t_ = now;
  }

 private:
  const char *label_;
  bool on_ = debug_enabled();
  std::chrono::steady_clock::time_point t_ = std::chrono::steady_clock::now();
};

struct WalkKey {
  std::string sample_id;
  uint32_t hap_index = 0;
  std::string seq_id;
  int64_t seq_start = -1, seq_end = -1;
};

// GFA front end on the device (src/io/gfa_parser.cpp:306-590 with the P/W
// steps resolved on the GPU): the graph as parse_gfa returns it, except
// that graph.paths / graph.walks hold only their offsets; the steps stay on
// the device, paths then walks back to back (offsets: np + nw + 1 entries).
struct DeviceParse {
  explicit DeviceParse(cudaStream_t st) : steps(st) {}
  Graph graph;
  DevVec<int32_t> steps;
  std::vector<uint64_t> offsets;
};
DeviceParse parse_gfa_device(Context &ctx, const std::string &path, int threads);
// Copies the parsed steps into graph.paths.steps / graph.walks.steps.
void download_steps(Context &ctx, const DeviceParse &r, Graph &g);
// Whether the device front end fits ctx's HBM budget for a file this size.
bool device_front_end_fits(const Context &ctx, uint64_t file_bytes);
// The parsed graph: the device front end when ctx.front_end is set and it
// fits the budget, else the host parser.
Graph parse_graph(Context &ctx, const std::string &gfa_path, int threads);

// src/workflows/compression_workflow.cpp:706 compress_gfa
Compressed compress_gfa(Context &ctx, const std::string &gfa_path, int rounds, uint64_t threshold, int delta_round,
                        int threads, bool show_stats);
// Same, from an already parsed graph (the graph's traversals are left as
// is).  d_steps (optional): the traversals' steps on the device, paths then
// walks back to back, used in place of g's host steps.
Compressed compress_graph(Context &ctx, const Graph &g, int rounds, uint64_t threshold, int delta_round,
                          int threads, bool show_stats, const int32_t *d_steps = nullptr);

// Growable text in malloc'd memory that is never zero-filled: the
// full-file text is written into it and handed to C callers as is
// (released with free).
class RawText {
 public:
  RawText() = default;
  RawText(const RawText &) = delete;
  RawText &operator=(const RawText &) = delete;
  ~RawText() { std::free(p_); }
  // k more bytes at the end, uninitialized; returns where they start.
  char *grow(size_t k);
  void append(const char *s, size_t k) { if (k) std::memcpy(grow(k), s, k); }
  void append(const std::string &s) { append(s.data(), s.size()); }
  const char *data() const { return p_; }
  size_t size() const { return n_; }
  // The buffer (NUL-terminated) and its ownership.
  char *release();

 private:
  char *p_ = nullptr;
  size_t n_ = 0, cap_ = 0;
};
// The whole decompressed GFA (the bytes write_gfa writes) into out.
void gfa_text_into(Context &ctx, const Compressed &c, int threads, RawText &out);

// src/io/gfa_writer.cpp:376 write_gfa_from_compressed_data (H,S,L,J,C,P,W)
void write_gfa(Context &ctx, const Compressed &c, const std::string &out_path, int threads);
// Whole GFA text in memory (same bytes as write_gfa).
std::string gfa_text(Context &ctx, const Compressed &c, int threads);

// src/workflows/decompression_workflow.cpp:255 decompress_gfa
Graph decompress_graph(Context &ctx, const Compressed &c, int threads);

// src/workflows/extraction_workflow.cpp:207-357
std::vector<std::string> extract_path_lines(Context &ctx, const Compressed &c, const std::vector<std::string> &names,
                                            int threads);
std::vector<std::string> extract_walk_lines(Context &ctx, const Compressed &c, const std::vector<WalkKey> &keys,
                                            int threads);
std::vector<std::string> extract_walk_lines_by_name(Context &ctx, const Compressed &c,
                                                    const std::vector<std::string> &names, int threads);

// Pangenome growth, include/workflows/growth_workflow.hpp:21-41: how P/W
// lines map to haplotypes (each line; PanSN sample#hap#seq with ":start-end"
// cleared; sample#hap; sample), the coverage histogram hist[c] (nodes
// covered by exactly c of the N groups, c = 0 .. N) and growth[k] (expected
// nodes covered by a random k-subset, k = 1 .. N; growth[0] unused).
enum class GroupMode { kPerPathWalk = 0, kSampleHapSeq = 1, kSampleHap = 2, kSample = 3 };
struct GrowthResult {
  uint32_t num_haplotypes = 0, num_nodes = 0;
  std::vector<uint64_t> hist;
  std::vector<double> growth;
};
// src/workflows/growth_workflow.cpp:261 compute_growth (coverage on the GPU)
GrowthResult compute_growth(Context &ctx, const Compressed &c, int threads, GroupMode mode);
// The group of every traversal (paths, then walks), first-seen order.
std::vector<uint32_t> growth_groups(const Compressed &c, GroupMode mode, uint32_t &ngroups);
// growth[k] from the coverage histogram (growth_workflow.cpp:106-118, 480-500).
std::vector<double> growth_curve(const std::vector<uint64_t> &hist, uint32_t N, int threads);

// Presence/absence ratios, include/workflows/pav_workflow.hpp:14-37: BED
// ranges on reference traversals (P names, or W "sample#hap#seq[:start-end]");
// numerators[range * groups + group] and denominators[range] in bases.
// Grouping: kPerPathWalk (each name), kSample, kSampleHap (PAV's own
// reading of PanSN names, pav_workflow.cpp:295-368).
struct PavRange {
  std::string chrom;
  uint64_t start = 0, end = 0;
  std::string name;
};
struct PavResult {
  std::vector<PavRange> ranges;
  std::vector<std::string> group_names;
  std::vector<uint64_t> denominators, numerators;
};
// src/workflows/pav_workflow.cpp:475 compute_pav (traversals decoded and
// node membership built on the GPU)
PavResult compute_pav(Context &ctx, const Compressed &c, const std::string &bed_path, int threads, GroupMode mode);

// src/workflows/add_haplotypes_workflow.cpp:579 add_haplotypes
void add_haplotypes(Context &ctx, Compressed &c, const std::string &path, int threads);
// Parsed add-haplotypes input: P-lines or W-lines (never both), with the
// checks of add_haplotypes_workflow.cpp's parser.
struct AppendInput {
  Traversals paths, walks;
  std::vector<std::string> names, overlaps, samples, seqids;
  std::vector<uint32_t> haps;
  std::vector<int64_t> starts, ends;
  bool has_paths = false, has_walks = false;
};
AppendInput parse_append_text(const std::string &gfa_text);

// The same with the appended P or W lines given as GFA text.
void add_haplotypes_text(Context &ctx, Compressed &c, const std::string &gfa_text, int threads);

// Rules and every encoded traversal of c (paths, then walks) into g.
void load_traversals(Context &ctx, const Compressed &c, Grammar &g, uint64_t &np, uint64_t &nw);

// Text pieces of traversal lines: prefix pre[t] before the steps of t and
// suffix suf[t] after them (empty traversals folded in; see TextPieces).
TextPieces make_pieces(const std::vector<std::string> &pre, const std::vector<std::string> &suf,
                       const std::vector<uint64_t> &off);

// Decoded rule columns (zstd + delta decode on the device) and text pieces.
void decode_rule_columns(Context &ctx, const Compressed &c, Grammar &g);
// Traversal t of `off` takes its fields from entry base + t of the columns.
TextPieces path_pieces(const std::vector<std::string> &names, const std::vector<std::string> &overlaps,
                       const std::vector<uint64_t> &off, size_t base = 0);
TextPieces walk_pieces(const std::vector<std::string> &samples, const std::vector<uint32_t> &haps,
                       const std::vector<std::string> &seqids, const std::vector<int64_t> &starts,
                       const std::vector<int64_t> &ends, const std::vector<uint64_t> &off, size_t base = 0);

}  // namespace gfz

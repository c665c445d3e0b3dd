// C ABI of libgfaz_gb300.so (declarations and reference mapping in
// include/gfaz_gb300.h).  Every entry point converts exceptions into a status
// code plus a thread-local message.
#include "../../include/gfaz_gb300.h"

#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>

#include "host/model.h"
#include "host/server.h"
#include "host/workflows.h"
#include "noalloc.h"
#include "pipeline.h"

struct gfz_context {
  explicit gfz_context(int dev, cudaStream_t st) : ctx(dev, st) {}
  gfz::Context ctx;
};
struct gfz_compressed {
  gfz::Compressed c;
};
struct gfz_grammar {
  explicit gfz_grammar(cudaStream_t st) : g(st), text(st) {}
  gfz::Grammar g;
  gfz::DevVec<char> text;
  bool text_external = false;  // the last decode_text wrote to the caller's buffer
  uint64_t text_size = 0;
};
struct gfz_graph {
  gfz::Graph g;
};

namespace {

thread_local std::string g_err;

gfz_status classify(const std::string &m) {
  if (m.find("not found") != std::string::npos) return GFZ_ERR_NOT_FOUND;
  if (m.find("failed to open") != std::string::npos || m.find("failed to write") != std::string::npos ||
      m.find("failed to read") != std::string::npos || m.find("failed to stat") != std::string::npos)
    return GFZ_ERR_IO;
  if (m.find("device error") != std::string::npos) return GFZ_ERR_DEVICE;
  return GFZ_ERR_FORMAT;
}

template <typename F>
gfz_status guard(F &&f) {
  try {
    f();
    g_err.clear();
    return GFZ_OK;
  } catch (const gfz::CudaError &e) {
    g_err = e.what();
    return GFZ_ERR_CUDA;
  } catch (const std::invalid_argument &e) {
    g_err = e.what();
    return GFZ_ERR_INVALID;
  } catch (const std::length_error &e) {
    g_err = e.what();
    return GFZ_ERR_BUFFER;
  } catch (const std::bad_alloc &) {
    g_err = "out of host memory";
    return GFZ_ERR_INTERNAL;
  } catch (const std::exception &e) {
    g_err = e.what();
    return classify(g_err);
  } catch (...) {
    g_err = "unknown error";
    return GFZ_ERR_INTERNAL;
  }
}

std::mutex g_default_mu;
std::unique_ptr<gfz_context> g_default;

gfz::Context &ctx_of(gfz_context *c) {
  if (c) return c->ctx;
  std::lock_guard<std::mutex> lk(g_default_mu);
  if (!g_default) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0)
      throw gfz::CudaError("no usable CUDA device: the GFAz transform runs on the GPU only");
    int dev = 0;
    if (const char *e = std::getenv("GFZ_DEVICE")) dev = std::atoi(e);
    g_default.reset(new gfz_context(dev, nullptr));
  }
  return g_default->ctx;
}

void require(bool ok, const char *what) {
  if (!ok) throw std::invalid_argument(what);
}

char *dup_bytes(const void *p, size_t n) {
  char *o = static_cast<char *>(std::malloc(n + 1));
  if (!o) throw std::bad_alloc();
  if (n) std::memcpy(o, p, n);
  o[n] = '\0';
  return o;
}

std::string join_lines(const std::vector<std::string> &v) {
  std::string s;
  for (const auto &x : v) s += x;
  return s;
}

const gfz::Block &block_by_name(const gfz::Compressed &c, const std::string &f) {
#define GFZ_B(name) \
  if (f == #name) return c.name;
  GFZ_B(rules_first) GFZ_B(rules_second) GFZ_B(paths) GFZ_B(names) GFZ_B(name_lengths) GFZ_B(overlaps)
  GFZ_B(overlap_lengths) GFZ_B(segment_sequences) GFZ_B(segment_seq_lengths) GFZ_B(link_from_ids)
  GFZ_B(link_to_ids) GFZ_B(link_from_orients) GFZ_B(link_to_orients) GFZ_B(link_overlap_nums)
  GFZ_B(link_overlap_ops) GFZ_B(walks) GFZ_B(walk_sample_ids) GFZ_B(walk_sample_id_lengths)
  GFZ_B(walk_hap_indices) GFZ_B(walk_seq_ids) GFZ_B(walk_seq_id_lengths) GFZ_B(walk_seq_starts)
  GFZ_B(walk_seq_ends) GFZ_B(jump_from_ids) GFZ_B(jump_to_ids) GFZ_B(jump_distances) GFZ_B(jump_rest_fields)
  GFZ_B(containment_container_ids) GFZ_B(containment_positions) GFZ_B(containment_overlaps)
#undef GFZ_B
  throw std::invalid_argument("unknown block field: " + f);
}

gfz::TextPieces pieces_from_meta(const gfz_line_meta *m, const std::vector<uint64_t> &off) {
  const size_t n = off.size() - 1;
  auto str = [](const char *const *a, size_t i) { return (a && a[i]) ? std::string(a[i]) : std::string(); };
  if (m->mode == GFZ_P_LINES) {
    std::vector<std::string> names(n), ovs(n);
    for (size_t i = 0; i < n; ++i) {
      names[i] = str(m->names, i);
      ovs[i] = str(m->overlaps, i);
    }
    return gfz::path_pieces(names, ovs, off);
  }
  std::vector<std::string> s(n), q(n);
  std::vector<uint32_t> h(n, 0);
  std::vector<int64_t> a(n, -1), b(n, -1);
  for (size_t i = 0; i < n; ++i) {
    s[i] = str(m->names, i);
    q[i] = str(m->seq_ids, i);
    if (m->hap_indices) h[i] = m->hap_indices[i];
    if (m->seq_starts) a[i] = m->seq_starts[i];
    if (m->seq_ends) b[i] = m->seq_ends[i];
  }
  return gfz::walk_pieces(s, h, q, a, b, off);
}

// Device bytes to the caller's buffer (complete after ctx.sync()).
void copy_out(gfz::Context &ctx, void *dst, const void *src_dev, size_t bytes, int where) {
  if (!bytes) return;
  if (where == GFZ_WHERE_DEVICE) {
    gfz::launch_copy_bytes(src_dev, dst, bytes, ctx.stream());
    ctx.count_launch();
  } else {
    ctx.download(dst, src_dev, bytes);
  }
}

}  // namespace

extern "C" {

const char *gfz_last_error(void) { return g_err.c_str(); }
const char *gfz_version(void) { return "gfaz_gb300 0.1 (sm_103a)"; }
void gfz_free(void *p) { std::free(p); }

int gfz_has_gpu(void) {
  int n = 0;
  return cudaGetDeviceCount(&n) == cudaSuccess && n > 0 ? 1 : 0;
}

unsigned gfz_zstd_version(void) {
  std::string why;
  return gfz::zstd_available(&why) ? gfz::zstd_version() : 0u;
}

gfz_status gfz_context_create(int device, void *cuda_stream, gfz_context **out) {
  return guard([&] {
    require(out, "out is NULL");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0)
      throw gfz::CudaError("no usable CUDA device: the GFAz transform runs on the GPU only");
    *out = new gfz_context(device, static_cast<cudaStream_t>(cuda_stream));
  });
}

void gfz_context_destroy(gfz_context *ctx) { delete ctx; }

gfz_status gfz_context_set_timing(gfz_context *ctx, int enabled) {
  return guard([&] { ctx_of(ctx).timing = enabled != 0; });
}

gfz_status gfz_context_kernel_stats(gfz_context *ctx, int reset, char **json, size_t *len) {
  return guard([&] {
    require(json && len, "json/len are NULL");
    gfz::Context &c = ctx_of(ctx);
    auto stats = c.kernel_stats();
    std::ostringstream o;
    o.precision(9);
    o << "{";
    for (const auto &kv : stats)
      o << "\"" << kv.first << "\": {\"ms\": " << kv.second.ms << ", \"launches\": " << kv.second.launches
        << ", \"bytes\": " << kv.second.bytes << "}, ";
    o << "\"_launches\": " << c.launches() << "}";
    const std::string s = o.str();
    *json = dup_bytes(s.data(), s.size());
    *len = s.size();
    if (reset) c.clear_kernel_stats();
  });
}

gfz_status gfz_context_set_option(gfz_context *ctx, const char *name, int64_t value) {
  return guard([&] {
    require(name, "name is NULL");
    gfz::Context &c = ctx_of(ctx);
    if (std::string(name) == "warp_dedup") c.warp_dedup = value != 0;
    else if (std::string(name) == "first_table_cap") {
      require(value >= 0 && (value & (value - 1)) == 0, "first_table_cap must be 0 or a power of two");
      c.first_table_cap = (uint64_t)value;
    } else if (std::string(name) == "count_kernel") {
      require(value >= -1 && value <= 3,
              "count_kernel must be -1 (tuned), 0 (tiled), 1 (tiled + warp folding), 2 (flat) or 3 (flat, 4 pairs)");
      c.count_kernel = (int)value;
    } else if (std::string(name) == "classify_kernel") {
      require(value >= -1 && value <= 1, "classify_kernel must be -1 (tuned), 0 (persistent) or 1 (flat)");
      c.classify_kernel = (int)value;
    } else if (std::string(name) == "hbm_budget") {
      require(value >= 0, "hbm_budget must be >= 0");
      c.hbm_budget = (uint64_t)value;
    } else if (std::string(name) == "encode_chunk") {
      require(value >= 0, "encode_chunk must be >= 0");
      c.encode_chunk = (uint64_t)value;
    } else if (std::string(name) == "decode_chunk") {
      require(value >= 0, "decode_chunk must be >= 0");
      c.decode_chunk = (uint64_t)value;
    } else if (std::string(name) == "slot_refs") {
      require(value == 0 || value == 1, "slot_refs must be 0 or 1");
      c.slot_refs = value != 0;
    } else if (std::string(name) == "front_end") {
      require(value == 0 || value == 1, "front_end must be 0 (host parser) or 1 (device)");
      c.front_end = (int)value;
    } else if (std::string(name) == "table_tuner") {
      require(value == 0 || value == 1, "table_tuner must be 0 or 1");
      c.table_tuner = value != 0;
    } else if (std::string(name) == "host_text") {
      require(value == 0 || value == 1, "host_text must be 0 (written by the kernel) or 1 (staged in HBM)");
      c.host_text = (int)value;
    } else if (std::string(name) == "static_text") {
      require(value == 0 || value == 1, "static_text must be 0 (host) or 1 (device)");
      c.static_text = (int)value;
    } else if (std::string(name) == "append_chunk") {
      require(value >= 0, "append_chunk must be >= 0");
      c.append_chunk = (uint64_t)value;
    } else throw std::invalid_argument(std::string("unknown option: ") + name);
  });
}

gfz_status gfz_compress_file(gfz_context *ctx, const char *gfa_path, int rounds, uint64_t threshold, int delta_round,
                             int threads, int show_stats, gfz_compressed **out) {
  return guard([&] {
    require(gfa_path && out, "gfa_path/out are NULL");
    gfz::Context &c = ctx_of(ctx);
    auto *r = new gfz_compressed();
    try {
      r->c = gfz::compress_gfa(c, gfa_path, rounds, threshold, delta_round, threads, show_stats != 0);
    } catch (...) {
      delete r;
      throw;
    }
    *out = r;
  });
}

gfz_status gfz_serialize(const gfz_compressed *c, const char *path) {
  return guard([&] {
    require(c && path, "container/path are NULL");
    gfz::serialize(c->c, path);
  });
}

gfz_status gfz_serialize_buffer(const gfz_compressed *c, void **out, size_t *len) {
  return guard([&] {
    require(c && out && len, "NULL argument");
    const std::vector<uint8_t> b = gfz::serialize_bytes(c->c);
    *out = dup_bytes(b.data(), b.size());
    *len = b.size();
  });
}

gfz_status gfz_deserialize(const char *path, gfz_compressed **out) {
  return guard([&] {
    require(path && out, "path/out are NULL");
    auto *r = new gfz_compressed();
    try {
      r->c = gfz::deserialize(path);
    } catch (...) {
      delete r;
      throw;
    }
    *out = r;
  });
}

gfz_status gfz_deserialize_buffer(const void *data, size_t len, gfz_compressed **out) {
  return guard([&] {
    require(out && (data || !len), "NULL argument");
    auto *r = new gfz_compressed();
    try {
      r->c = gfz::deserialize_bytes(static_cast<const uint8_t *>(data), len);
    } catch (...) {
      delete r;
      throw;
    }
    *out = r;
  });
}

void gfz_compressed_free(gfz_compressed *c) { delete c; }

gfz_status gfz_write_gfa(gfz_context *ctx, const gfz_compressed *c, const char *out_path, int threads) {
  return guard([&] {
    require(c && out_path, "container/path are NULL");
    gfz::write_gfa(ctx_of(ctx), c->c, out_path, threads);
  });
}

gfz_status gfz_gfa_text(gfz_context *ctx, const gfz_compressed *c, int threads, char **out, size_t *len) {
  return guard([&] {
    require(c && out && len, "NULL argument");
    gfz::RawText t;
    gfz::gfa_text_into(ctx_of(ctx), c->c, threads, t);
    *len = t.size();
    *out = t.release();
  });
}

gfz_status gfz_extract_path_lines(gfz_context *ctx, const gfz_compressed *c, const char *const *names, size_t n,
                                  int threads, char **out, size_t *len) {
  return guard([&] {
    require(c && out && len && (names || !n), "NULL argument");
    std::vector<std::string> v;
    for (size_t i = 0; i < n; ++i) v.emplace_back(names[i] ? names[i] : "");
    const std::string s = join_lines(gfz::extract_path_lines(ctx_of(ctx), c->c, v, threads));
    *out = dup_bytes(s.data(), s.size());
    *len = s.size();
  });
}

gfz_status gfz_extract_walk_lines(gfz_context *ctx, const gfz_compressed *c, const gfz_walk_key *keys, size_t n,
                                  int threads, char **out, size_t *len) {
  return guard([&] {
    require(c && out && len && (keys || !n), "NULL argument");
    std::vector<gfz::WalkKey> v;
    for (size_t i = 0; i < n; ++i) {
      gfz::WalkKey k;
      k.sample_id = keys[i].sample_id ? keys[i].sample_id : "";
      k.hap_index = keys[i].hap_index;
      k.seq_id = keys[i].seq_id ? keys[i].seq_id : "";
      k.seq_start = keys[i].seq_start;
      k.seq_end = keys[i].seq_end;
      v.push_back(k);
    }
    const std::string s = join_lines(gfz::extract_walk_lines(ctx_of(ctx), c->c, v, threads));
    *out = dup_bytes(s.data(), s.size());
    *len = s.size();
  });
}

gfz_status gfz_extract_walk_lines_by_name(gfz_context *ctx, const gfz_compressed *c, const char *const *names,
                                          size_t n, int threads, char **out, size_t *len) {
  return guard([&] {
    require(c && out && len && (names || !n), "NULL argument");
    std::vector<std::string> v;
    for (size_t i = 0; i < n; ++i) v.emplace_back(names[i] ? names[i] : "");
    const std::string s = join_lines(gfz::extract_walk_lines_by_name(ctx_of(ctx), c->c, v, threads));
    *out = dup_bytes(s.data(), s.size());
    *len = s.size();
  });
}

gfz_status gfz_add_haplotypes(gfz_context *ctx, gfz_compressed *c, const char *path, int threads) {
  return guard([&] {
    require(c && path, "container/path are NULL");
    // all-or-nothing: work on a copy
    gfz::Compressed work = c->c;
    gfz::add_haplotypes(ctx_of(ctx), work, path, threads);
    c->c = std::move(work);
  });
}

gfz_status gfz_parse_gfa(gfz_context *ctx, const char *path, int threads, int device, gfz_graph **out) {
  return guard([&] {
    require(path && out, "path/out are NULL");
    auto *g = new gfz_graph();
    try {
      if (device) {
        gfz::Context &c = ctx_of(ctx);
        gfz::DeviceParse r = gfz::parse_gfa_device(c, path, threads);
        gfz::download_steps(c, r, r.graph);
        g->g = std::move(r.graph);
      } else {
        g->g = gfz::parse_gfa(path, threads);
      }
    } catch (...) {
      delete g;
      throw;
    }
    *out = g;
  });
}

gfz_status gfz_growth(gfz_context *ctx, const gfz_compressed *c, int threads, int group_by, uint32_t *num_haplotypes,
                      uint32_t *num_nodes, uint64_t **hist, double **growth) {
  return guard([&] {
    require(c && num_haplotypes && num_nodes && hist && growth, "NULL argument");
    require(group_by >= 0 && group_by <= 3, "group_by must be 0 (path), 1 (sample-hap-seq), 2 (sample-hap) or 3 (sample)");
    const gfz::GrowthResult r = gfz::compute_growth(ctx_of(ctx), c->c, threads, (gfz::GroupMode)group_by);
    *num_haplotypes = r.num_haplotypes;
    *num_nodes = r.num_nodes;
    *hist = nullptr;
    *growth = nullptr;
    if (r.num_haplotypes) {
      std::unique_ptr<char, decltype(&std::free)> hb(dup_bytes(r.hist.data(), r.hist.size() * 8), &std::free);
      *growth = reinterpret_cast<double *>(dup_bytes(r.growth.data(), r.growth.size() * 8));
      *hist = reinterpret_cast<uint64_t *>(hb.release());
    }
  });
}

gfz_status gfz_pav(gfz_context *ctx, const gfz_compressed *c, const char *bed_path, int threads, int group_by,
                   char **ranges, size_t *ranges_len, char **groups, size_t *groups_len, uint64_t *nranges,
                   uint64_t *ngroups, uint64_t **denominators, uint64_t **numerators) {
  return guard([&] {
    require(c && bed_path && ranges && ranges_len && groups && groups_len && nranges && ngroups && denominators &&
                numerators,
            "NULL argument");
    require(group_by == 0 || group_by == 2 || group_by == 3, "group_by must be 0 (per traversal), 2 (sample#hap) or 3 (sample)");
    const gfz::PavResult r = gfz::compute_pav(ctx_of(ctx), c->c, bed_path, threads, (gfz::GroupMode)group_by);
    std::string rs, gs;
    for (const auto &q : r.ranges)
      rs += q.chrom + "\t" + std::to_string(q.start) + "\t" + std::to_string(q.end) + "\t" + q.name + "\n";
    for (const auto &n : r.group_names) gs += n + "\n";
    // every buffer first, so that a failed allocation leaves no output set
    std::unique_ptr<char, decltype(&std::free)> rb(dup_bytes(rs.data(), rs.size()), &std::free);
    std::unique_ptr<char, decltype(&std::free)> gb(dup_bytes(gs.data(), gs.size()), &std::free);
    std::unique_ptr<char, decltype(&std::free)> db(dup_bytes(r.denominators.data(), r.denominators.size() * 8),
                                                   &std::free);
    char *nb = dup_bytes(r.numerators.data(), r.numerators.size() * 8);
    *ranges = rb.release();
    *ranges_len = rs.size();
    *groups = gb.release();
    *groups_len = gs.size();
    *nranges = r.ranges.size();
    *ngroups = r.group_names.size();
    *denominators = reinterpret_cast<uint64_t *>(db.release());
    *numerators = reinterpret_cast<uint64_t *>(nb);
  });
}

gfz_status gfz_decompress_graph(gfz_context *ctx, const gfz_compressed *c, int threads, gfz_graph **out) {
  return guard([&] {
    require(c && out, "NULL argument");
    auto *g = new gfz_graph();
    try {
      g->g = gfz::decompress_graph(ctx_of(ctx), c->c, threads);
    } catch (...) {
      delete g;
      throw;
    }
    *out = g;
  });
}

void gfz_graph_free(gfz_graph *g) { delete g; }

gfz_status gfz_compressed_info(const gfz_compressed *c, gfz_container_info *info) {
  return guard([&] {
    require(c && info, "NULL argument");
    std::memset(info, 0, sizeof(*info));
    info->num_paths = c->c.sequence_lengths.size();
    info->num_walks = c->c.walk_lengths.size();
    info->num_links = c->c.num_links;
    info->num_jumps = c->c.num_jumps;
    info->num_containments = c->c.num_containments;
    info->num_layers = c->c.layers.size();
    info->total_rules = c->c.total_rules();
    info->min_rule_id = c->c.min_rule_id();
    info->delta_round = c->c.delta_round;
  });
}

gfz_status gfz_compressed_layers(const gfz_compressed *c, int64_t *rows, size_t max_rows) {
  return guard([&] {
    require(c && (rows || !max_rows), "NULL argument");
    for (size_t i = 0; i < c->c.layers.size() && i < max_rows; ++i) {
      const auto &l = c->c.layers[i];
      rows[5 * i] = l.k;
      rows[5 * i + 1] = l.start_id;
      rows[5 * i + 2] = l.end_id;
      rows[5 * i + 3] = (int64_t)l.flattened_offset;
      rows[5 * i + 4] = (int64_t)l.element_count;
    }
  });
}

gfz_status gfz_compressed_u32(const gfz_compressed *c, const char *field, const uint32_t **data, size_t *n) {
  return guard([&] {
    require(c && field && data && n, "NULL argument");
    const std::string f(field);
    const std::vector<uint32_t> *v = nullptr;
    if (f == "sequence_lengths") v = &c->c.sequence_lengths;
    else if (f == "original_path_lengths") v = &c->c.original_path_lengths;
    else if (f == "walk_lengths") v = &c->c.walk_lengths;
    else if (f == "original_walk_lengths") v = &c->c.original_walk_lengths;
    else throw std::invalid_argument("unknown u32 field: " + f);
    *data = v->data();
    *n = v->size();
  });
}

gfz_status gfz_compressed_block(const gfz_compressed *c, const char *field, void **out, size_t *len) {
  return guard([&] {
    require(c && field && out && len, "NULL argument");
    const std::vector<uint8_t> b = gfz::unzstd(block_by_name(c->c, field));
    *out = dup_bytes(b.data(), b.size());
    *len = b.size();
  });
}

gfz_status gfz_graph_traversals(const gfz_graph *g, int kind, const int32_t **steps, const uint64_t **offsets,
                                uint64_t *ntrav) {
  return guard([&] {
    require(g && steps && offsets && ntrav, "NULL argument");
    const gfz::Traversals &t = kind == 0 ? g->g.paths : g->g.walks;
    *steps = t.steps.data();
    *offsets = t.offsets.data();
    *ntrav = t.size();
  });
}

gfz_status gfz_graph_strings(const gfz_graph *g, const char *field, char **out, size_t *len) {
  return guard([&] {
    require(g && field && out && len, "NULL argument");
    const std::string f(field);
    std::string s;
    const std::vector<std::string> *v = nullptr;
    if (f == "path_names") v = &g->g.path_names;
    else if (f == "path_overlaps") v = &g->g.path_overlaps;
    else if (f == "walk_sample_ids") v = &g->g.walk_sample_ids;
    else if (f == "walk_seq_ids") v = &g->g.walk_seq_ids;
    else if (f == "segment_names") v = &g->g.node_names;
    else if (f == "segment_sequences") v = &g->g.node_sequences;
    else if (f == "header") s = g->g.header_line;
    else throw std::invalid_argument("unknown string field: " + f);
    // segment columns: index 0 is the 1-based ids' placeholder
    const size_t first = f.rfind("segment_", 0) == 0 ? 1 : 0;
    if (v)
      for (size_t i = first; i < v->size(); ++i) s += (*v)[i] + "\n";
    *out = dup_bytes(s.data(), s.size());
    *len = s.size();
  });
}

gfz_status gfz_graph_walk_numbers(const gfz_graph *g, const uint32_t **haps, const int64_t **starts,
                                  const int64_t **ends, uint64_t *n) {
  return guard([&] {
    require(g && haps && starts && ends && n, "NULL argument");
    *haps = g->g.walk_hap_indices.data();
    *starts = g->g.walk_seq_starts.data();
    *ends = g->g.walk_seq_ends.data();
    *n = g->g.walk_hap_indices.size();
  });
}

gfz_status gfz_graph_counts(const gfz_graph *g, uint64_t *segments, uint64_t *links, uint64_t *jumps,
                            uint64_t *containments) {
  return guard([&] {
    require(g, "NULL argument");
    if (segments) *segments = g->g.num_segments();
    if (links) *links = g->g.link_from.size();
    if (jumps) *jumps = g->g.jump_from.size();
    if (containments) *containments = g->g.cont_container.size();
  });
}

gfz_status gfz_encode(gfz_context *ctx, const int32_t *steps, const uint64_t *offsets, uint64_t ntrav, int rounds,
                      uint64_t threshold, int delta_round, int where, gfz_grammar **out) {
  return guard([&] {
    require(offsets && out, "offsets/out are NULL");
    gfz::Context &c = ctx_of(ctx);
    std::vector<uint64_t> off(offsets, offsets + ntrav + 1);
    const uint64_t n = off.back();
    require(steps || n == 0, "steps is NULL");
    if (threshold > 2)
      fprintf(stderr,
              "Warning: freq_threshold > 2 not fully supported with two-set optimization. Using threshold=2.\n");
    auto g = std::make_unique<gfz_grammar>(c.stream());
    if (where == GFZ_WHERE_DEVICE) {
      gfz::encode_traversals(c, steps, off, gfz::EncodeParams{rounds, delta_round}, g->g);
    } else {
      gfz::encode_host(c, {gfz::HostSeg{steps, n}}, off, gfz::EncodeParams{rounds, delta_round}, g->g);
    }
    *out = g.release();
  });
}

gfz_status gfz_grammar_info_get(const gfz_grammar *g, gfz_grammar_info *info) {
  return guard([&] {
    require(g && info, "NULL argument");
    info->ntrav = g->g.ntrav;
    info->encoded_len = g->g.h_off.empty() ? 0 : g->g.h_off.back();
    info->num_rules = g->g.nrules;
    info->layer_start = g->g.layer_start;
    info->next_id = g->g.next_id;
    info->rounds_done = g->g.rounds_done;
    info->delta_round = g->g.delta_round;
  });
}

gfz_status gfz_grammar_copy(gfz_context *ctx, const gfz_grammar *g, int32_t *encoded, uint64_t *offsets,
                            int64_t *rules, int where) {
  return guard([&] {
    require(g, "grammar is NULL");
    gfz::Context &c = ctx_of(ctx);
    const uint64_t m = g->g.h_off.empty() ? 0 : g->g.h_off.back();
    if (encoded) copy_out(c, encoded, g->g.enc.ptr, m * 4, where);
    if (rules) copy_out(c, rules, g->g.rules.ptr, g->g.nrules * 8, where);
    if (offsets) std::memcpy(offsets, g->g.h_off.data(), g->g.h_off.size() * 8);
    c.sync();
  });
}

gfz_status gfz_grammar_rule_columns(gfz_context *ctx, const gfz_grammar *g, int32_t *first, int32_t *second,
                                    int where) {
  return guard([&] {
    require(g && first && second, "NULL argument");
    gfz::Context &c = ctx_of(ctx);
    gfz::DevVec<int32_t> f(c.stream()), s(c.stream());
    gfz::rule_columns_delta(c, g->g, f, s);
    copy_out(c, first, f.ptr, g->g.nrules * 4, where);
    copy_out(c, second, s.ptr, g->g.nrules * 4, where);
    c.sync();
  });
}

gfz_status gfz_grammar_load(gfz_context *ctx, const int32_t *encoded, const uint64_t *offsets, uint64_t ntrav,
                            const int32_t *rules_first, const int32_t *rules_second, uint64_t num_rules,
                            uint32_t min_rule_id, int delta_round, int where, gfz_grammar **out) {
  return guard([&] {
    require(offsets && out, "NULL argument");
    require(num_rules == 0 || (rules_first && rules_second), "rule columns are NULL");
    gfz::Context &c = ctx_of(ctx);
    auto g = std::make_unique<gfz_grammar>(c.stream());
    std::vector<uint64_t> off(offsets, offsets + ntrav + 1);
    const uint64_t m = off.back();
    std::vector<int32_t> hf, hs, he;
    const int32_t *pf = rules_first, *ps = rules_second, *pe = encoded;
    if (where == GFZ_WHERE_DEVICE) {
      // stage through the host once; loading is not on the timed path
      hf.resize(num_rules);
      hs.resize(num_rules);
      he.resize(m);
      if (num_rules) {
        gfz::cuda_check(cudaMemcpy(hf.data(), rules_first, num_rules * 4, cudaMemcpyDeviceToHost), "copy");
        gfz::cuda_check(cudaMemcpy(hs.data(), rules_second, num_rules * 4, cudaMemcpyDeviceToHost), "copy");
      }
      if (m) gfz::cuda_check(cudaMemcpy(he.data(), encoded, m * 4, cudaMemcpyDeviceToHost), "copy");
      pf = hf.data();
      ps = hs.data();
      pe = he.data();
    }
    gfz::load_rules(c, g->g, pf, ps, num_rules, min_rule_id);
    g->g.delta_round = delta_round < 0 ? 0 : delta_round;
    gfz::load_encoded(c, g->g, pe, off);
    c.sync();
    *out = g.release();
  });
}

void gfz_grammar_free(gfz_grammar *g) { delete g; }

gfz_status gfz_decode(gfz_context *ctx, gfz_grammar *g, uint64_t t0, uint64_t t1, int32_t *out, uint64_t cap,
                      uint64_t *n_out, uint64_t *offsets_out, int where) {
  return guard([&] {
    require(g && n_out, "NULL argument");
    gfz::Context &c = ctx_of(ctx);
    gfz::DevVec<int32_t> x(c.stream());
    std::vector<uint64_t> off;
    gfz::decode_traversals(c, g->g, t0, t1, x, off);
    *n_out = off.back();
    if (offsets_out) std::memcpy(offsets_out, off.data(), off.size() * 8);
    if (out) {
      if (cap < off.back()) throw std::length_error("output buffer too small");
      copy_out(c, out, x.ptr, off.back() * 4, where);
    }
    c.sync();
  });
}

gfz_status gfz_decode_text(gfz_context *ctx, gfz_grammar *g, uint64_t t0, uint64_t t1, const gfz_line_meta *meta,
                           char *out, uint64_t cap, uint64_t *size, int where) {
  return guard([&] {
    require(g && meta && size, "NULL argument");
    require(t0 <= t1 && t1 <= g->g.ntrav, "traversal range out of bounds");
    gfz::Context &c = ctx_of(ctx);
    auto pieces = [&](const std::vector<uint64_t> &off) { return pieces_from_meta(meta, off); };
    // device memory or page-locked host memory: the kernels write the text
    // there directly (over the chip-to-chip link for host memory)
    char *direct = nullptr;
    if (out) {
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, out) == cudaSuccess &&
          ((at.type == cudaMemoryTypeDevice && at.device == c.device()) || at.type == cudaMemoryTypeHost) &&
          at.devicePointer)
        direct = static_cast<char *>(at.devicePointer);
      else
        cudaGetLastError();  // not a CUDA allocation
    }
    if (direct) {
      g->text_size = gfz::decode_text(c, g->g, t0, t1, pieces, meta->mode, g->text, direct, cap);
      c.sync();
      g->text_external = true;
    } else {
      g->text_size = gfz::decode_text(c, g->g, t0, t1, pieces, meta->mode, g->text);
      g->text_external = false;
    }
    *size = g->text_size;
    if (out && !direct) {
      if (cap < g->text_size) throw std::length_error("output buffer too small");
      copy_out(c, out, g->text.ptr, g->text_size, where);
      c.sync();
    }
    (void)where;
  });
}

gfz_status gfz_grammar_text(const gfz_grammar *g, const char **device_text, uint64_t *size) {
  return guard([&] {
    require(g && device_text && size, "NULL argument");
    require(!g->text_external, "the last gfz_decode_text wrote its text to the caller's buffer");
    *device_text = g->text.ptr;
    *size = g->text_size;
  });
}

struct gfz_server {
  std::unique_ptr<gfz::Server> s;
};

gfz_status gfz_server_create(int device, const gfz_compressed *c, uint64_t hbm_budget, int workers,
                             gfz_server **out) {
  return guard([&] {
    require(c && out, "NULL argument");
    require(workers >= 1 && workers <= 64, "workers must be in 1..64");
    auto srv = std::make_unique<gfz_server>();
    srv->s = std::make_unique<gfz::Server>(device, c->c, hbm_budget, workers);
    *out = srv.release();
  });
}

gfz_status gfz_server_submit_path(gfz_server *s, const char *name, uint64_t *ticket) {
  return guard([&] {
    require(s && name && ticket, "NULL argument");
    *ticket = s->s->submit_path(name);
  });
}

gfz_status gfz_server_submit_walk(gfz_server *s, const gfz_walk_key *key, uint64_t *ticket) {
  return guard([&] {
    require(s && key && key->sample_id && key->seq_id && ticket, "NULL argument");
    gfz::WalkKey k;
    k.sample_id = key->sample_id;
    k.hap_index = key->hap_index;
    k.seq_id = key->seq_id;
    k.seq_start = key->seq_start;
    k.seq_end = key->seq_end;
    *ticket = s->s->submit_walk(k);
  });
}

gfz_status gfz_server_submit_append(gfz_server *s, const char *gfa_text, size_t len, uint64_t *ticket) {
  return guard([&] {
    require(s && (gfa_text || !len) && ticket, "NULL argument");
    *ticket = s->s->submit_append(std::string(gfa_text ? gfa_text : "", len));
  });
}

gfz_status gfz_server_wait(gfz_server *s, uint64_t ticket, const char **line, size_t *len, double *latency_ms) {
  return guard([&] {
    require(s && line && len, "NULL argument");
    size_t n = 0;
    *line = s->s->wait(ticket, &n, latency_ms);
    *len = n;
  });
}

gfz_status gfz_server_request_times(gfz_server *s, uint64_t ticket, double *queue_ms, double *service_ms,
                                    uint32_t *batch_size) {
  return guard([&] {
    require(s, "NULL argument");
    s->s->times(ticket, queue_ms, service_ms, batch_size);
  });
}

gfz_status gfz_server_collect(gfz_server *s, uint64_t ticket, size_t *len, double *latency_ms, double *queue_ms,
                              double *service_ms, uint32_t *batch_size) {
  return guard([&] {
    require(s && len, "NULL argument");
    size_t n = 0;
    s->s->wait(ticket, &n, latency_ms);
    s->s->times(ticket, queue_ms, service_ms, batch_size);
    s->s->release(ticket);
    *len = n;
  });
}

gfz_status gfz_server_release(gfz_server *s, uint64_t ticket) {
  return guard([&] {
    require(s, "NULL argument");
    s->s->release(ticket);
  });
}

gfz_status gfz_server_stats(gfz_server *s, uint64_t *batches, uint64_t *requests, uint64_t *max_batch) {
  return guard([&] {
    require(s, "NULL argument");
    const gfz::Server::Stats st = s->s->stats();
    if (batches) *batches = st.batches;
    if (requests) *requests = st.requests;
    if (max_batch) *max_batch = st.max_batch;
  });
}

void gfz_server_destroy(gfz_server *s) { delete s; }

gfz_status gfz_inverse_delta_noalloc(const int32_t *steps_in, int32_t *steps_out, uint64_t n, const uint64_t *offsets,
                                     uint64_t ntrav, int delta_round, void *cuda_stream) {
  return guard([&] {
    gfz::inverse_delta_noalloc(steps_in, steps_out, n, offsets, ntrav, delta_round,
                               static_cast<cudaStream_t>(cuda_stream));
  });
}

}  // extern "C"

// Host workflows (see workflows.h).  Container assembly, metadata columns and
// S/L/J/C text stay on the host exactly as in the reference; every traversal
// transform (delta coding, grammar rounds, expansion, inverse delta, P/W
// text) runs on the GPU through the device pipeline.
#include "workflows.h"

#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstring>
#include <exception>
#include <fstream>
#include <future>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <unordered_map>
#include <unordered_set>

namespace gfz {

namespace {

constexpr const char *kCompErr = "Compression workflow error: ";
constexpr const char *kWriterErr = "GFA writer error: ";
constexpr const char *kExtractErr = "Extraction workflow error: ";
constexpr const char *kAddErr = "Add-haplotypes workflow error: ";

std::vector<uint32_t> lengths_of(const std::vector<uint64_t> &off, uint64_t t0, uint64_t t1) {
  std::vector<uint32_t> v;
  v.reserve(t1 - t0);
  for (uint64_t t = t0; t < t1; ++t) v.push_back((uint32_t)(off[t + 1] - off[t]));
  return v;
}

std::vector<uint64_t> offsets_of(const std::vector<uint32_t> &lens) {
  std::vector<uint64_t> off(lens.size() + 1, 0);
  for (size_t i = 0; i < lens.size(); ++i) off[i + 1] = off[i] + lens[i];
  return off;
}

CompressedOptColumn compress_opt(const OptColumn &c) {
  CompressedOptColumn o;
  o.tag = c.tag;
  o.type = c.type;
  switch (c.type) {
    case 'i':
      o.num_elements = c.ints.size();
      o.ints = varint_i64(c.ints);
      break;
    case 'f':
      o.num_elements = c.floats.size();
      o.floats = zstd_f32(c.floats);
      break;
    case 'A':
      o.num_elements = c.chars.size();
      o.chars = zstd_chars(c.chars);
      break;
    case 'Z': case 'J': case 'H':
      o.num_elements = c.string_lengths.size();
      o.strings = zstd_str(c.strings);
      o.string_lengths = zstd_u32(c.string_lengths);
      break;
    case 'B':
      o.num_elements = c.b_subtypes.size();
      o.b_subtypes = zstd_chars(c.b_subtypes);
      o.b_lengths = zstd_u32(c.b_lengths);
      o.b_bytes = zstd_bytes(c.b_bytes.data(), c.b_bytes.size());
      break;
    default:
      throw std::invalid_argument(std::string(kCompErr) + "unsupported optional field type '" +
                                  std::string(1, c.type) + "' for tag '" + c.tag + "'");
  }
  return o;
}

OptColumn decompress_opt(const CompressedOptColumn &c) {
  OptColumn o;
  o.tag = c.tag;
  o.type = c.type;
  switch (c.type) {
    case 'i': o.ints = unvarint_i64(c.ints, c.num_elements); break;
    case 'f': o.floats = unzstd_f32(c.floats); break;
    case 'A': o.chars = unzstd_chars(c.chars); break;
    case 'Z': case 'J': case 'H':
      o.strings = unzstd_str(c.strings);
      o.string_lengths = unzstd_u32(c.string_lengths);
      break;
    case 'B': {
      o.b_subtypes = unzstd_chars(c.b_subtypes);
      o.b_lengths = unzstd_u32(c.b_lengths);
      const std::vector<uint8_t> b = unzstd(c.b_bytes);
      o.b_bytes.assign(b.begin(), b.end());
      break;
    }
    default:
      throw std::runtime_error(std::string(kWriterErr) + "unsupported optional field type");
  }
  return o;
}

size_t b_elem(char s) {
  switch (s) {
    case 'c': case 'C': return 1;
    case 's': case 'S': return 2;
    case 'i': case 'I': case 'f': return 4;
    default: return 0;
  }
}

// Default stream formatting of a float (operator<< on an ostringstream).
std::string fmt_float(float v) {
  std::ostringstream o;
  o << v;
  return o.str();
}

using FieldOffsets = std::vector<std::vector<size_t>>;

FieldOffsets field_offsets(const std::vector<OptColumn> &cols) {
  FieldOffsets f(cols.size());
  for (size_t c = 0; c < cols.size(); ++c) {
    const OptColumn &col = cols[c];
    if (col.type == 'Z' || col.type == 'J' || col.type == 'H') {
      f[c].assign(col.string_lengths.size() + 1, 0);
      for (size_t i = 0; i < col.string_lengths.size(); ++i) f[c][i + 1] = f[c][i] + col.string_lengths[i];
    } else if (col.type == 'B') {
      f[c].assign(col.b_lengths.size() + 1, 0);
      for (size_t i = 0; i < col.b_lengths.size(); ++i)
        f[c][i + 1] = f[c][i] + (size_t)col.b_lengths[i] * b_elem(col.b_subtypes[i]);
    }
  }
  return f;
}

// src/io/gfa_write_utils.cpp:78-165 format_optional_fields
void append_opt_fields(std::string &out, const std::vector<OptColumn> &cols, const FieldOffsets &offs, size_t i) {
  for (size_t c = 0; c < cols.size(); ++c) {
    const OptColumn &col = cols[c];
    switch (col.type) {
      case 'i':
        if (i < col.ints.size() && col.ints[i] != std::numeric_limits<int64_t>::min())
          out += "\t" + col.tag + ":i:" + std::to_string(col.ints[i]);
        break;
      case 'f':
        if (i < col.floats.size() && col.floats[i] != std::numeric_limits<float>::lowest())
          out += "\t" + col.tag + ":f:" + fmt_float(col.floats[i]);
        break;
      case 'A':
        if (i < col.chars.size() && col.chars[i] != '\0') out += "\t" + col.tag + ":A:" + std::string(1, col.chars[i]);
        break;
      case 'Z': case 'J': case 'H':
        if (i < col.string_lengths.size() && col.string_lengths[i] > 0) {
          out += "\t" + col.tag + ":" + std::string(1, col.type) + ":";
          out.append(col.strings, offs[c][i], col.string_lengths[i]);
        }
        break;
      case 'B':
        if (i < col.b_lengths.size()) {
          const char sub = col.b_subtypes[i];
          const uint32_t cnt = col.b_lengths[i];
          if (sub != '\0' && cnt > 0) {
            const size_t es = b_elem(sub);
            const uint8_t *p = col.b_bytes.data() + offs[c][i];
            out += "\t" + col.tag + ":B:" + std::string(1, sub);
            for (uint32_t k = 0; k < cnt; ++k) {
              out += ',';
              const uint8_t *q = p + (size_t)k * es;
              if (sub == 'c') { int8_t v; std::memcpy(&v, q, 1); out += std::to_string(v); }
              else if (sub == 'C') { out += std::to_string(q[0]); }
              else if (sub == 's') { int16_t v; std::memcpy(&v, q, 2); out += std::to_string(v); }
              else if (sub == 'S') { uint16_t v; std::memcpy(&v, q, 2); out += std::to_string(v); }
              else if (sub == 'i') { int32_t v; std::memcpy(&v, q, 4); out += std::to_string(v); }
              else if (sub == 'I') { uint32_t v; std::memcpy(&v, q, 4); out += std::to_string(v); }
              else if (sub == 'f') { float v; std::memcpy(&v, q, 4); out += fmt_float(v); }
            }
          }
        }
        break;
    }
  }
}

// Static (non-traversal) columns decoded for the writer.
struct StaticFields {
  std::string seg_seq;
  std::vector<uint32_t> seg_len;
  std::vector<OptColumn> seg_opt, link_opt;
  std::vector<uint32_t> lf, lt, lnum;
  std::vector<char> lfo, lto, lop;
  std::vector<uint32_t> jf, jt;
  std::vector<char> jfo, jto;
  std::vector<std::string> jdist, jrest;
  std::vector<uint32_t> cc, cd, cpos;
  std::vector<char> cco, cdo;
  std::vector<std::string> cov, crest;
};

// The columns are independent, so they decode in parallel (each zstd frame
// itself decodes on one thread).
StaticFields decode_static(const Compressed &d) {
  StaticFields s;
#pragma omp parallel sections num_threads(4)
  {
#pragma omp section
    s.seg_seq = unzstd_str(d.segment_sequences);
#pragma omp section
    {
      s.seg_len = unzstd_u32(d.segment_seq_lengths);
      for (const auto &c : d.segment_optional) s.seg_opt.push_back(decompress_opt(c));
      for (const auto &c : d.link_optional) s.link_opt.push_back(decompress_opt(c));
    }
#pragma omp section
    {
      s.lf = undelta_varint_u32(d.link_from_ids, d.num_links);
      s.lt = undelta_varint_u32(d.link_to_ids, d.num_links);
    }
#pragma omp section
    {
      s.lfo = unorientations(d.link_from_orients, d.num_links);
      s.lto = unorientations(d.link_to_orients, d.num_links);
      s.lnum = unzstd_u32(d.link_overlap_nums);
      s.lop = unzstd_chars(d.link_overlap_ops);
    }
  }
  if (d.num_jumps > 0) {
    s.jf = undelta_varint_u32(d.jump_from_ids, d.num_jumps);
    s.jt = undelta_varint_u32(d.jump_to_ids, d.num_jumps);
    s.jfo = unorientations(d.jump_from_orients, d.num_jumps);
    s.jto = unorientations(d.jump_to_orients, d.num_jumps);
    s.jdist = split_strings(unzstd_str(d.jump_distances), unzstd_u32(d.jump_distance_lengths), true, kWriterErr);
    s.jrest = split_strings(unzstd_str(d.jump_rest_fields), unzstd_u32(d.jump_rest_lengths), true, kWriterErr);
  }
  if (d.num_containments > 0) {
    s.cc = undelta_varint_u32(d.containment_container_ids, d.num_containments);
    s.cd = undelta_varint_u32(d.containment_contained_ids, d.num_containments);
    s.cco = unorientations(d.containment_container_orients, d.num_containments);
    s.cdo = unorientations(d.containment_contained_orients, d.num_containments);
    s.cpos = unzstd_u32(d.containment_positions);
    s.cov = split_strings(unzstd_str(d.containment_overlaps), unzstd_u32(d.containment_overlap_lengths), true,
                          kWriterErr);
    s.crest = split_strings(unzstd_str(d.containment_rest_fields), unzstd_u32(d.containment_rest_lengths), true,
                            kWriterErr);
  }
  return s;
}

// S lines (host formatting).
void s_text_host(const StaticFields &s, std::string &out) {
  const FieldOffsets so = field_offsets(s.seg_opt);
  std::string line;
  size_t sp = 0;
  for (size_t i = 0; i < s.seg_len.size(); ++i) {
    line = "S\t";
    line += std::to_string(i + 1);
    line += '\t';
    const uint32_t len = s.seg_len[i];
    if (sp + len > s.seg_seq.size())
      throw std::runtime_error(std::string(kWriterErr) + "segment sequence column is truncated");
    line.append(s.seg_seq, sp, len);
    sp += len;
    append_opt_fields(line, s.seg_opt, so, i);
    line += '\n';
    out += line;
  }
}

// L lines (host formatting).
void l_text_host(const StaticFields &s, std::string &out) {
  const FieldOffsets lo = field_offsets(s.link_opt);
  std::string line;
  for (size_t i = 0; i < s.lf.size(); ++i) {
    line = "L\t";
    line += std::to_string(s.lf[i]);
    line += '\t';
    line += s.lfo[i];
    line += '\t';
    line += std::to_string(s.lt[i]);
    line += '\t';
    line += s.lto[i];
    line += '\t';
    if (i < s.lop.size() && s.lop[i] != '\0') {
      line += std::to_string(s.lnum[i]);
      line += s.lop[i];
    } else {
      line += '*';
    }
    append_opt_fields(line, s.link_opt, lo, i);
    line += '\n';
    out += line;
  }
}

// J and C lines.
void jc_text(const StaticFields &s, std::string &out) {
  std::string line;
  for (size_t i = 0; i < s.jf.size(); ++i) {
    line = "J\t" + std::to_string(s.jf[i]) + "\t" + s.jfo[i] + "\t" + std::to_string(s.jt[i]) + "\t" + s.jto[i] + "\t";
    line += i < s.jdist.size() ? s.jdist[i] : "*";
    if (i < s.jrest.size() && !s.jrest[i].empty()) line += "\t" + s.jrest[i];
    line += '\n';
    out += line;
  }
  for (size_t i = 0; i < s.cc.size(); ++i) {
    line = "C\t" + std::to_string(s.cc[i]) + "\t" + s.cco[i] + "\t" + std::to_string(s.cd[i]) + "\t" + s.cdo[i] +
           "\t" + std::to_string(s.cpos[i]) + "\t";
    line += i < s.cov.size() ? s.cov[i] : "*";
    if (i < s.crest.size() && !s.crest[i].empty()) line += "\t" + s.crest[i];
    line += '\n';
    out += line;
  }
}

// H, S, L, J, C text on the host (src/io/gfa_writer.cpp:597-700)
std::string static_text(const Compressed &d, const StaticFields &s) {
  std::string out;
  if (!d.header_line.empty()) out += d.header_line + "\n";
  s_text_host(s, out);
  l_text_host(s, out);
  jc_text(s, out);
  return out;
}

// The optional-field text of lines 0 .. n-1 (what append_opt_fields adds),
// formatted in parallel: blob[off[i] .. off[i+1]).  Empty when there is no
// column.
void opt_extras(const std::vector<OptColumn> &cols, size_t n, int nth, std::string &blob,
                std::vector<uint64_t> &off) {
  blob.clear();
  off.clear();
  if (cols.empty() || !n) return;
  const FieldOffsets fo = field_offsets(cols);
  const int T = std::max(1, std::min<int>(nth, (int)(n / 4096 + 1)));
  std::vector<std::string> part(T);
  off.assign(n + 1, 0);
#pragma omp parallel for schedule(static) num_threads(T)
  for (int t = 0; t < T; ++t) {
    const size_t a = n * t / T, b = n * (t + 1) / T;
    for (size_t i = a; i < b; ++i) {
      append_opt_fields(part[t], cols, fo, i);
      off[i + 1] = part[t].size();  // relative to the part, fixed below
    }
  }
  uint64_t base = 0;
  for (int t = 0; t < T; ++t) {
    const size_t a = n * t / T, b = n * (t + 1) / T;
    for (size_t i = a; i < b; ++i) off[i + 1] += base;
    base += part[t].size();
    blob += part[t];
    std::string().swap(part[t]);
  }
}

template <typename T>
void upload_vec(Context &ctx, DevVec<T> &d, const T *p, uint64_t n) {
  d.resize(std::max<uint64_t>(n, 1));
  if (n) cuda_check(cudaMemcpyAsync(d.ptr, p, n * sizeof(T), cudaMemcpyHostToDevice, ctx.stream()), "upload");
}

// Lines of one kind written on the device and appended to out.
void static_lines_device(Context &ctx, StaticTextSource src, const std::string &ex, const std::vector<uint64_t> &exo,
                         std::string &out) {
  if (!src.n) return;
  cudaStream_t st = ctx.stream();
  DevVec<char> dex(st);
  DevVec<uint64_t> dexo(st), len(st), loff(st);
  if (!exo.empty()) {
    upload_vec(ctx, dex, ex.data(), ex.size());
    upload_vec(ctx, dexo, exo.data(), exo.size());
    src.ex = dex.ptr;
    src.ex_off = dexo.ptr;
  }
  len.resize(src.n);
  loff.resize(src.n + 1);
  ctx.tbegin("static_text", 0);
  launch_static_len(src, len.ptr, st);
  ctx.tend();
  exclusive_scan(ctx, len.ptr, src.n, loff.ptr, "static_text");
  uint64_t total = 0;
  cuda_check(cudaMemcpyAsync(&total, loff.ptr + src.n, 8, cudaMemcpyDeviceToHost, st), "download");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
  DevVec<char> text(st);
  text.resize((total + 15) & ~15ull);
  ctx.tbegin("static_text", (double)total);
  launch_static_write(src, loff.ptr, total, text.ptr, st);
  ctx.tend();
  const size_t o = out.size();
  out.resize(o + total);
  cuda_check(cudaMemcpyAsync(&out[o], text.ptr, total, cudaMemcpyDeviceToHost, st), "text download");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
}

// H, S, L, J, C text with the S and L lines written on the device.
std::string static_text_device(Context &ctx, const Compressed &d, const StaticFields &s, int nth) {
  std::string out;
  if (!d.header_line.empty()) out += d.header_line + "\n";
  cudaStream_t st = ctx.stream();
  std::string ex;
  std::vector<uint64_t> exo;
  {
    const uint64_t ns = s.seg_len.size();
    uint64_t need = 0;
    for (uint64_t i = 0; i < ns; ++i) need += s.seg_len[i];
    if (need > s.seg_seq.size())
      throw std::runtime_error(std::string(kWriterErr) + "segment sequence column is truncated");
    DevVec<char> seq(st);
    DevVec<uint32_t> slen(st);
    DevVec<uint64_t> soff(st);
    upload_vec(ctx, seq, s.seg_seq.data(), need);
    upload_vec(ctx, slen, s.seg_len.data(), ns);
    soff.resize(ns + 1);
    exclusive_scan(ctx, slen.ptr, ns, soff.ptr, "static_text");
    opt_extras(s.seg_opt, ns, nth, ex, exo);
    StaticTextSource src{};
    src.kind = 0;
    src.n = ns;
    src.seq = seq.ptr;
    src.seq_off = soff.ptr;
    src.seg_len = slen.ptr;
    static_lines_device(ctx, src, ex, exo, out);
  }
  {
    const uint64_t nl = s.lf.size();
    std::vector<uint32_t> lnum(s.lnum);
    std::vector<char> lop(s.lop);
    lnum.resize(nl, 0);
    lop.resize(nl, '\0');
    DevVec<uint32_t> lf(st), lt(st), num(st);
    DevVec<char> lfo(st), lto(st), op(st);
    upload_vec(ctx, lf, s.lf.data(), nl);
    upload_vec(ctx, lt, s.lt.data(), nl);
    upload_vec(ctx, num, lnum.data(), nl);
    upload_vec(ctx, lfo, s.lfo.data(), nl);
    upload_vec(ctx, lto, s.lto.data(), nl);
    upload_vec(ctx, op, lop.data(), nl);
    opt_extras(s.link_opt, nl, nth, ex, exo);
    StaticTextSource src{};
    src.kind = 1;
    src.n = nl;
    src.lf = lf.ptr;
    src.lt = lt.ptr;
    src.lnum = num.ptr;
    src.lfo = lfo.ptr;
    src.lto = lto.ptr;
    src.lop = op.ptr;
    static_lines_device(ctx, src, ex, exo, out);
  }
  jc_text(s, out);
  return out;
}

}  // namespace

// Text pieces for the emission kernel: for non-empty traversal t the
// prefix (preceded by the full lines of any empty traversals before it) is
// blob[pre_off[t] .. pre_off[t+1]) and its suffix blob[suf_off[t] ..
// suf_off[t+1]); prefixes and suffixes live in two halves of one blob.
// Lines of empty traversals after the last non-empty one form the tail.
TextPieces make_pieces(const std::vector<std::string> &pre, const std::vector<std::string> &suf,
                       const std::vector<uint64_t> &off) {
  const size_t n = pre.size();
  TextPieces r;
  r.pre_off.assign(n + 1, 0);
  r.suf_off.assign(n + 1, 0);
  std::string pres, sufs, pending;
  for (size_t t = 0; t < n; ++t) {
    const bool empty = off[t + 1] == off[t];
    r.pre_off[t] = pres.size();
    r.suf_off[t] = sufs.size();
    if (empty) {
      pending += pre[t];
      pending += suf[t];
    } else {
      pres += pending;
      pres += pre[t];
      pending.clear();
      sufs += suf[t];
    }
  }
  r.pre_off[n] = pres.size();
  r.suf_off[n] = sufs.size();
  // shift suffix offsets behind the prefixes in one blob
  for (auto &o : r.suf_off) o += pres.size();
  r.blob = pres + sufs;
  r.tail = pending;
  return r;
}

TextPieces path_pieces(const std::vector<std::string> &names, const std::vector<std::string> &overlaps,
                       const std::vector<uint64_t> &off, size_t base) {
  const size_t n = off.size() - 1;
  std::vector<std::string> pre(n), suf(n);
  for (size_t i = 0; i < n; ++i) {
    const size_t t = base + i;
    const std::string &name = t < names.size() ? names[t] : std::to_string(t);
    const std::string ov = t < overlaps.size() ? overlaps[t] : std::string();
    pre[i] = "P\t" + name + "\t";
    suf[i] = "\t" + (ov.empty() ? std::string("*") : ov) + "\n";
  }
  return make_pieces(pre, suf, off);
}

TextPieces walk_pieces(const std::vector<std::string> &samples, const std::vector<uint32_t> &haps,
                       const std::vector<std::string> &seqids, const std::vector<int64_t> &starts,
                       const std::vector<int64_t> &ends, const std::vector<uint64_t> &off, size_t base) {
  const size_t n = off.size() - 1;
  std::vector<std::string> pre(n), suf(n, "\n");
  for (size_t i = 0; i < n; ++i) {
    const size_t t = base + i;
    const std::string sample = t < samples.size() ? samples[t] : "sample";
    const uint32_t hap = t < haps.size() ? haps[t] : 0;
    const std::string seqid = t < seqids.size() ? seqids[t] : "unknown";
    const int64_t st = t < starts.size() ? starts[t] : -1;
    const int64_t en = t < ends.size() ? ends[t] : -1;
    pre[i] = "W\t" + sample + "\t" + std::to_string(hap) + "\t" + seqid + "\t" +
             (st >= 0 ? std::to_string(st) : std::string("*")) + "\t" +
             (en >= 0 ? std::to_string(en) : std::string("*")) + "\t";
  }
  return make_pieces(pre, suf, off);
}

// ---------------------------------------------------------------------------
// Compression
// ---------------------------------------------------------------------------
Compressed compress_graph(Context &ctx, const Graph &g, int rounds, uint64_t threshold, int delta_round, int threads,
                          bool show_stats, const int32_t *d_steps) {
  const int nth = resolve_threads(threads);
  // zstd workers: the given thread count, or every host core when none is
  // given.  The compressed bytes do not depend on the worker count (zstd's
  // multithreaded mode cuts jobs by size; checked with the reference CLI
  // at 1 to 16 workers), only the time does.
  const int zw = threads > 0 ? nth : std::max<int>(nth, (int)std::max(1L, sysconf(_SC_NPROCESSORS_ONLN)));
  set_zstd_threads(zw);
  Compressed out;
  out.header_line = g.header_line;
  if (delta_round < 0) {
    std::cerr << "Warning: delta_round=" << delta_round << " is invalid, clamping to 0" << std::endl;
    delta_round = 0;
  }
  out.delta_round = delta_round;
  const uint64_t np = g.paths.size(), nw = g.walks.size();
  out.original_path_lengths = lengths_of(g.paths.offsets.empty() ? std::vector<uint64_t>{0} : g.paths.offsets, 0, np);
  out.original_walk_lengths = lengths_of(g.walks.offsets.empty() ? std::vector<uint64_t>{0} : g.walks.offsets, 0, nw);
  if (threshold > 2)
    std::cerr << "Warning: freq_threshold > 2 not fully supported with two-set optimization. Using threshold=2."
              << std::endl;

  // one stream: paths then walks
  const uint64_t NP = np ? g.paths.offsets.back() : 0, NW = nw ? g.walks.offsets.back() : 0;
  std::vector<uint64_t> off(np + nw + 1, 0);
  for (uint64_t t = 0; t < np; ++t) off[t + 1] = g.paths.offsets[t + 1];
  for (uint64_t t = 0; t < nw; ++t) off[np + t + 1] = NP + g.walks.offsets[t + 1];
  cudaStream_t st = ctx.stream();
  PhaseClock clk("compress");
  // The segment columns hold segments 1 .. min(S, next_id - 1)
  // (compression_utils.cpp:81-101), where next_id is known only after the
  // transform; it is S unless the stream's ids stay below S.  Their zstd
  // (the largest column) starts for S on a host thread while the transform
  // runs, and is redone for the smaller count in the other case.
  struct SegColumns {
    Block seq, lens;
    size_t ns = 0;
  };
  auto seg_columns = [&g, nth, zw](size_t ns) {
    set_zstd_threads(zw);
    SegColumns r;
    r.ns = ns;
    std::vector<uint32_t> lens(ns);
    std::vector<uint64_t> so(ns + 1, 0);
    for (size_t i = 0; i < ns; ++i) {
      lens[i] = (uint32_t)g.node_sequences[i + 1].size();
      so[i + 1] = so[i] + g.node_sequences[i + 1].size();
    }
    std::string cat(so[ns], '\0');
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int64_t i = 0; i < (int64_t)ns; ++i)
      std::memcpy(&cat[so[i]], g.node_sequences[i + 1].data(), g.node_sequences[i + 1].size());
    r.seq = zstd_str(cat);
    r.lens = zstd_u32(lens);
    return r;
  };
  const size_t S = g.node_sequences.empty() ? 0 : g.node_sequences.size() - 1;
  std::future<SegColumns> fseg = std::async(std::launch::async, seg_columns, S);
  Grammar gram(st);
  if (d_steps)
    encode_traversals(ctx, d_steps, off, EncodeParams{rounds, delta_round}, gram);
  else
    encode_host(ctx, {HostSeg{g.paths.steps.data(), NP}, HostSeg{g.walks.steps.data(), NW}}, off,
                EncodeParams{rounds, delta_round}, gram);

  // rule columns (split + delta on the device)
  DevVec<int32_t> dfirst(st), dsecond(st);
  rule_columns_delta(ctx, gram, dfirst, dsecond);
  std::vector<int32_t> first(gram.nrules), second(gram.nrules);
  if (gram.nrules) {
    cuda_check(cudaMemcpyAsync(first.data(), dfirst.ptr, gram.nrules * 4, cudaMemcpyDeviceToHost, st), "download");
    cuda_check(cudaMemcpyAsync(second.data(), dsecond.ptr, gram.nrules * 4, cudaMemcpyDeviceToHost, st), "download");
  }
  std::vector<int32_t> enc(gram.h_off.back());
  if (!enc.empty())
    cuda_check(cudaMemcpyAsync(enc.data(), gram.enc.ptr, enc.size() * 4, cudaMemcpyDeviceToHost, st), "download");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
  clk.mark("transform + downloads");
  const uint32_t rule_count = gram.next_id - gram.layer_start;
  out.layers.push_back(LayerRange{2, gram.layer_start, gram.next_id, 0, (uint64_t)rule_count * 2});

  const uint64_t ep = gram.h_off[np];
  out.sequence_lengths = lengths_of(gram.h_off, 0, np);
  std::vector<int32_t> pflat(enc.begin(), enc.begin() + (ptrdiff_t)ep);
  std::string names_cat, ov_cat;
  std::vector<uint32_t> name_lens, ov_lens;
  join_strings(g.path_names, names_cat, name_lens);
  join_strings(g.path_overlaps, ov_cat, ov_lens);
  const size_t ns = std::min<size_t>(S, gram.next_id - 1);
  clk.mark("host columns");

#pragma omp parallel sections num_threads(std::min(nth, 8))
  {
#pragma omp section
    {
      set_zstd_threads(zw);
      out.rules_first = zstd_i32(first);
      out.rules_second = zstd_i32(second);
    }
#pragma omp section
    {
      set_zstd_threads(zw);
      out.paths = zstd_i32(pflat);
      out.names = zstd_str(names_cat);
      out.name_lengths = zstd_u32(name_lens);
      out.overlaps = zstd_str(ov_cat);
      out.overlap_lengths = zstd_u32(ov_lens);
    }
#pragma omp section
    {
      set_zstd_threads(zw);
      if (nw) {
        std::vector<int32_t> wflat(enc.begin() + (ptrdiff_t)ep, enc.end());
        out.walk_lengths = lengths_of(gram.h_off, np, np + nw);
        out.walks = zstd_i32(wflat);
        std::string sc, qc;
        std::vector<uint32_t> sl, ql;
        join_strings(g.walk_sample_ids, sc, sl);
        join_strings(g.walk_seq_ids, qc, ql);
        out.walk_sample_ids = zstd_str(sc);
        out.walk_sample_id_lengths = zstd_u32(sl);
        out.walk_hap_indices = zstd_u32(g.walk_hap_indices);
        out.walk_seq_ids = zstd_str(qc);
        out.walk_seq_id_lengths = zstd_u32(ql);
        out.walk_seq_starts = varint_i64(g.walk_seq_starts);
        out.walk_seq_ends = varint_i64(g.walk_seq_ends);
      }
    }
#pragma omp section
    {
      set_zstd_threads(zw);
      out.num_links = g.link_from.size();
      out.link_from_ids = delta_varint_u32(g.link_from);
      out.link_to_ids = delta_varint_u32(g.link_to);
      out.link_from_orients = orientations(g.link_from_orients);
      out.link_to_orients = orientations(g.link_to_orients);
      out.link_overlap_nums = zstd_u32(g.link_overlap_nums);
      out.link_overlap_ops = zstd_chars(g.link_overlap_ops);
    }
#pragma omp section
    {
      set_zstd_threads(zw);
      for (const auto &c : g.segment_optional) out.segment_optional.push_back(compress_opt(c));
      for (const auto &c : g.link_optional) out.link_optional.push_back(compress_opt(c));
      if (!g.jump_from.empty()) {
        std::string dc, rc;
        std::vector<uint32_t> dl, rl;
        join_strings(g.jump_distances, dc, dl);
        join_strings(g.jump_rest, rc, rl);
        out.num_jumps = g.jump_from.size();
        out.jump_from_ids = delta_varint_u32(g.jump_from);
        out.jump_to_ids = delta_varint_u32(g.jump_to);
        out.jump_from_orients = orientations(g.jump_from_orients);
        out.jump_to_orients = orientations(g.jump_to_orients);
        out.jump_distances = zstd_str(dc);
        out.jump_distance_lengths = zstd_u32(dl);
        out.jump_rest_fields = zstd_str(rc);
        out.jump_rest_lengths = zstd_u32(rl);
      }
      if (!g.cont_container.empty()) {
        std::string oc, rc;
        std::vector<uint32_t> ol, rl;
        join_strings(g.cont_overlaps, oc, ol);
        join_strings(g.cont_rest, rc, rl);
        out.num_containments = g.cont_container.size();
        out.containment_container_ids = delta_varint_u32(g.cont_container);
        out.containment_contained_ids = delta_varint_u32(g.cont_contained);
        out.containment_container_orients = orientations(g.cont_container_orients);
        out.containment_contained_orients = orientations(g.cont_contained_orients);
        out.containment_positions = zstd_u32(g.cont_positions);
        out.containment_overlaps = zstd_str(oc);
        out.containment_overlap_lengths = zstd_u32(ol);
        out.containment_rest_fields = zstd_str(rc);
        out.containment_rest_lengths = zstd_u32(rl);
      }
    }
  }
  SegColumns sc = fseg.get();
  if (sc.ns != ns) sc = seg_columns(ns);
  out.segment_sequences = std::move(sc.seq);
  out.segment_seq_lengths = std::move(sc.lens);
  clk.mark("zstd of every column");
  if (show_stats) {
    std::cerr << "\n=== Compressed Data Breakdown ===\n"
              << "Rules (2-mer grammar): " << rule_count << " rules, " << gram.rounds_done << " rounds\n"
              << "  rules_first_zstd:       " << out.rules_first.payload.size() << " B\n"
              << "  rules_second_zstd:      " << out.rules_second.payload.size() << " B\n"
              << "Paths (P-lines): " << np << "\n  paths_zstd:             " << out.paths.payload.size() << " B\n"
              << "Segments (S-lines): " << ns << "\nLinks (L-lines): " << out.num_links << "\n";
    if (nw) std::cerr << "Walks (W-lines): " << nw << "\n  walks_zstd:             " << out.walks.payload.size() << " B\n";
  }
  return out;
}

namespace {
uint64_t file_size(const std::string &path) {
  struct stat sb;
  return stat(path.c_str(), &sb) == 0 ? (uint64_t)sb.st_size : 0;
}
}  // namespace

bool device_front_end_fits(const Context &ctx, uint64_t file_bytes) {
  // the file, line and tile arrays, the steps (at most half the bytes / 2
  // steps of 4 bytes)
  return !ctx.hbm_budget || 3 * file_bytes + (64ull << 20) <= ctx.hbm_budget;
}

Graph parse_graph(Context &ctx, const std::string &gfa_path, int threads) {
  if (ctx.front_end && device_front_end_fits(ctx, file_size(gfa_path))) {
    DeviceParse r = parse_gfa_device(ctx, gfa_path, threads);
    download_steps(ctx, r, r.graph);
    return std::move(r.graph);
  }
  return parse_gfa(gfa_path, threads);
}

Compressed compress_gfa(Context &ctx, const std::string &gfa_path, int rounds, uint64_t threshold, int delta_round,
                        int threads, bool show_stats) {
  if (ctx.front_end && device_front_end_fits(ctx, file_size(gfa_path))) {
    DeviceParse r = parse_gfa_device(ctx, gfa_path, threads);
    const uint64_t n = r.offsets.back();
    if (resident_fits(ctx, n))
      return compress_graph(ctx, r.graph, rounds, threshold, delta_round, threads, show_stats, r.steps.ptr);
    download_steps(ctx, r, r.graph);
    r.steps.release();
    return compress_graph(ctx, r.graph, rounds, threshold, delta_round, threads, show_stats);
  }
  const Graph g = parse_gfa(gfa_path, threads);
  return compress_graph(ctx, g, rounds, threshold, delta_round, threads, show_stats);
}

// ---------------------------------------------------------------------------
// Decompression
// ---------------------------------------------------------------------------
void decode_rule_columns(Context &ctx, const Compressed &c, Grammar &g) {
  const std::vector<int32_t> f = unzstd_i32(c.rules_first), s = unzstd_i32(c.rules_second);
  if (f.size() != s.size()) throw std::runtime_error(std::string(kWriterErr) + "rule columns differ in length");
  load_rules(ctx, g, f.data(), s.data(), f.size(), c.min_rule_id());
  g.delta_round = c.delta_round;
}

namespace {

// All traversals (paths then walks) uploaded into one grammar.
struct LoadedStreams {
  uint64_t np = 0, nw = 0;
};

LoadedStreams load_all(Context &ctx, const Compressed &c, Grammar &g, const char *err_prefix) {
  // the four zstd frames decode in parallel
  std::vector<int32_t> f, s, p, w;
#pragma omp parallel sections num_threads(4)
  {
#pragma omp section
    f = unzstd_i32(c.rules_first);
#pragma omp section
    s = unzstd_i32(c.rules_second);
#pragma omp section
    if (!c.paths.payload.empty()) p = unzstd_i32(c.paths);
#pragma omp section
    if (!c.walks.payload.empty()) w = unzstd_i32(c.walks);
  }
  if (f.size() != s.size()) throw std::runtime_error(std::string(kWriterErr) + "rule columns differ in length");
  load_rules(ctx, g, f.data(), s.data(), f.size(), c.min_rule_id());
  g.delta_round = c.delta_round;
  const std::vector<uint64_t> po = offsets_of(c.sequence_lengths), wo = offsets_of(c.walk_lengths);
  if (po.back() > p.size() || wo.back() > w.size())
    throw std::runtime_error(std::string(err_prefix) + "flattened sequence block is truncated");
  LoadedStreams ls{c.sequence_lengths.size(), c.walk_lengths.size()};
  std::vector<uint64_t> off(ls.np + ls.nw + 1, 0);
  for (uint64_t t = 0; t < ls.np; ++t) off[t + 1] = po[t + 1];
  for (uint64_t t = 0; t < ls.nw; ++t) off[ls.np + t + 1] = po.back() + wo[t + 1];
  std::vector<int32_t> all;
  all.reserve(off.back());
  all.insert(all.end(), p.begin(), p.begin() + (ptrdiff_t)po.back());
  all.insert(all.end(), w.begin(), w.begin() + (ptrdiff_t)wo.back());
  load_encoded(ctx, g, all.data(), off);
  return ls;
}

}  // namespace

void load_traversals(Context &ctx, const Compressed &c, Grammar &g, uint64_t &np, uint64_t &nw) {
  const LoadedStreams ls = load_all(ctx, c, g, "Extraction workflow error: ");
  np = ls.np;
  nw = ls.nw;
}

namespace {

void download_text(Context &ctx, const DevVec<char> &text, uint64_t n, std::string &out) {
  const size_t o = out.size();
  out.resize(o + n);
  if (n)
    cuda_check(cudaMemcpyAsync(&out[o], text.ptr, n, cudaMemcpyDeviceToHost, ctx.stream()), "text download");
  cuda_check(cudaStreamSynchronize(ctx.stream()), "stream sync");
}

}  // namespace

char *RawText::grow(size_t k) {
  if (n_ + k + 1 > cap_) {
    size_t c = std::max<size_t>(cap_ * 2, n_ + k + 1);
    char *q = static_cast<char *>(std::realloc(p_, c));
    if (!q) throw std::bad_alloc();
    p_ = q;
    cap_ = c;
  }
  char *at = p_ + n_;
  n_ += k;
  return at;
}

char *RawText::release() {
  grow(0);
  p_[n_] = '\0';
  char *q = p_;
  p_ = nullptr;
  n_ = cap_ = 0;
  return q;
}

namespace {

// Device text -> host memory through two page-locked staging buffers: the
// copy engine fills one while host threads copy the other out.
void download_raw(Context &ctx, const char *dev, uint64_t n, char *dst, int nth) {
  cudaStream_t st = ctx.stream();
  const uint64_t piece = 128ull << 20;
  cudaEvent_t ev[2];
  cuda_check(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming), "event");
  cuda_check(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming), "event");
  char *stage[2] = {reinterpret_cast<char *>(ctx.host_buffer(0, piece / 4)),
                    reinterpret_cast<char *>(ctx.host_buffer(1, piece / 4))};
  auto issue = [&](uint64_t k) {
    const uint64_t o = k * piece, m = std::min(piece, n - o);
    cuda_check(cudaMemcpyAsync(stage[k & 1], dev + o, m, cudaMemcpyDeviceToHost, st), "text download");
    cuda_check(cudaEventRecord(ev[k & 1], st), "event");
  };
  const uint64_t pieces = (n + piece - 1) / piece;
  if (pieces) issue(0);
  for (uint64_t k = 0; k < pieces; ++k) {
    cuda_check(cudaEventSynchronize(ev[k & 1]), "event sync");
    if (k + 1 < pieces) issue(k + 1);  // the other staging buffer is free
    const uint64_t o = k * piece, m = std::min(piece, n - o);
    const int T = std::max(1, std::min(nth, (int)(m >> 22) + 1));
#pragma omp parallel for schedule(static) num_threads(T)
    for (int t = 0; t < T; ++t) {
      const uint64_t a = m * t / T, b = m * (t + 1) / T;
      std::memcpy(dst + o + a, stage[k & 1] + a, b - a);
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
}

}  // namespace

namespace {

// Boundaries [b[i], b[i+1]) of consecutive groups of the n traversals whose
// expanded steps (lens) stay within `chunk` (a longer traversal is a group
// of its own); chunk 0 gives one group.
std::vector<uint64_t> traversal_groups(uint64_t n, const std::vector<uint32_t> &lens, uint64_t chunk) {
  std::vector<uint64_t> b{0};
  if (!chunk) {
    if (n) b.push_back(n);
    return b;
  }
  uint64_t acc = 0;
  for (uint64_t t = 0; t < n; ++t) {
    const uint64_t len = t < lens.size() ? lens[t] : 0;
    if (t > b.back() && acc + len > chunk) {
      b.push_back(t);
      acc = 0;
    }
    acc += len;
  }
  if (n) b.push_back(n);
  return b;
}

}  // namespace

void gfa_text_into(Context &ctx, const Compressed &c, int threads, RawText &out) {
  const int nth = resolve_threads(threads);
  set_zstd_threads(nth);
  PhaseClock clk("gfa text");
  // The static columns' zstd runs on its own host thread while the grammar
  // loads and the P text is written on the device; that text waits in HBM
  // until the H/S/L/J/C text before it is in place.  An error in the static
  // columns is reported first, as when the steps ran one after the other.
  // With ctx.decode_chunk set, P and W text are written in traversal groups
  // of at most that many expanded steps, each downloaded before the next is
  // decoded, so the device holds one group's output at a time.
  std::future<StaticFields> fs = std::async(std::launch::async, [&c] { return decode_static(c); });
  Grammar g(ctx.stream());
  DevVec<char> text(ctx.stream());
  LoadedStreams ls{};
  uint64_t pn = 0;
  std::vector<std::string> names, ovs;
  std::exception_ptr dev_err;
  try {
    ls = load_all(ctx, c, g, kWriterErr);
    clk.mark("rules + encoded streams (zstd, upload)");
    if (ls.np) {
      names = split_strings(unzstd_str(c.names), unzstd_u32(c.name_lengths), true, kWriterErr);
      ovs = split_strings(unzstd_str(c.overlaps), unzstd_u32(c.overlap_lengths), true, kWriterErr);
      if (!ctx.decode_chunk) {
        pn = decode_text(
            ctx, g, 0, ls.np, [&](const std::vector<uint64_t> &xoff) { return path_pieces(names, ovs, xoff); }, 0,
            text);
        clk.mark("P text (device)");
      }
    }
  } catch (...) {
    dev_err = std::current_exception();
  }
  const StaticFields s = fs.get();
  if (dev_err) std::rethrow_exception(dev_err);
  clk.mark("static columns (zstd, overlapped)");
  out.append(ctx.static_text ? static_text_device(ctx, c, s, nth) : static_text(c, s));
  clk.mark("H/S/L/J/C text");
  if (ls.np) {
    if (!ctx.decode_chunk) {
      download_raw(ctx, text.ptr, pn, out.grow(pn), nth);
    } else {
      const std::vector<uint64_t> b = traversal_groups(ls.np, c.original_path_lengths, ctx.decode_chunk);
      for (size_t i = 0; i + 1 < b.size(); ++i) {
        const uint64_t n = decode_text(
            ctx, g, b[i], b[i + 1],
            [&](const std::vector<uint64_t> &xoff) { return path_pieces(names, ovs, xoff, b[i]); }, 0, text);
        download_raw(ctx, text.ptr, n, out.grow(n), nth);
      }
    }
    clk.mark("P text download");
  }
  if (ls.nw) {
    const auto samples =
        split_strings(unzstd_str(c.walk_sample_ids), unzstd_u32(c.walk_sample_id_lengths), true, kWriterErr);
    const auto haps = unzstd_u32(c.walk_hap_indices);
    const auto seqids = split_strings(unzstd_str(c.walk_seq_ids), unzstd_u32(c.walk_seq_id_lengths), true, kWriterErr);
    const auto starts = unvarint_i64(c.walk_seq_starts, c.walk_lengths.size());
    const auto ends = unvarint_i64(c.walk_seq_ends, c.walk_lengths.size());
    const std::vector<uint64_t> b = traversal_groups(ls.nw, c.original_walk_lengths, ctx.decode_chunk);
    for (size_t i = 0; i + 1 < b.size(); ++i) {
      const uint64_t n = decode_text(
          ctx, g, ls.np + b[i], ls.np + b[i + 1],
          [&](const std::vector<uint64_t> &xoff) {
            return walk_pieces(samples, haps, seqids, starts, ends, xoff, b[i]);
          },
          1, text);
      download_raw(ctx, text.ptr, n, out.grow(n), nth);
    }
  }
}

std::string gfa_text(Context &ctx, const Compressed &c, int threads) {
  RawText t;
  gfa_text_into(ctx, c, threads, t);
  return std::string(t.data() ? t.data() : "", t.size());
}

void write_gfa(Context &ctx, const Compressed &c, const std::string &out_path, int threads) {
  std::ofstream out(out_path, std::ios::binary);
  if (!out) throw std::runtime_error(std::string(kWriterErr) + "failed to open output file: " + out_path);
  RawText text;
  gfa_text_into(ctx, c, threads, text);
  out.write(text.data(), (std::streamsize)text.size());
  if (!out) throw std::runtime_error(std::string(kWriterErr) + "failed to write output file: " + out_path);
}

Graph decompress_graph(Context &ctx, const Compressed &c, int threads) {
  set_zstd_threads(resolve_threads(threads));
  Graph g;
  g.header_line = c.header_line;
  // the static columns' zstd runs on its own host thread while the
  // traversals decode; its errors are raised at the same point as before
  std::future<StaticFields> fs = std::async(std::launch::async, [&c] { return decode_static(c); });
  Grammar gram(ctx.stream());
  const LoadedStreams ls = load_all(ctx, c, gram, kWriterErr);
  auto fetch = [&](uint64_t t0, uint64_t t1, Traversals &tv) {
    DevVec<int32_t> x(ctx.stream());
    decode_traversals(ctx, gram, t0, t1, x, tv.offsets);
    tv.steps.resize(tv.offsets.back());
    if (!tv.steps.empty())
      cuda_check(cudaMemcpyAsync(tv.steps.data(), x.ptr, tv.steps.size() * 4, cudaMemcpyDeviceToHost, ctx.stream()),
                 "download");
    cuda_check(cudaStreamSynchronize(ctx.stream()), "stream sync");
  };
  fetch(0, ls.np, g.paths);
  fetch(ls.np, ls.np + ls.nw, g.walks);
  g.path_names = split_strings(unzstd_str(c.names), unzstd_u32(c.name_lengths), false, kWriterErr);
  g.path_overlaps = split_strings(unzstd_str(c.overlaps), unzstd_u32(c.overlap_lengths), false, kWriterErr);
  g.walk_sample_ids = split_strings(unzstd_str(c.walk_sample_ids), unzstd_u32(c.walk_sample_id_lengths), false, "");
  g.walk_hap_indices = unzstd_u32(c.walk_hap_indices);
  g.walk_seq_ids = split_strings(unzstd_str(c.walk_seq_ids), unzstd_u32(c.walk_seq_id_lengths), false, "");
  g.walk_seq_starts = unvarint_i64(c.walk_seq_starts, c.walk_lengths.size());
  g.walk_seq_ends = unvarint_i64(c.walk_seq_ends, c.walk_lengths.size());
  StaticFields s = fs.get();
  const size_t ns = s.seg_len.size();
  std::vector<uint64_t> so(ns + 1, 0);
  for (size_t i = 0; i < ns; ++i) so[i + 1] = so[i] + s.seg_len[i];
  if (ns && so[ns - 1] > s.seg_seq.size())
    throw std::runtime_error(std::string(kWriterErr) + "segment sequence column is truncated");
  g.node_names.resize(ns + 1);
  g.node_sequences.resize(ns + 1);
#pragma omp parallel for schedule(static) num_threads(resolve_threads(threads))
  for (int64_t i = 0; i < (int64_t)ns; ++i) {
    g.node_names[i + 1] = std::to_string(i + 1);
    g.node_sequences[i + 1] = s.seg_seq.substr(so[i], s.seg_len[i]);  // the last may run short
  }
  g.segment_optional = std::move(s.seg_opt);
  g.link_from = std::move(s.lf);
  g.link_to = std::move(s.lt);
  g.link_from_orients = std::move(s.lfo);
  g.link_to_orients = std::move(s.lto);
  g.link_overlap_nums = std::move(s.lnum);
  g.link_overlap_ops = std::move(s.lop);
  g.link_optional = std::move(s.link_opt);
  g.jump_from = std::move(s.jf);
  g.jump_to = std::move(s.jt);
  g.jump_from_orients = std::move(s.jfo);
  g.jump_to_orients = std::move(s.jto);
  g.jump_distances = std::move(s.jdist);
  g.jump_rest = std::move(s.jrest);
  g.cont_container = std::move(s.cc);
  g.cont_contained = std::move(s.cd);
  g.cont_container_orients = std::move(s.cco);
  g.cont_contained_orients = std::move(s.cdo);
  g.cont_positions = std::move(s.cpos);
  g.cont_overlaps = std::move(s.cov);
  g.cont_rest = std::move(s.crest);
  return g;
}

// ---------------------------------------------------------------------------
// Extraction
// ---------------------------------------------------------------------------
namespace {

std::vector<std::string> split_lines(const std::string &text, size_t n) {
  std::vector<std::string> lines;
  lines.reserve(n);
  size_t b = 0;
  for (size_t i = 0; i < text.size(); ++i)
    if (text[i] == '\n') {
      lines.push_back(text.substr(b, i + 1 - b));
      b = i + 1;
    }
  return lines;
}

// Decodes the selected traversals of one stream kind into text lines.
std::vector<std::string> decode_selected(Context &ctx, const Compressed &c, const Block &stream,
                                         const std::vector<uint32_t> &lens, const std::vector<size_t> &idx,
                                         const std::vector<std::string> &pre, const std::vector<std::string> &suf,
                                         int mode) {
  const std::vector<int32_t> flat = unzstd_i32(stream);
  const std::vector<uint64_t> off = offsets_of(lens);
  std::vector<int32_t> sel;
  std::vector<uint64_t> soff(1, 0);
  for (size_t i : idx) {
    if (i >= lens.size()) throw std::out_of_range(std::string(kExtractErr) + "sequence index out of range");
    if (off[i] + lens[i] > flat.size())
      throw std::runtime_error(std::string(kExtractErr) + "flattened sequence block is truncated");
    sel.insert(sel.end(), flat.begin() + (ptrdiff_t)off[i], flat.begin() + (ptrdiff_t)off[i + 1]);
    soff.push_back(sel.size());
  }
  Grammar g(ctx.stream());
  decode_rule_columns(ctx, c, g);
  load_encoded(ctx, g, sel.data(), soff);
  DevVec<char> text(ctx.stream());
  const uint64_t n = decode_text(
      ctx, g, 0, idx.size(), [&](const std::vector<uint64_t> &xoff) { return make_pieces(pre, suf, xoff); }, mode,
      text);
  std::string s;
  download_text(ctx, text, n, s);
  return split_lines(s, idx.size());
}

}  // namespace

std::vector<std::string> extract_path_lines(Context &ctx, const Compressed &c, const std::vector<std::string> &names,
                                            int threads) {
  set_zstd_threads(resolve_threads(threads));
  if (names.empty()) return {};
  const auto stored = split_strings(unzstd_str(c.names), unzstd_u32(c.name_lengths), true, kExtractErr);
  std::unordered_map<std::string, size_t> index;
  for (size_t i = 0; i < stored.size(); ++i)
    if (!index.emplace(stored[i], i).second)
      throw std::runtime_error(std::string(kExtractErr) + "path name is ambiguous: " + stored[i]);
  std::vector<size_t> idx;
  for (const auto &n : names) {
    auto it = index.find(n);
    if (it == index.end()) throw std::runtime_error(std::string(kExtractErr) + "path not found: " + n);
    idx.push_back(it->second);
  }
  const auto ovs = split_strings(unzstd_str(c.overlaps), unzstd_u32(c.overlap_lengths), true, kExtractErr);
  std::vector<std::string> pre, suf;
  for (size_t k = 0; k < idx.size(); ++k) {
    const std::string ov = idx[k] < ovs.size() ? ovs[idx[k]] : std::string();
    pre.push_back("P\t" + names[k] + "\t");
    suf.push_back("\t" + (ov.empty() ? std::string("*") : ov) + "\n");
  }
  return decode_selected(ctx, c, c.paths, c.sequence_lengths, idx, pre, suf, 0);
}

static std::vector<std::string> walk_lines_for(Context &ctx, const Compressed &c, const std::vector<WalkKey> &keys,
                                               const std::vector<size_t> &idx) {
  std::vector<std::string> pre, suf;
  for (const auto &k : keys) {
    pre.push_back("W\t" + k.sample_id + "\t" + std::to_string(k.hap_index) + "\t" + k.seq_id + "\t" +
                  (k.seq_start >= 0 ? std::to_string(k.seq_start) : std::string("*")) + "\t" +
                  (k.seq_end >= 0 ? std::to_string(k.seq_end) : std::string("*")) + "\t");
    suf.push_back("\n");
  }
  return decode_selected(ctx, c, c.walks, c.walk_lengths, idx, pre, suf, 1);
}

std::vector<std::string> extract_walk_lines(Context &ctx, const Compressed &c, const std::vector<WalkKey> &keys,
                                            int threads) {
  set_zstd_threads(resolve_threads(threads));
  if (keys.empty()) return {};
  const auto samples =
      split_strings(unzstd_str(c.walk_sample_ids), unzstd_u32(c.walk_sample_id_lengths), true, kExtractErr);
  const auto haps = unzstd_u32(c.walk_hap_indices);
  const auto seqids = split_strings(unzstd_str(c.walk_seq_ids), unzstd_u32(c.walk_seq_id_lengths), true, kExtractErr);
  const auto starts = unvarint_i64(c.walk_seq_starts, c.walk_lengths.size());
  const auto ends = unvarint_i64(c.walk_seq_ends, c.walk_lengths.size());
  std::vector<size_t> idx;
  for (const auto &k : keys) {
    size_t found = c.walk_lengths.size();
    for (size_t i = 0; i < c.walk_lengths.size(); ++i) {
      if (i < samples.size() && i < haps.size() && i < seqids.size() && i < starts.size() && i < ends.size() &&
          samples[i] == k.sample_id && haps[i] == k.hap_index && seqids[i] == k.seq_id && starts[i] == k.seq_start &&
          ends[i] == k.seq_end) {
        found = i;
        break;
      }
    }
    if (found == c.walk_lengths.size())
      throw std::runtime_error(std::string(kExtractErr) + "walk not found for the provided identifier: " +
                               k.sample_id + "\t" + std::to_string(k.hap_index) + "\t" + k.seq_id + "\t" +
                               std::to_string(k.seq_start) + "\t" + std::to_string(k.seq_end));
    idx.push_back(found);
  }
  return walk_lines_for(ctx, c, keys, idx);
}

std::vector<std::string> extract_walk_lines_by_name(Context &ctx, const Compressed &c,
                                                    const std::vector<std::string> &names, int threads) {
  set_zstd_threads(resolve_threads(threads));
  if (names.empty()) return {};
  const auto samples =
      split_strings(unzstd_str(c.walk_sample_ids), unzstd_u32(c.walk_sample_id_lengths), true, kExtractErr);
  std::unordered_map<std::string, size_t> index;
  for (size_t i = 0; i < samples.size(); ++i)
    if (!index.emplace(samples[i], i).second)
      throw std::runtime_error(std::string(kExtractErr) + "walk name is ambiguous: " + samples[i]);
  std::vector<size_t> idx;
  for (const auto &n : names) {
    auto it = index.find(n);
    if (it == index.end()) throw std::runtime_error(std::string(kExtractErr) + "walk not found: " + n);
    idx.push_back(it->second);
  }
  const auto haps = unzstd_u32(c.walk_hap_indices);
  const auto seqids = split_strings(unzstd_str(c.walk_seq_ids), unzstd_u32(c.walk_seq_id_lengths), true, kExtractErr);
  const auto starts = unvarint_i64(c.walk_seq_starts, c.walk_lengths.size());
  const auto ends = unvarint_i64(c.walk_seq_ends, c.walk_lengths.size());
  std::vector<WalkKey> keys;
  for (size_t k = 0; k < names.size(); ++k) {
    const size_t i = idx[k];
    WalkKey key;
    key.sample_id = names[k];
    key.hap_index = i < haps.size() ? haps[i] : 0;
    key.seq_id = i < seqids.size() ? seqids[i] : "unknown";
    key.seq_start = i < starts.size() ? starts[i] : -1;
    key.seq_end = i < ends.size() ? ends[i] : -1;
    keys.push_back(key);
  }
  // resolve through the full-key scan, as the reference does
  return extract_walk_lines(ctx, c, keys, threads);
}

// ---------------------------------------------------------------------------
// Add-haplotypes
// ---------------------------------------------------------------------------
namespace {

std::string_view field(std::string_view line, size_t &pos) {
  while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
  const size_t b = pos;
  while (pos < line.size() && line[pos] != ' ' && line[pos] != '\t') ++pos;
  return line.substr(b, pos - b);
}

bool numeric(std::string_view v) {
  if (v.empty()) return false;
  for (char ch : v)
    if (ch < '0' || ch > '9') return false;
  return true;
}

uint32_t strict_u32(std::string_view v, const char *what) {
  if (!numeric(v)) throw std::runtime_error(std::string(kAddErr) + what + " must be numeric");
  uint64_t x = 0;
  for (char ch : v) {
    x = x * 10 + (uint64_t)(ch - '0');
    if (x > 0xFFFFFFFFull) throw std::runtime_error(std::string(kAddErr) + what + " overflows uint32");
  }
  return (uint32_t)x;
}

int64_t strict_i64_or_star(std::string_view v, const char *what) {
  if (v == "*") return -1;
  if (v.empty()) throw std::runtime_error(std::string(kAddErr) + what + " is empty");
  size_t p = 0;
  const bool neg = v[0] == '-';
  if (neg) ++p;
  if (p >= v.size()) throw std::runtime_error(std::string(kAddErr) + what + " is invalid");
  int64_t x = 0;
  for (; p < v.size(); ++p) {
    const char ch = v[p];
    if (ch < '0' || ch > '9') throw std::runtime_error(std::string(kAddErr) + what + " must be an integer or '*'");
    const int dgt = ch - '0';
    if (!neg) {
      if (x > (std::numeric_limits<int64_t>::max() - dgt) / 10)
        throw std::runtime_error(std::string(kAddErr) + what + " overflows int64");
      x = x * 10 + dgt;
    } else {
      if (x < (std::numeric_limits<int64_t>::min() + dgt) / 10)
        throw std::runtime_error(std::string(kAddErr) + what + " overflows int64");
      x = x * 10 - dgt;
    }
  }
  return x;
}

int32_t strict_node(std::string_view v, char o, const char *what) {
  const uint32_t id = strict_u32(v, what);
  if (id == 0) throw std::runtime_error(std::string(kAddErr) + what + " must be 1-based and non-zero");
  return (o == '-' || o == '<') ? -(int32_t)id : (int32_t)id;
}

AppendInput parse_append_stream(std::istream &in) {
  AppendInput a;
  a.paths.offsets.push_back(0);
  a.walks.offsets.push_back(0);
  std::string line;
  size_t ln = 0;
  while (std::getline(in, line)) {
    ++ln;
    if (line.empty()) continue;
    const char type = line[0];
    if (type == 'H' || type == '#') continue;
    const std::string_view v(line);
    if (type == 'P' || type == 'W') {
      if ((type == 'P' && a.has_walks) || (type == 'W' && a.has_paths))
        throw std::runtime_error(std::string(kAddErr) +
                                 "input file mixes P-lines and W-lines; use a pure path or pure walk file");
    }
    if (type == 'P') {
      size_t pos = 1;
      const std::string_view name = field(v, pos), steps = field(v, pos);
      while (pos < v.size() && (v[pos] == ' ' || v[pos] == '\t')) ++pos;
      const std::string ov(v.substr(pos));
      if (name.empty()) throw std::runtime_error(std::string(kAddErr) + "P-line path name is empty");
      size_t s0 = 0;
      for (size_t k = 0; k <= steps.size(); ++k) {
        if (k == steps.size() || steps[k] == ',') {
          if (k > s0) {
            const std::string_view tok = steps.substr(s0, k - s0);
            if (tok.size() < 2) throw std::runtime_error(std::string(kAddErr) + "invalid P-line node token");
            const char o = tok.back();
            if (o != '+' && o != '-')
              throw std::runtime_error(std::string(kAddErr) + "P-line node orientation must be '+' or '-'");
            const std::string_view nm = tok.substr(0, tok.size() - 1);
            if (!numeric(nm))
              throw std::runtime_error(std::string(kAddErr) +
                                       "CPU .gfaz does not store original segment names; appended P-lines must use "
                                       "numeric segment IDs");
            a.paths.steps.push_back(strict_node(nm, o, "P-line segment ID"));
          }
          s0 = k + 1;
        }
      }
      a.names.emplace_back(name);
      a.overlaps.push_back(ov);
      a.paths.offsets.push_back(a.paths.steps.size());
      a.has_paths = true;
    } else if (type == 'W') {
      size_t pos = 1;
      const std::string_view sample = field(v, pos), hap = field(v, pos), seqid = field(v, pos);
      const std::string_view st = field(v, pos), en = field(v, pos), walk = field(v, pos);
      if (sample.empty()) throw std::runtime_error(std::string(kAddErr) + "W-line sample_id is empty");
      size_t p = 0;
      while (p < walk.size()) {
        const char o = walk[p];
        if (o != '>' && o != '<') throw std::runtime_error(std::string(kAddErr) + "W-line walk string is malformed");
        size_t e = p + 1;
        while (e < walk.size() && walk[e] != '>' && walk[e] != '<') ++e;
        const std::string_view nm = walk.substr(p + 1, e - p - 1);
        if (!numeric(nm))
          throw std::runtime_error(std::string(kAddErr) +
                                   "CPU .gfaz does not store original segment names; appended W-lines must use "
                                   "numeric segment IDs");
        a.walks.steps.push_back(strict_node(nm, o, "W-line segment ID"));
        p = e;
      }
      a.samples.emplace_back(sample);
      a.haps.push_back(strict_u32(hap, "W-line hap_index"));
      a.seqids.emplace_back(seqid);
      a.starts.push_back(strict_i64_or_star(st, "W-line seq_start"));
      a.ends.push_back(strict_i64_or_star(en, "W-line seq_end"));
      a.walks.offsets.push_back(a.walks.steps.size());
      a.has_walks = true;
    } else {
      throw std::runtime_error(std::string(kAddErr) + "unsupported line type '" + std::string(1, type) +
                               "' at line " + std::to_string(ln) + "; only H/P/W lines are accepted");
    }
  }
  if (!a.has_paths && !a.has_walks)
    throw std::runtime_error(std::string(kAddErr) + "input file does not contain any P-lines or W-lines");
  return a;
}

AppendInput parse_append(const std::string &path) {
  std::ifstream in(path);
  if (!in.is_open()) throw std::runtime_error(std::string(kAddErr) + "failed to open input file '" + path + "'");
  return parse_append_stream(in);
}

std::string walk_identity(const std::string &s, uint32_t h, const std::string &q, int64_t a, int64_t b) {
  return s + '\x1f' + std::to_string(h) + '\x1f' + q + '\x1f' + std::to_string(a) + '\x1f' + std::to_string(b);
}

// Delta + collision check + per-layer stack encoding on the GPU; appends
// encoded traversals to flat/lens.
void encode_append(Context &ctx, const Compressed &c, const Traversals &tv, std::vector<int32_t> &flat,
                   std::vector<uint32_t> &lens) {
  Grammar g(ctx.stream());
  decode_rule_columns(ctx, c, g);
  std::vector<Layer> layers;
  for (const auto &l : c.layers) layers.push_back(Layer{l.k, l.start_id, l.end_id, l.flattened_offset, l.element_count});
  std::vector<int32_t> steps = tv.steps;
  std::vector<uint64_t> out_lens;
  uint32_t max_abs = 0;
  append_encode(ctx, g.first.ptr, g.second.ptr, g.nrules, layers, c.delta_round, steps, tv.offsets, out_lens,
                max_abs);
  if (!c.layers.empty() && max_abs >= c.min_rule_id())
    throw std::runtime_error(std::string(kAddErr) + "delta-encoded appended sequence reaches ID " +
                             std::to_string(max_abs) + ", which collides with the stored rule region starting at " +
                             std::to_string(c.min_rule_id()));
  flat.insert(flat.end(), steps.begin(), steps.end());
  for (size_t t = 0; t + 1 < tv.offsets.size(); ++t) lens.push_back((uint32_t)out_lens[t]);
}

}  // namespace

AppendInput parse_append_text(const std::string &gfa_text) {
  std::istringstream in(gfa_text);
  return parse_append_stream(in);
}

static void add_haplotypes_input(Context &ctx, Compressed &c, const AppendInput &in);

void add_haplotypes(Context &ctx, Compressed &c, const std::string &path, int threads) {
  set_zstd_threads(resolve_threads(threads));
  add_haplotypes_input(ctx, c, parse_append(path));
}

void add_haplotypes_text(Context &ctx, Compressed &c, const std::string &gfa_text, int threads) {
  set_zstd_threads(resolve_threads(threads));
  std::istringstream in(gfa_text);
  add_haplotypes_input(ctx, c, parse_append_stream(in));
}

static void add_haplotypes_input(Context &ctx, Compressed &c, const AppendInput &in) {
  if (in.has_paths) {
    std::vector<std::string> names = split_strings(unzstd_str(c.names), unzstd_u32(c.name_lengths), true, kAddErr);
    std::unordered_set<std::string> seen(names.begin(), names.end());
    for (const auto &n : in.names)
      if (!seen.insert(n).second)
        throw std::runtime_error(std::string(kAddErr) + "path name already exists or is duplicated: " + n);
    std::vector<std::string> ovs = split_strings(unzstd_str(c.overlaps), unzstd_u32(c.overlap_lengths), true, kAddErr);
    std::vector<int32_t> flat = unzstd_i32(c.paths);
    for (size_t t = 0; t < in.names.size(); ++t)
      c.original_path_lengths.push_back((uint32_t)(in.paths.offsets[t + 1] - in.paths.offsets[t]));
    encode_append(ctx, c, in.paths, flat, c.sequence_lengths);
    names.insert(names.end(), in.names.begin(), in.names.end());
    ovs.insert(ovs.end(), in.overlaps.begin(), in.overlaps.end());
    std::string nc, oc;
    std::vector<uint32_t> nl, ol;
    join_strings(names, nc, nl);
    join_strings(ovs, oc, ol);
    c.paths = zstd_i32(flat);
    c.names = zstd_str(nc);
    c.name_lengths = zstd_u32(nl);
    c.overlaps = zstd_str(oc);
    c.overlap_lengths = zstd_u32(ol);
  } else {
    std::vector<std::string> samples =
        split_strings(unzstd_str(c.walk_sample_ids), unzstd_u32(c.walk_sample_id_lengths), true, kAddErr);
    std::vector<uint32_t> haps = unzstd_u32(c.walk_hap_indices);
    std::vector<std::string> seqids =
        split_strings(unzstd_str(c.walk_seq_ids), unzstd_u32(c.walk_seq_id_lengths), true, kAddErr);
    std::vector<int64_t> starts = unvarint_i64(c.walk_seq_starts, c.walk_lengths.size());
    std::vector<int64_t> ends = unvarint_i64(c.walk_seq_ends, c.walk_lengths.size());
    std::unordered_set<std::string> seen;
    for (size_t i = 0; i < samples.size(); ++i)
      seen.insert(walk_identity(samples[i], i < haps.size() ? haps[i] : 0, i < seqids.size() ? seqids[i] : "",
                                i < starts.size() ? starts[i] : 0, i < ends.size() ? ends[i] : 0));
    for (size_t i = 0; i < in.samples.size(); ++i)
      if (!seen.insert(walk_identity(in.samples[i], in.haps[i], in.seqids[i], in.starts[i], in.ends[i])).second)
        throw std::runtime_error(std::string(kAddErr) + "walk identifier already exists or is duplicated: " +
                                 in.samples[i] + "\t" + std::to_string(in.haps[i]) + "\t" + in.seqids[i] + "\t" +
                                 std::to_string(in.starts[i]) + "\t" + std::to_string(in.ends[i]));
    std::vector<int32_t> flat = unzstd_i32(c.walks);
    for (size_t t = 0; t < in.samples.size(); ++t)
      c.original_walk_lengths.push_back((uint32_t)(in.walks.offsets[t + 1] - in.walks.offsets[t]));
    encode_append(ctx, c, in.walks, flat, c.walk_lengths);
    samples.insert(samples.end(), in.samples.begin(), in.samples.end());
    haps.insert(haps.end(), in.haps.begin(), in.haps.end());
    seqids.insert(seqids.end(), in.seqids.begin(), in.seqids.end());
    starts.insert(starts.end(), in.starts.begin(), in.starts.end());
    ends.insert(ends.end(), in.ends.begin(), in.ends.end());
    std::string sc, qc;
    std::vector<uint32_t> sl, ql;
    join_strings(samples, sc, sl);
    join_strings(seqids, qc, ql);
    c.walks = zstd_i32(flat);
    c.walk_sample_ids = zstd_str(sc);
    c.walk_sample_id_lengths = zstd_u32(sl);
    c.walk_hap_indices = zstd_u32(haps);
    c.walk_seq_ids = zstd_str(qc);
    c.walk_seq_id_lengths = zstd_u32(ql);
    c.walk_seq_starts = varint_i64(starts);
    c.walk_seq_ends = varint_i64(ends);
  }
}

}  // namespace gfz

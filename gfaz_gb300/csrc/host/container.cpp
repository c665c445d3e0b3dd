// .gfaz v5 container reader / writer.
//
// Field order, widths and length prefixes follow the reference writer
// (src/codec/serialization.cpp:137-236): little-endian PODs, u64 counts, a
// block is (u64 original_size, u64 n, n bytes), a string is (u64 n, bytes),
// a u32 vector is (u64 count, data).  The reader validates every length
// against the remaining bytes, so truncated or corrupted files raise an
// error instead of reading past the end.
#include <cstring>
#include <fstream>
#include <iostream>
#include <stdexcept>

#include "model.h"

namespace gfz {

namespace {

constexpr const char *kErr = "GFAZ serialization error: ";

struct Writer {
  std::vector<uint8_t> out;
  template <typename T>
  void pod(const T &v) {
    const uint8_t *p = reinterpret_cast<const uint8_t *>(&v);
    out.insert(out.end(), p, p + sizeof(T));
  }
  void bytes(const void *p, size_t n) {
    const uint8_t *b = static_cast<const uint8_t *>(p);
    out.insert(out.end(), b, b + n);
  }
  void str(const std::string &s) {
    pod<uint64_t>(s.size());
    bytes(s.data(), s.size());
  }
  void u32vec(const std::vector<uint32_t> &v) {
    pod<uint64_t>(v.size());
    bytes(v.data(), v.size() * 4);
  }
  void block(const Block &b) {
    pod<uint64_t>(b.original_size);
    pod<uint64_t>(b.payload.size());
    bytes(b.payload.data(), b.payload.size());
  }
  void opt(const CompressedOptColumn &c) {
    str(c.tag);
    pod<char>(c.type);
    pod<uint64_t>(c.num_elements);
    for (const Block *b : {&c.ints, &c.floats, &c.chars, &c.strings, &c.string_lengths, &c.b_subtypes, &c.b_lengths,
                           &c.b_bytes})
      block(*b);
  }
};

struct Reader {
  const uint8_t *p;
  size_t n, pos = 0;
  void need(uint64_t k) {
    if (k > n - pos) throw std::runtime_error(std::string(kErr) + "file is truncated or corrupted");
  }
  template <typename T>
  T pod() {
    need(sizeof(T));
    T v;
    std::memcpy(&v, p + pos, sizeof(T));
    pos += sizeof(T);
    return v;
  }
  std::string str() {
    const uint64_t k = pod<uint64_t>();
    need(k);
    std::string s(reinterpret_cast<const char *>(p + pos), k);
    pos += k;
    return s;
  }
  std::vector<uint32_t> u32vec() {
    const uint64_t k = pod<uint64_t>();
    if (k > (n - pos) / 4) need(UINT64_MAX);
    std::vector<uint32_t> v(k);
    std::memcpy(v.data(), p + pos, k * 4);
    pos += k * 4;
    return v;
  }
  Block block() {
    Block b;
    b.original_size = pod<uint64_t>();
    const uint64_t k = pod<uint64_t>();
    need(k);
    b.payload.assign(p + pos, p + pos + k);
    pos += k;
    return b;
  }
  CompressedOptColumn opt() {
    CompressedOptColumn c;
    c.tag = str();
    c.type = pod<char>();
    c.num_elements = pod<uint64_t>();
    for (Block *b : {&c.ints, &c.floats, &c.chars, &c.strings, &c.string_lengths, &c.b_subtypes, &c.b_lengths,
                     &c.b_bytes})
      *b = block();
    return c;
  }
};

}  // namespace

std::vector<uint8_t> serialize_bytes(const Compressed &d) {
  Writer w;
  w.pod<uint32_t>(kGfazMagic);
  w.pod<uint32_t>(kGfazVersion);
  w.str(d.header_line);
  w.pod<uint64_t>(d.layers.size());
  for (const auto &r : d.layers) {
    w.pod<int32_t>(r.k);
    w.pod<uint32_t>(r.start_id);
    w.pod<uint32_t>(r.end_id);
    w.pod<uint64_t>(r.flattened_offset);
    w.pod<uint64_t>(r.element_count);
  }
  w.u32vec(d.sequence_lengths);
  w.u32vec(d.original_path_lengths);
  w.block(d.rules_first);
  w.block(d.rules_second);
  w.block(d.paths);
  w.pod<int32_t>(d.delta_round);
  w.block(d.names);
  w.block(d.name_lengths);
  w.block(d.overlaps);
  w.block(d.overlap_lengths);
  w.block(d.segment_sequences);
  w.block(d.segment_seq_lengths);
  w.pod<uint64_t>(d.segment_optional.size());
  for (const auto &c : d.segment_optional) w.opt(c);
  w.block(d.link_from_ids);
  w.block(d.link_to_ids);
  w.block(d.link_from_orients);
  w.block(d.link_to_orients);
  w.block(d.link_overlap_nums);
  w.block(d.link_overlap_ops);
  w.pod<uint64_t>(d.num_links);
  w.pod<uint64_t>(d.link_optional.size());
  for (const auto &c : d.link_optional) w.opt(c);
  w.pod<uint64_t>(d.num_jumps);
  for (const Block *b : {&d.jump_from_ids, &d.jump_from_orients, &d.jump_to_ids, &d.jump_to_orients,
                         &d.jump_distances, &d.jump_distance_lengths, &d.jump_rest_fields, &d.jump_rest_lengths})
    w.block(*b);
  w.pod<uint64_t>(d.num_containments);
  for (const Block *b :
       {&d.containment_container_ids, &d.containment_container_orients, &d.containment_contained_ids,
        &d.containment_contained_orients, &d.containment_positions, &d.containment_overlaps,
        &d.containment_overlap_lengths, &d.containment_rest_fields, &d.containment_rest_lengths})
    w.block(*b);
  w.u32vec(d.walk_lengths);
  w.u32vec(d.original_walk_lengths);
  for (const Block *b : {&d.walks, &d.walk_sample_ids, &d.walk_sample_id_lengths, &d.walk_hap_indices,
                         &d.walk_seq_ids, &d.walk_seq_id_lengths, &d.walk_seq_starts, &d.walk_seq_ends})
    w.block(*b);
  return std::move(w.out);
}

void serialize(const Compressed &d, const std::string &path) {
  std::ofstream out(path, std::ios::binary);
  if (!out) throw std::runtime_error(std::string(kErr) + "failed to open output file: " + path);
  const std::vector<uint8_t> bytes = serialize_bytes(d);
  out.write(reinterpret_cast<const char *>(bytes.data()), (std::streamsize)bytes.size());
  if (!out) throw std::runtime_error(std::string(kErr) + "failed to write output file: " + path);
}

Compressed deserialize_bytes(const uint8_t *data, size_t n) {
  Reader r{data, n};
  if (n < 4 || r.pod<uint32_t>() != kGfazMagic)
    throw std::runtime_error(std::string(kErr) + "invalid file format (magic mismatch)");
  const uint32_t version = r.pod<uint32_t>();
  if (version != kGfazVersion)
    throw std::runtime_error(std::string(kErr) + "unsupported file version " + std::to_string(version) +
                             " (expected " + std::to_string(kGfazVersion) + ")");
  Compressed d;
  d.header_line = r.str();
  const uint64_t nl = r.pod<uint64_t>();
  if (nl > (n - r.pos) / 28) r.need(UINT64_MAX);
  for (uint64_t i = 0; i < nl; ++i) {
    LayerRange l;
    l.k = r.pod<int32_t>();
    l.start_id = r.pod<uint32_t>();
    l.end_id = r.pod<uint32_t>();
    l.flattened_offset = r.pod<uint64_t>();
    l.element_count = r.pod<uint64_t>();
    d.layers.push_back(l);
  }
  d.sequence_lengths = r.u32vec();
  d.original_path_lengths = r.u32vec();
  d.rules_first = r.block();
  d.rules_second = r.block();
  d.paths = r.block();
  d.delta_round = r.pod<int32_t>();
  if (d.delta_round < 0) {
    std::cerr << "Warning: serialized delta_round=" << d.delta_round << " is invalid, clamping to 0" << std::endl;
    d.delta_round = 0;
  }
  d.names = r.block();
  d.name_lengths = r.block();
  d.overlaps = r.block();
  d.overlap_lengths = r.block();
  d.segment_sequences = r.block();
  d.segment_seq_lengths = r.block();
  const uint64_t so = r.pod<uint64_t>();
  for (uint64_t i = 0; i < so; ++i) d.segment_optional.push_back(r.opt());
  d.link_from_ids = r.block();
  d.link_to_ids = r.block();
  d.link_from_orients = r.block();
  d.link_to_orients = r.block();
  d.link_overlap_nums = r.block();
  d.link_overlap_ops = r.block();
  d.num_links = r.pod<uint64_t>();
  const uint64_t lo = r.pod<uint64_t>();
  for (uint64_t i = 0; i < lo; ++i) d.link_optional.push_back(r.opt());
  d.num_jumps = r.pod<uint64_t>();
  for (Block *b : {&d.jump_from_ids, &d.jump_from_orients, &d.jump_to_ids, &d.jump_to_orients, &d.jump_distances,
                   &d.jump_distance_lengths, &d.jump_rest_fields, &d.jump_rest_lengths})
    *b = r.block();
  d.num_containments = r.pod<uint64_t>();
  for (Block *b : {&d.containment_container_ids, &d.containment_container_orients, &d.containment_contained_ids,
                   &d.containment_contained_orients, &d.containment_positions, &d.containment_overlaps,
                   &d.containment_overlap_lengths, &d.containment_rest_fields, &d.containment_rest_lengths})
    *b = r.block();
  d.walk_lengths = r.u32vec();
  d.original_walk_lengths = r.u32vec();
  for (Block *b : {&d.walks, &d.walk_sample_ids, &d.walk_sample_id_lengths, &d.walk_hap_indices, &d.walk_seq_ids,
                   &d.walk_seq_id_lengths, &d.walk_seq_starts, &d.walk_seq_ends})
    *b = r.block();
  return d;
}

Compressed deserialize(const std::string &path) {
  std::ifstream in(path, std::ios::binary | std::ios::ate);
  if (!in) throw std::runtime_error(std::string(kErr) + "failed to open input file: " + path);
  const std::streamsize n = in.tellg();
  in.seekg(0);
  std::vector<uint8_t> buf((size_t)std::max<std::streamsize>(n, 0));
  if (n > 0 && !in.read(reinterpret_cast<char *>(buf.data()), n))
    throw std::runtime_error(std::string(kErr) + "failed to read input file: " + path);
  return deserialize_bytes(buf.data(), buf.size());
}

}  // namespace gfz

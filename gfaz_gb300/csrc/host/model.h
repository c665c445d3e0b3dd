// In-memory model of the .gfaz container and of a parsed GFA graph.
//
// The container layout mirrors the reference's CompressedData
// (include/model/compressed_data.hpp:40-120) field for field, because the
// serialized byte stream (src/codec/serialization.cpp:137-236) must be
// identical.  The parsed graph keeps P and W traversals flattened (one int32
// stream + u64 offsets per kind) so they can be uploaded to the GPU as is.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "codec.h"

namespace gfz {

constexpr uint32_t kGfazMagic = 0x5A414647;  // "GFAZ"
constexpr uint32_t kGfazVersion = 5;

struct LayerRange {
  int32_t k = 2;
  uint32_t start_id = 0, end_id = 0;
  uint64_t flattened_offset = 0, element_count = 0;
};

struct CompressedOptColumn {
  std::string tag;
  char type = '\0';
  uint64_t num_elements = 0;
  Block ints, floats, chars, strings, string_lengths, b_subtypes, b_lengths, b_bytes;
};

struct Compressed {
  std::string header_line;
  std::vector<LayerRange> layers;
  Block rules_first, rules_second;
  int32_t delta_round = 1;

  std::vector<uint32_t> sequence_lengths, original_path_lengths;
  Block paths, names, name_lengths, overlaps, overlap_lengths;

  Block segment_sequences, segment_seq_lengths;
  std::vector<CompressedOptColumn> segment_optional;

  uint64_t num_links = 0;
  Block link_from_ids, link_to_ids, link_from_orients, link_to_orients, link_overlap_nums, link_overlap_ops;
  std::vector<CompressedOptColumn> link_optional;

  uint64_t num_jumps = 0;
  Block jump_from_ids, jump_from_orients, jump_to_ids, jump_to_orients, jump_distances, jump_distance_lengths,
      jump_rest_fields, jump_rest_lengths;

  uint64_t num_containments = 0;
  Block containment_container_ids, containment_container_orients, containment_contained_ids,
      containment_contained_orients, containment_positions, containment_overlaps, containment_overlap_lengths,
      containment_rest_fields, containment_rest_lengths;

  std::vector<uint32_t> walk_lengths, original_walk_lengths;
  Block walks, walk_sample_ids, walk_sample_id_lengths, walk_hap_indices, walk_seq_ids, walk_seq_id_lengths,
      walk_seq_starts, walk_seq_ends;

  uint32_t min_rule_id() const { return layers.empty() ? 0 : layers[0].start_id; }
  uint64_t total_rules() const {
    uint64_t c = 0;
    for (const auto &l : layers) c += (uint64_t)(l.end_id - l.start_id);
    return c;
  }
};

// Optional-field column (SAM-style types i, f, A, Z, J, H, B).
struct OptColumn {
  std::string tag;
  char type = '\0';
  std::vector<int64_t> ints;
  std::vector<float> floats;
  std::vector<char> chars;
  std::string strings;
  std::vector<uint32_t> string_lengths;
  std::vector<char> b_subtypes;
  std::vector<uint32_t> b_lengths;
  std::vector<uint8_t> b_bytes;
};

struct Traversals {
  std::vector<int32_t> steps;    // signed 1-based node ids, back to back
  std::vector<uint64_t> offsets; // size() + 1 entries
  uint64_t size() const { return offsets.empty() ? 0 : offsets.size() - 1; }
};

struct Graph {
  std::string header_line;
  // segments: index 0 is a placeholder so node ids are 1-based
  std::vector<std::string> node_names;
  std::vector<std::string> node_sequences;
  std::vector<OptColumn> segment_optional;

  Traversals paths;
  std::vector<std::string> path_names, path_overlaps;

  Traversals walks;
  std::vector<std::string> walk_sample_ids, walk_seq_ids;
  std::vector<uint32_t> walk_hap_indices;
  std::vector<int64_t> walk_seq_starts, walk_seq_ends;

  std::vector<uint32_t> link_from, link_to, link_overlap_nums;
  std::vector<char> link_from_orients, link_to_orients, link_overlap_ops;
  std::vector<OptColumn> link_optional;

  std::vector<uint32_t> jump_from, jump_to;
  std::vector<char> jump_from_orients, jump_to_orients;
  std::vector<std::string> jump_distances, jump_rest;

  std::vector<uint32_t> cont_container, cont_contained, cont_positions;
  std::vector<char> cont_container_orients, cont_contained_orients;
  std::vector<std::string> cont_overlaps, cont_rest;

  uint64_t num_segments() const { return node_sequences.empty() ? 0 : node_sequences.size() - 1; }
};

// .gfaz v5 reader / writer (errors prefixed "GFAZ serialization error: ").
void serialize(const Compressed &c, const std::string &path);
std::vector<uint8_t> serialize_bytes(const Compressed &c);
Compressed deserialize(const std::string &path);
Compressed deserialize_bytes(const uint8_t *data, size_t n);

// GFA v1 parser (errors prefixed "GFA parser error: ").
Graph parse_gfa(const std::string &path, int threads);

}  // namespace gfz

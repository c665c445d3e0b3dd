// GFA v1 front end (host).  Produces the Graph model with P and W
// traversals flattened for the GPU.
//
// Behaviour follows the reference parser (src/io/gfa_parser.cpp):
//  * lines are split on '\n' only and classified by their first byte
//    (:353-404); the last H line is the header;
//  * fields are separated by runs of spaces/tabs (next_field, :124-131);
//  * S lines are read in order and assign 1-based ids in first-seen order;
//    when every segment name is the decimal form of its id, names resolve
//    by parsing the number, otherwise through the name table (:268-307,
//    :881-890); unresolved names give id 0 and the step/line is dropped;
//  * optional fields TAG:T:VALUE become typed columns padded with
//    sentinels (INT64_MIN, -FLT_MAX, '\0', empty) (:463-630);
//  * P steps are comma-separated name+orientation, W steps '>'/'<'
//    prefixed names; W start/end '*' -> -1 (:347-461);
//  * J and C lines keep their distance / overlap strings and the rest of
//    the line re-joined with tabs (:807-879).
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string_view>
#include <unordered_map>

#include "model.h"

namespace gfz {

namespace {

constexpr const char *kErr = "GFA parser error: ";
constexpr const char *kWarn = "GFA parser warning: ";

int64_t parse_i64(std::string_view s) {
  if (s.empty()) throw std::invalid_argument("parse_int64: empty");
  size_t i = 0;
  const bool neg = s[0] == '-';
  if (neg) i = 1;
  if (i >= s.size()) throw std::invalid_argument("parse_int64: no digits");
  // accumulate toward the sign so INT64_MIN is representable
  const int64_t lim = neg ? std::numeric_limits<int64_t>::min() : std::numeric_limits<int64_t>::max();
  const int64_t cut = lim / 10;
  const int cutlim = neg ? -(int)(lim % 10) : (int)(lim % 10);
  int64_t v = 0;
  for (; i < s.size(); ++i) {
    const char c = s[i];
    if (c < '0' || c > '9') break;
    const int d = c - '0';
    if (!neg) {
      if (v > cut || (v == cut && d > cutlim)) throw std::out_of_range("parse_int64: overflow");
      v = v * 10 + d;
    } else {
      if (v < cut || (v == cut && d > cutlim)) throw std::out_of_range("parse_int64: overflow");
      v = v * 10 - d;
    }
  }
  return v;
}

uint32_t parse_u32(std::string_view s) {
  if (s.empty()) throw std::invalid_argument("parse_uint32: empty");
  uint32_t v = 0;
  bool any = false;
  const uint32_t cut = std::numeric_limits<uint32_t>::max() / 10, cutlim = std::numeric_limits<uint32_t>::max() % 10;
  for (char c : s) {
    if (c < '0' || c > '9') break;
    any = true;
    const uint32_t d = (uint32_t)(c - '0');
    if (v > cut || (v == cut && d > cutlim)) throw std::out_of_range("parse_uint32: overflow");
    v = v * 10 + d;
  }
  if (!any) throw std::invalid_argument("parse_uint32: no digits");
  return v;
}

float parse_f32(std::string_view s) {
  if (s.empty()) throw std::invalid_argument("parse_float: empty");
  std::string tmp(s);
  errno = 0;
  char *end = nullptr;
  const float v = std::strtof(tmp.c_str(), &end);
  if (end == tmp.c_str()) throw std::invalid_argument("parse_float: no digits");
  if (errno == ERANGE) throw std::out_of_range("parse_float: overflow");
  return v;
}

inline std::string_view next_field(std::string_view line, size_t &pos) {
  while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
  const size_t b = pos;
  while (pos < line.size() && line[pos] != ' ' && line[pos] != '\t') ++pos;
  return line.substr(b, pos - b);
}

bool all_digits(std::string_view s) {
  if (s.empty()) return false;
  for (char c : s)
    if (c < '0' || c > '9') return false;
  return true;
}

uint32_t overlap_number(std::string_view v, char &op) {
  uint32_t num = 0;
  size_t i = 0;
  while (i < v.size() && v[i] >= '0' && v[i] <= '9') {
    num = num * 10 + (uint32_t)(v[i] - '0');
    ++i;
  }
  op = i < v.size() ? v[i] : '\0';
  return num;
}

size_t b_elem_size(char sub) {
  switch (sub) {
    case 'c': case 'C': return 1;
    case 's': case 'S': return 2;
    case 'i': case 'I': case 'f': return 4;
    default: return 0;
  }
}

void pad_column(OptColumn &c, size_t n) {
  switch (c.type) {
    case 'i': while (c.ints.size() < n) c.ints.push_back(std::numeric_limits<int64_t>::min()); break;
    case 'f': while (c.floats.size() < n) c.floats.push_back(std::numeric_limits<float>::lowest()); break;
    case 'A': while (c.chars.size() < n) c.chars.push_back('\0'); break;
    case 'Z': case 'J': case 'H': while (c.string_lengths.size() < n) c.string_lengths.push_back(0); break;
    case 'B':
      while (c.b_subtypes.size() < n) {
        c.b_subtypes.push_back('\0');
        c.b_lengths.push_back(0);
      }
      break;
  }
}

// One optional-field column set (segments or links) with tag lookup.
struct OptSet {
  std::vector<OptColumn> *cols;
  std::unordered_map<uint16_t, std::pair<char, size_t>> meta;
  const char *kind;  // "" or "link "

  void add(std::string_view f, size_t index) {
    if (f.size() < 5 || f[2] != ':' || f[4] != ':') return;
    const uint16_t key = (uint16_t)(((unsigned char)f[0] << 8) | (unsigned char)f[1]);
    const char type = f[3];
    const std::string_view val = f.substr(5);
    auto it = meta.find(key);
    if (it == meta.end()) {
      meta[key] = {type, cols->size()};
      OptColumn c;
      c.tag = std::string(f.substr(0, 2));
      c.type = type;
      cols->push_back(std::move(c));
      it = meta.find(key);
    }
    OptColumn &c = (*cols)[it->second.second];
    if (type != it->second.first)
      throw std::runtime_error(std::string("Type mismatch for ") + kind + "tag '" + c.tag + "': expected '" +
                               std::string(1, it->second.first) + "', got '" + std::string(1, type) + "'");
    switch (type) {
      case 'i':
        while (c.ints.size() < index) c.ints.push_back(std::numeric_limits<int64_t>::min());
        c.ints.push_back(parse_i64(val));
        break;
      case 'f':
        while (c.floats.size() < index) c.floats.push_back(std::numeric_limits<float>::lowest());
        c.floats.push_back(parse_f32(val));
        break;
      case 'A':
        while (c.chars.size() < index) c.chars.push_back('\0');
        c.chars.push_back(val.empty() ? '\0' : val[0]);
        break;
      case 'Z': case 'J': case 'H':
        while (c.string_lengths.size() < index) c.string_lengths.push_back(0);
        c.strings.append(val.data(), val.size());
        c.string_lengths.push_back((uint32_t)val.size());
        break;
      case 'B': {
        while (c.b_subtypes.size() < index) {
          c.b_subtypes.push_back('\0');
          c.b_lengths.push_back(0);
        }
        if (val.size() < 2 || val[1] != ',') {
          c.b_subtypes.push_back('\0');
          c.b_lengths.push_back(0);
          break;
        }
        const char sub = val[0];
        c.b_subtypes.push_back(sub);
        if (b_elem_size(sub) == 0) {
          c.b_lengths.push_back(0);
          break;
        }
        std::vector<uint8_t> bytes;
        uint32_t count = 0;
        std::istringstream ss{std::string(val.substr(2))};
        std::string tok;
        auto put = [&bytes](const void *p, size_t k) {
          const uint8_t *b = static_cast<const uint8_t *>(p);
          bytes.insert(bytes.end(), b, b + k);
        };
        while (std::getline(ss, tok, ',')) {
          if (tok.empty()) continue;
          count++;
          if (sub == 'f') { float v = parse_f32(tok); put(&v, 4); }
          else if (sub == 'c') { int8_t v = (int8_t)parse_i64(tok); put(&v, 1); }
          else if (sub == 'C') { uint8_t v = (uint8_t)parse_u32(tok); put(&v, 1); }
          else if (sub == 's') { int16_t v = (int16_t)parse_i64(tok); put(&v, 2); }
          else if (sub == 'S') { uint16_t v = (uint16_t)parse_u32(tok); put(&v, 2); }
          else if (sub == 'i') { int32_t v = (int32_t)parse_i64(tok); put(&v, 4); }
          else if (sub == 'I') { uint32_t v = parse_u32(tok); put(&v, 4); }
        }
        c.b_lengths.push_back(count);
        c.b_bytes.insert(c.b_bytes.end(), bytes.begin(), bytes.end());
        break;
      }
      default:
        std::cerr << kWarn << "unsupported " << kind << "optional field type '" << type << "' for tag '" << c.tag
                  << "'" << std::endl;
    }
  }
};

struct Mapped {
  const char *data = nullptr;
  size_t size = 0;
  int fd = -1;
  ~Mapped() {
    if (data && size) munmap(const_cast<char *>(data), size);
    if (fd >= 0) close(fd);
  }
};

struct Line {
  size_t off, len;
};

}  // namespace

Graph parse_gfa(const std::string &path, int threads) {
  Graph g;
  g.node_names.emplace_back();
  g.node_sequences.emplace_back();
  Mapped m;
  m.fd = open(path.c_str(), O_RDONLY);
  if (m.fd < 0)
    throw std::runtime_error(std::string(kErr) + "failed to open input file '" + path + "': " + std::strerror(errno));
  struct stat sb;
  if (fstat(m.fd, &sb) != 0)
    throw std::runtime_error(std::string(kErr) + "failed to stat input file '" + path + "': " + std::strerror(errno));
  m.size = (size_t)sb.st_size;
  if (m.size) {
    void *p = mmap(nullptr, m.size, PROT_READ, MAP_PRIVATE, m.fd, 0);
    if (p == MAP_FAILED)
      throw std::runtime_error(std::string(kErr) + "failed to mmap input file '" + path + "': " + std::strerror(errno));
    m.data = static_cast<const char *>(p);
    madvise(p, m.size, MADV_SEQUENTIAL);
  }
  const char *d = m.data;
  std::vector<Line> S, L, P, W, J, C;
  size_t start = 0;
  for (size_t i = 0; i <= m.size; ++i) {
    if (i == m.size || d[i] == '\n') {
      const size_t len = i - start;
      if (len > 0) {
        switch (d[start]) {
          case 'S': S.push_back({start, len}); break;
          case 'H': g.header_line.assign(d + start, len); break;
          case 'L': L.push_back({start, len}); break;
          case 'P': P.push_back({start, len}); break;
          case 'W': W.push_back({start, len}); break;
          case 'J': J.push_back({start, len}); break;
          case 'C': C.push_back({start, len}); break;
          default: break;
        }
      }
      start = i + 1;
    }
  }

  // S lines: sequential, assigning ids in first-seen order
  std::unordered_map<std::string_view, uint32_t> lookup;
  lookup.reserve(S.size());
  bool numeric = true;
  g.node_names.reserve(S.size() + 1);
  g.node_sequences.reserve(S.size() + 1);
  OptSet seg_opt{&g.segment_optional, {}, ""};
  for (const Line &ln : S) {
    const std::string_view line(d + ln.off, ln.len);
    size_t pos = 1;
    const std::string_view name = next_field(line, pos);
    const std::string_view seq = next_field(line, pos);
    size_t index;
    auto it = lookup.find(name);
    if (it == lookup.end()) {
      if (numeric && !all_digits(name)) numeric = false;
      const uint32_t id = (uint32_t)g.node_names.size();
      if (numeric && parse_u32(name) != id) numeric = false;
      g.node_names.emplace_back(name);
      g.node_sequences.emplace_back(seq);
      // names stay valid: they point into the mapped file
      lookup.emplace(name, id);
      index = id - 1;
    } else {
      index = it->second - 1;
    }
    while (pos < line.size()) {
      const std::string_view f = next_field(line, pos);
      if (f.empty()) break;
      seg_opt.add(f, index);
    }
  }
  const size_t nseg = g.node_names.size() - 1;
  for (auto &c : g.segment_optional) pad_column(c, nseg);

  auto resolve = [&](std::string_view name) -> uint32_t {
    if (name.empty()) return 0;
    if (numeric) return parse_u32(name);
    auto it = lookup.find(name);
    return it == lookup.end() ? 0 : it->second;
  };

  // L lines
  OptSet link_opt{&g.link_optional, {}, "link "};
  for (const Line &ln : L) {
    const std::string_view line(d + ln.off, ln.len);
    size_t pos = 1;
    const std::string_view fn = next_field(line, pos), fo = next_field(line, pos);
    const std::string_view tn = next_field(line, pos), to = next_field(line, pos);
    const std::string_view ov = next_field(line, pos);
    const uint32_t a = resolve(fn), b = resolve(tn);
    if (a == 0 || b == 0) continue;
    g.link_from.push_back(a);
    g.link_to.push_back(b);
    g.link_from_orients.push_back(fo.empty() ? '+' : fo[0]);
    g.link_to_orients.push_back(to.empty() ? '+' : to[0]);
    if (ov.empty() || ov == "*") {
      g.link_overlap_nums.push_back(0);
      g.link_overlap_ops.push_back('\0');
    } else {
      char op;
      g.link_overlap_nums.push_back(overlap_number(ov, op));
      g.link_overlap_ops.push_back(op);
    }
    const size_t li = g.link_from.size() - 1;
    while (pos < line.size()) {
      const std::string_view f = next_field(line, pos);
      if (f.empty()) break;
      link_opt.add(f, li);
    }
  }
  for (auto &c : g.link_optional) pad_column(c, g.link_from.size());

  // P / W lines in parallel, one vector per line, then flattened
  std::vector<std::vector<int32_t>> ptrav(P.size()), wtrav(W.size());
  g.path_names.resize(P.size());
  g.path_overlaps.resize(P.size());
  g.walk_sample_ids.resize(W.size());
  g.walk_seq_ids.resize(W.size());
  g.walk_hap_indices.resize(W.size());
  g.walk_seq_starts.resize(W.size());
  g.walk_seq_ends.resize(W.size());
  const int nth = resolve_threads(threads);
  std::string first_error;
  bool failed = false;
#pragma omp parallel for schedule(dynamic) num_threads(nth)
  for (int64_t i = 0; i < (int64_t)P.size(); ++i) {
    try {
      const std::string_view line(d + P[i].off, P[i].len);
      size_t pos = 1;
      while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
      size_t b = pos;
      while (pos < line.size() && line[pos] != ' ' && line[pos] != '\t') ++pos;
      g.path_names[i].assign(line.substr(b, pos - b));
      while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
      b = pos;
      while (pos < line.size() && line[pos] != ' ' && line[pos] != '\t') ++pos;
      const std::string_view steps = line.substr(b, pos - b);
      while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
      g.path_overlaps[i].assign(line.substr(pos));
      std::vector<int32_t> &out = ptrav[i];
      size_t commas = 0;
      for (char c : steps) commas += c == ',';
      out.reserve(commas + 1);
      size_t s0 = 0;
      for (size_t k = 0; k <= steps.size(); ++k) {
        if (k == steps.size() || steps[k] == ',') {
          if (k > s0) {
            const std::string_view tok = steps.substr(s0, k - s0);
            const char o = tok.back();
            const uint32_t id = resolve(tok.substr(0, tok.size() - 1));
            if (id != 0) out.push_back(o == '-' ? -(int32_t)id : (int32_t)id);
          }
          s0 = k + 1;
        }
      }
    } catch (const std::exception &e) {
#pragma omp critical
      {
        if (!failed) first_error = e.what();
        failed = true;
      }
    }
  }
#pragma omp parallel for schedule(dynamic) num_threads(nth)
  for (int64_t i = 0; i < (int64_t)W.size(); ++i) {
    try {
      const std::string_view line(d + W[i].off, W[i].len);
      size_t pos = 1;
      const std::string_view sample = next_field(line, pos), hap = next_field(line, pos);
      const std::string_view seqid = next_field(line, pos), st = next_field(line, pos);
      const std::string_view en = next_field(line, pos), walk = next_field(line, pos);
      std::vector<int32_t> &out = wtrav[i];
      size_t nsteps = 0;
      for (char c : walk) nsteps += (c == '>' || c == '<');
      out.reserve(nsteps);
      size_t p = 0;
      while (p < walk.size()) {
        const char o = walk[p];
        if (o != '>' && o != '<') {
          ++p;
          continue;
        }
        size_t e = p + 1;
        while (e < walk.size() && walk[e] != '>' && walk[e] != '<') ++e;
        if (e > p + 1) {
          const uint32_t id = resolve(walk.substr(p + 1, e - p - 1));
          if (id != 0) out.push_back(o == '<' ? -(int32_t)id : (int32_t)id);
        }
        p = e;
      }
      g.walk_sample_ids[i].assign(sample);
      uint32_t h = 0;
      for (char c : hap) h = h * 10 + (uint32_t)(c - '0');
      g.walk_hap_indices[i] = h;
      g.walk_seq_ids[i].assign(seqid);
      g.walk_seq_starts[i] = st == "*" ? -1 : parse_i64(st);
      g.walk_seq_ends[i] = en == "*" ? -1 : parse_i64(en);
    } catch (const std::exception &e) {
#pragma omp critical
      {
        if (!failed) first_error = e.what();
        failed = true;
      }
    }
  }
  if (failed) throw std::runtime_error(first_error);
  auto flatten = [](std::vector<std::vector<int32_t>> &v, Traversals &t) {
    t.offsets.assign(v.size() + 1, 0);
    for (size_t i = 0; i < v.size(); ++i) t.offsets[i + 1] = t.offsets[i] + v[i].size();
    t.steps.resize(t.offsets.back());
    for (size_t i = 0; i < v.size(); ++i) {
      std::copy(v[i].begin(), v[i].end(), t.steps.begin() + (ptrdiff_t)t.offsets[i]);
      std::vector<int32_t>().swap(v[i]);
    }
  };
  flatten(ptrav, g.paths);
  flatten(wtrav, g.walks);

  // J / C lines
  for (const Line &ln : J) {
    const std::string_view line(d + ln.off, ln.len);
    size_t pos = 1;
    const std::string_view fn = next_field(line, pos), fo = next_field(line, pos);
    const std::string_view tn = next_field(line, pos), to = next_field(line, pos);
    const std::string_view dist = next_field(line, pos);
    const uint32_t a = resolve(fn), b = resolve(tn);
    if (a == 0 || b == 0) continue;
    g.jump_from.push_back(a);
    g.jump_from_orients.push_back(fo.empty() ? '+' : fo[0]);
    g.jump_to.push_back(b);
    g.jump_to_orients.push_back(to.empty() ? '+' : to[0]);
    g.jump_distances.emplace_back(dist);
    std::string rest;
    while (pos < line.size()) {
      const std::string_view f = next_field(line, pos);
      if (f.empty()) break;
      if (!rest.empty()) rest += '\t';
      rest.append(f.data(), f.size());
    }
    g.jump_rest.push_back(std::move(rest));
  }
  for (const Line &ln : C) {
    const std::string_view line(d + ln.off, ln.len);
    size_t pos = 1;
    const std::string_view cn = next_field(line, pos), co = next_field(line, pos);
    const std::string_view tn = next_field(line, pos), to = next_field(line, pos);
    const std::string_view ps = next_field(line, pos), ov = next_field(line, pos);
    const uint32_t a = resolve(cn), b = resolve(tn);
    if (a == 0 || b == 0) continue;
    g.cont_container.push_back(a);
    g.cont_container_orients.push_back(co.empty() ? '+' : co[0]);
    g.cont_contained.push_back(b);
    g.cont_contained_orients.push_back(to.empty() ? '+' : to[0]);
    g.cont_positions.push_back(parse_u32(ps));
    g.cont_overlaps.emplace_back(ov);
    std::string rest;
    while (pos < line.size()) {
      const std::string_view f = next_field(line, pos);
      if (f.empty()) break;
      if (!rest.empty()) rest += '\t';
      rest.append(f.data(), f.size());
    }
    g.cont_rest.push_back(std::move(rest));
  }
  return g;
}

}  // namespace gfz

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

#include <array>
#include <cerrno>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string_view>
#include <unordered_map>

#include "codec.h"
#include "model.h"
#include "workflows.h"

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
  Mapped() = default;
  Mapped(const Mapped &) = delete;
  Mapped &operator=(const Mapped &) = delete;
  Mapped(Mapped &&o) noexcept : data(o.data), size(o.size), fd(o.fd) {
    o.data = nullptr;
    o.size = 0;
    o.fd = -1;
  }
  ~Mapped() {
    if (data && size) munmap(const_cast<char *>(data), size);
    if (fd >= 0) close(fd);
  }
};

struct Line {
  size_t off, len;
};

Mapped map_file(const std::string &path) {
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
  return m;
}

// Lines by record type, in file order.
struct Lines {
  std::vector<Line> S, L, P, W, J, C;
  void add(const char *d, size_t start, size_t len, Graph &g) {
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
};

void scan_lines(const char *d, size_t n, Lines &ls, Graph &g) {
  size_t start = 0;
  while (start < n) {
    const void *nl = std::memchr(d + start, '\n', n - start);
    const size_t end = nl ? (size_t)(static_cast<const char *>(nl) - d) : n;
    if (end > start) ls.add(d, start, end - start, g);
    start = end + 1;
  }
}

// Segment names: numeric (every name the decimal form of its id) or the
// name table built from the S lines.
struct Names {
  std::unordered_map<std::string_view, uint32_t> lookup;
  std::vector<std::string_view> by_id;  // 1-based; filled when not numeric
  bool numeric = true;
  uint32_t resolve(std::string_view name) const {
    if (name.empty()) return 0;
    if (numeric) return parse_u32(name);
    auto it = lookup.find(name);
    return it == lookup.end() ? 0 : it->second;
  }
};

// S lines, assigning ids in first-seen order.  When the i-th S line is
// named i + 1 for every i (the common numeric layout: no duplicate can
// occur and every id equals its name), the lines are read in parallel;
// otherwise in order with the name table.
void parse_segments(const char *d, const std::vector<Line> &S, Graph &g, Names &nm, int threads) {
  OptSet seg_opt{&g.segment_optional, {}, ""};
  const int64_t ns = (int64_t)S.size();
  const int nth = resolve_threads(threads);
  std::vector<uint8_t> plain(ns, 0);
  std::vector<uint32_t> rest(ns, 0);  // offset of the optional fields in the line (0: none)
  bool simple = true;
#pragma omp parallel for schedule(static) num_threads(nth) reduction(&& : simple)
  for (int64_t i = 0; i < ns; ++i) {
    const std::string_view line(d + S[i].off, S[i].len);
    size_t pos = 1;
    const std::string_view name = next_field(line, pos);
    next_field(line, pos);
    while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
    rest[i] = pos < line.size() ? (uint32_t)std::min<size_t>(pos, UINT32_MAX) : 0;
    bool ok = all_digits(name) && name.size() <= 10;
    if (ok) {
      uint64_t v = 0;
      for (char c : name) v = v * 10 + (uint64_t)(c - '0');
      ok = v == (uint64_t)i + 1;
    }
    simple = simple && ok && (rest[i] == 0 || S[i].len <= UINT32_MAX);
  }
  if (simple) {
    g.node_names.resize(ns + 1);
    g.node_sequences.resize(ns + 1);
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int64_t i = 0; i < ns; ++i) {
      const std::string_view line(d + S[i].off, S[i].len);
      size_t pos = 1;
      g.node_names[i + 1].assign(next_field(line, pos));
      g.node_sequences[i + 1].assign(next_field(line, pos));
    }
    for (int64_t i = 0; i < ns; ++i) {
      if (!rest[i]) continue;
      const std::string_view line(d + S[i].off, S[i].len);
      size_t pos = rest[i];
      while (pos < line.size()) {
        const std::string_view f = next_field(line, pos);
        if (f.empty()) break;
        seg_opt.add(f, (size_t)i);
      }
    }
  } else {
    nm.lookup.reserve(S.size());
    g.node_names.reserve(S.size() + 1);
    g.node_sequences.reserve(S.size() + 1);
    nm.by_id.assign(1, std::string_view());
    for (const Line &ln : S) {
      const std::string_view line(d + ln.off, ln.len);
      size_t pos = 1;
      const std::string_view name = next_field(line, pos);
      const std::string_view seq = next_field(line, pos);
      size_t index;
      auto it = nm.lookup.find(name);
      if (it == nm.lookup.end()) {
        if (nm.numeric && !all_digits(name)) nm.numeric = false;
        const uint32_t id = (uint32_t)g.node_names.size();
        if (nm.numeric && parse_u32(name) != id) nm.numeric = false;
        g.node_names.emplace_back(name);
        g.node_sequences.emplace_back(seq);
        // names stay valid: they point into the mapped file
        nm.lookup.emplace(name, id);
        nm.by_id.push_back(name);
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
  }
  const size_t nseg = g.node_names.size() - 1;
  for (auto &c : g.segment_optional) pad_column(c, nseg);
}

// L lines.  The fields are read in parallel; the order-dependent work runs
// after, in line order: a line's name error is raised where the sequential
// parser would raise it (before that line's optional fields, after the
// optional fields of earlier lines), and optional-field columns are built
// in line order.
void parse_links(const char *d, const std::vector<Line> &L, const Names &nm, Graph &g, int threads) {
  OptSet link_opt{&g.link_optional, {}, "link "};
  const int64_t nl = (int64_t)L.size();
  struct Link {
    uint32_t a = 0, b = 0, num = 0;
    size_t rest = 0;  // offset of the optional fields in the line (0: none)
    char fo = '+', to = '+', op = '\0';
    bool err = false;
  };
  std::vector<Link> v(nl);
  std::vector<std::string> errs;
  std::vector<int64_t> err_at;
#pragma omp parallel for schedule(static) num_threads(resolve_threads(threads))
  for (int64_t i = 0; i < nl; ++i) {
    const std::string_view line(d + L[i].off, L[i].len);
    size_t pos = 1;
    const std::string_view fn = next_field(line, pos), fo = next_field(line, pos);
    const std::string_view tn = next_field(line, pos), to = next_field(line, pos);
    const std::string_view ov = next_field(line, pos);
    Link &k = v[i];
    try {
      k.a = nm.resolve(fn);
      k.b = nm.resolve(tn);
    } catch (const std::exception &e) {
      k.err = true;
#pragma omp critical
      {
        errs.emplace_back(e.what());
        err_at.push_back(i);
      }
      continue;
    }
    k.fo = fo.empty() ? '+' : fo[0];
    k.to = to.empty() ? '+' : to[0];
    if (!ov.empty() && ov != "*") k.num = overlap_number(ov, k.op);
    while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
    k.rest = pos < line.size() ? pos : 0;
  }
  int64_t first_err = nl;
  std::string first_msg;
  for (size_t e = 0; e < err_at.size(); ++e)
    if (err_at[e] < first_err) {
      first_err = err_at[e];
      first_msg = errs[e];
    }
  // kept links (both ends resolved), in order
  std::vector<uint64_t> at(nl + 1, 0);
  for (int64_t i = 0; i < nl; ++i) at[i + 1] = at[i] + (!v[i].err && v[i].a && v[i].b);
  // optional fields and the first error, in line order
  for (int64_t i = 0; i < nl; ++i) {
    if (i == first_err) throw std::runtime_error(first_msg);
    const Link &k = v[i];
    if (!k.a || !k.b || !k.rest) continue;
    const std::string_view line(d + L[i].off, L[i].len);
    size_t pos = k.rest;
    while (pos < line.size()) {
      const std::string_view f = next_field(line, pos);
      if (f.empty()) break;
      link_opt.add(f, at[i]);
    }
  }
  const uint64_t n = at[nl];
  g.link_from.resize(n);
  g.link_to.resize(n);
  g.link_from_orients.resize(n);
  g.link_to_orients.resize(n);
  g.link_overlap_nums.resize(n);
  g.link_overlap_ops.resize(n);
#pragma omp parallel for schedule(static) num_threads(resolve_threads(threads))
  for (int64_t i = 0; i < nl; ++i) {
    const Link &k = v[i];
    if (k.err || !k.a || !k.b) continue;
    const uint64_t j = at[i];
    g.link_from[j] = k.a;
    g.link_to[j] = k.b;
    g.link_from_orients[j] = k.fo;
    g.link_to_orients[j] = k.to;
    g.link_overlap_nums[j] = k.num;
    g.link_overlap_ops[j] = k.op;
  }
  for (auto &c : g.link_optional) pad_column(c, n);
}

// P line header: the name and, from the end of the steps field, the
// overlap (the rest of the line after the blanks that follow the steps).
void path_header(std::string_view line, size_t steps_end, Graph &g, size_t i) {
  size_t pos = 1;
  while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
  const size_t b = pos;
  while (pos < line.size() && line[pos] != ' ' && line[pos] != '\t') ++pos;
  g.path_names[i].assign(line.substr(b, pos - b));
  pos = steps_end;
  while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
  g.path_overlaps[i].assign(line.substr(pos));
}

// W line header fields (sample, hap, seq id, start, end); throws on a
// malformed start / end.
void walk_header(std::string_view line, Graph &g, size_t i) {
  size_t pos = 1;
  const std::string_view sample = next_field(line, pos), hap = next_field(line, pos);
  const std::string_view seqid = next_field(line, pos), st = next_field(line, pos);
  const std::string_view en = next_field(line, pos);
  g.walk_sample_ids[i].assign(sample);
  uint32_t h = 0;
  for (char c : hap) h = h * 10 + (uint32_t)(c - '0');
  g.walk_hap_indices[i] = h;
  g.walk_seq_ids[i].assign(seqid);
  g.walk_seq_starts[i] = st == "*" ? -1 : parse_i64(st);
  g.walk_seq_ends[i] = en == "*" ? -1 : parse_i64(en);
}

void size_traversals(Graph &g, size_t np, size_t nw) {
  g.path_names.resize(np);
  g.path_overlaps.resize(np);
  g.walk_sample_ids.resize(nw);
  g.walk_seq_ids.resize(nw);
  g.walk_hap_indices.resize(nw);
  g.walk_seq_starts.resize(nw);
  g.walk_seq_ends.resize(nw);
}

// P / W lines on the host, in parallel, one vector per line, then flattened.
void parse_traversals_host(const char *d, const Lines &ls, const Names &nm, int threads, Graph &g) {
  const std::vector<Line> &P = ls.P, &W = ls.W;
  std::vector<std::vector<int32_t>> ptrav(P.size()), wtrav(W.size());
  size_traversals(g, P.size(), W.size());
  const int nth = resolve_threads(threads);
  std::string first_error;
  bool failed = false;
#pragma omp parallel for schedule(dynamic) num_threads(nth)
  for (int64_t i = 0; i < (int64_t)P.size(); ++i) {
    try {
      const std::string_view line(d + P[i].off, P[i].len);
      size_t pos = 1;
      while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
      while (pos < line.size() && line[pos] != ' ' && line[pos] != '\t') ++pos;
      while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t')) ++pos;
      const size_t b = pos;
      while (pos < line.size() && line[pos] != ' ' && line[pos] != '\t') ++pos;
      const std::string_view steps = line.substr(b, pos - b);
      path_header(line, pos, g, (size_t)i);
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
            const uint32_t id = nm.resolve(tok.substr(0, tok.size() - 1));
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
      for (int f = 0; f < 5; ++f) next_field(line, pos);
      const std::string_view walk = next_field(line, pos);
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
          const uint32_t id = nm.resolve(walk.substr(p + 1, e - p - 1));
          if (id != 0) out.push_back(o == '<' ? -(int32_t)id : (int32_t)id);
        }
        p = e;
      }
      walk_header(line, g, (size_t)i);
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
}

void parse_jumps_containments(const char *d, const Lines &ls, const Names &nm, Graph &g) {
  for (const Line &ln : ls.J) {
    const std::string_view line(d + ln.off, ln.len);
    size_t pos = 1;
    const std::string_view fn = next_field(line, pos), fo = next_field(line, pos);
    const std::string_view tn = next_field(line, pos), to = next_field(line, pos);
    const std::string_view dist = next_field(line, pos);
    const uint32_t a = nm.resolve(fn), b = nm.resolve(tn);
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
  for (const Line &ln : ls.C) {
    const std::string_view line(d + ln.off, ln.len);
    size_t pos = 1;
    const std::string_view cn = next_field(line, pos), co = next_field(line, pos);
    const std::string_view tn = next_field(line, pos), to = next_field(line, pos);
    const std::string_view ps = next_field(line, pos), ov = next_field(line, pos);
    const uint32_t a = nm.resolve(cn), b = nm.resolve(tn);
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
}

Graph empty_graph() {
  Graph g;
  g.node_names.emplace_back();
  g.node_sequences.emplace_back();
  return g;
}

}  // namespace

Graph parse_gfa(const std::string &path, int threads) {
  Graph g = empty_graph();
  const Mapped m = map_file(path);
  const char *d = m.data;
  Lines ls;
  scan_lines(d, m.size, ls, g);
  Names nm;
  parse_segments(d, ls.S, g, nm, threads);
  parse_links(d, ls.L, nm, g, threads);
  parse_traversals_host(d, ls, nm, threads, g);
  parse_jumps_containments(d, ls, nm, g);
  return g;
}

// ---------------------------------------------------------------------------
// Device front end: the file in HBM; line index, P/W field bounds and step
// tokens on the GPU (parse_kernels.cu); S/L/J/C lines and the short P/W
// header fields on the host.  Same Graph as parse_gfa for every input,
// errors included (with one thread, parse_gfa reports the first P error,
// else the first W line's error, token errors before start/end errors).
// ---------------------------------------------------------------------------
namespace {

template <typename T>
T download_one(const T *p, cudaStream_t st) {
  T v;
  cuda_check(cudaMemcpyAsync(&v, p, sizeof(T), cudaMemcpyDeviceToHost, st), "download");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
  return v;
}

// One launch bracketed by the context's kernel timer (algorithmic bytes).
template <class F>
void timed(Context &ctx, const char *name, double bytes, F &&launch) {
  ctx.tbegin(name, bytes);
  launch();
  ctx.tend();
}

void scan_u32(Context &ctx, const uint32_t *in, uint64_t n, uint64_t *out) {
  exclusive_scan(ctx, in, n, out, "gfa_scan");
}


// Lines by type from the device line index (type[i], line ends eol), in
// parallel: per-thread counts, then each thread fills its share.  slot of
// a P/W line = its rank among the P and W lines.
void line_lists(const std::vector<uint8_t> &type, const std::vector<uint64_t> &eol, uint64_t nl, uint64_t n, int nth,
                Lines &ls, std::vector<uint64_t> &pslot, std::vector<uint64_t> &wslot) {
  const uint64_t nlines = type.size();
  auto kind_of = [](uint8_t t) -> int {
    switch (t) {
      case 'S': return 0;
      case 'L': return 1;
      case 'P': return 2;
      case 'W': return 3;
      case 'J': return 4;
      case 'C': return 5;
      default: return -1;
    }
  };
  std::vector<Line> *lists[6] = {&ls.S, &ls.L, &ls.P, &ls.W, &ls.J, &ls.C};
  const int T = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)nth, nlines / 65536 + 1));
  std::vector<std::array<uint64_t, 6>> cnt(T + 1);
  for (auto &c : cnt) c.fill(0);
#pragma omp parallel for schedule(static) num_threads(T)
  for (int t = 0; t < T; ++t) {
    const uint64_t a = nlines * t / T, b = nlines * (t + 1) / T;
    for (uint64_t i = a; i < b; ++i) {
      const int k = kind_of(type[i]);
      if (k >= 0) cnt[t + 1][k]++;
    }
  }
  for (int t = 0; t < T; ++t)
    for (int k = 0; k < 6; ++k) cnt[t + 1][k] += cnt[t][k];
  for (int k = 0; k < 6; ++k) lists[k]->resize(cnt[T][k]);
  pslot.resize(cnt[T][2]);
  wslot.resize(cnt[T][3]);
#pragma omp parallel for schedule(static) num_threads(T)
  for (int t = 0; t < T; ++t) {
    const uint64_t a = nlines * t / T, b = nlines * (t + 1) / T;
    std::array<uint64_t, 6> at = cnt[t];
    for (uint64_t i = a; i < b; ++i) {
      const int k = kind_of(type[i]);
      if (k < 0) continue;
      const uint64_t s = i ? eol[i - 1] + 1 : 0, e = i < nl ? eol[i] : n;
      if (k == 2) pslot[at[2]] = at[2] + at[3];
      if (k == 3) wslot[at[3]] = at[2] + at[3];
      (*lists[k])[at[k]++] = Line{(size_t)s, (size_t)(e - s)};
    }
  }
}

const char *token_error(uint32_t code) {
  return code == kParseOverflow ? "parse_uint32: overflow" : "parse_uint32: no digits";
}

}  // namespace

DeviceParse parse_gfa_device(Context &ctx, const std::string &path, int threads) {
  DeviceParse r(ctx.stream());
  Graph &g = r.graph;
  g = empty_graph();
  const Mapped m = map_file(path);
  const char *d = m.data;
  const uint64_t n = m.size;
  cudaStream_t st = ctx.stream();
  Lines ls;
  Names nm;
  if (!n) {
    size_traversals(g, 0, 0);
    g.paths.offsets.assign(1, 0);
    g.walks.offsets.assign(1, 0);
    r.offsets.assign(1, 0);
    return r;
  }
  ctx.reset_status();
  PhaseClock clk("gfa front end");
  // the file, zero-padded to 16 bytes
  const uint64_t npad = (n + 15) & ~15ull;
  DevVec<char> text(st);
  text.resize(npad);
  if (npad > n) cuda_check(cudaMemsetAsync(text.ptr + n, 0, npad - n, st), "memset");
  cuda_check(cudaMemcpyAsync(text.ptr, d, n, cudaMemcpyHostToDevice, st), "file upload");
  // line index
  const uint64_t nt = parse_num_tiles(n);
  DevVec<uint32_t> cnt(st), cnt2(st);
  DevVec<uint64_t> nl_off(st);
  cnt.resize(nt);
  nl_off.resize(nt + 1);
  timed(ctx, "gfa_newlines", (double)n, [&] { launch_nl_count(text.ptr, n, cnt.ptr, st); });
  scan_u32(ctx, cnt.ptr, nt, nl_off.ptr);
  const uint64_t nl = download_one(nl_off.ptr + nt, st);
  clk.mark("upload + newline count");
  const uint64_t nlines = nl + (d[n - 1] != '\n' ? 1 : 0);
  DevVec<uint64_t> eol(st), slotoff(st);
  DevVec<uint8_t> type(st);
  DevVec<uint32_t> ispw(st);
  eol.resize(nl ? nl : 1);
  type.resize(nlines);
  ispw.resize(nlines);
  slotoff.resize(nlines + 1);
  timed(ctx, "gfa_newlines", (double)n + 8.0 * nl, [&] { launch_nl_write(text.ptr, n, nl_off.ptr, eol.ptr, st); });
  timed(ctx, "gfa_line_heads", 13.0 * nlines,
        [&] { launch_line_heads(text.ptr, n, eol.ptr, nl, nlines, type.ptr, ispw.ptr, st); });
  scan_u32(ctx, ispw.ptr, nlines, slotoff.ptr);
  std::vector<uint8_t> htype(nlines);
  std::vector<uint64_t> heol(nl);
  uint64_t npw = 0;
  cuda_check(cudaMemcpyAsync(htype.data(), type.ptr, nlines, cudaMemcpyDeviceToHost, st), "download");
  if (nl) cuda_check(cudaMemcpyAsync(heol.data(), eol.ptr, nl * 8, cudaMemcpyDeviceToHost, st), "download");
  cuda_check(cudaMemcpyAsync(&npw, slotoff.ptr + nlines, 8, cudaMemcpyDeviceToHost, st), "download");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
  DevVec<PWLine> pw(st);
  pw.resize(npw ? npw : 1);
  timed(ctx, "gfa_line_fields", 9.0 * nlines + 32.0 * npw,
        [&] { launch_line_fields(text.ptr, n, eol.ptr, nl, nlines, type.ptr, slotoff.ptr, pw.ptr, st); });
  timed(ctx, "gfa_field_ends", (double)n,
        [&] { launch_field_ends(text.ptr, n, nl_off.ptr, nlines, slotoff.ptr, pw.ptr, st); });
  std::vector<uint64_t> pslot, wslot;  // record slot of each P / W line
  line_lists(htype, heol, nl, n, resolve_threads(threads), ls, pslot, wslot);
  for (uint64_t i = nlines; i-- > 0;)
    if (htype[i] == 'H') {  // the last H line is the header
      const uint64_t s = i ? heol[i - 1] + 1 : 0, e = i < nl ? heol[i] : n;
      g.header_line.assign(d + s, e - s);
      break;
    }
  std::vector<uint8_t>().swap(htype);
  std::vector<uint64_t>().swap(heol);
  clk.mark("line index");

  parse_segments(d, ls.S, g, nm, threads);
  clk.mark("S lines");
  NameIndex ni{nullptr, 0, nullptr, nullptr};
  DevVec<uint32_t> slots(st), nlen(st);
  DevVec<uint64_t> noff(st);
  if (!nm.numeric) {
    const uint64_t nn = nm.by_id.size() - 1;
    uint64_t cap = 1024;
    while (cap < 2 * nn) cap <<= 1;
    std::vector<uint64_t> ho(nn + 1, 0);
    std::vector<uint32_t> hl(nn + 1, 0);
    for (uint64_t id = 1; id <= nn; ++id) {
      ho[id] = (uint64_t)(nm.by_id[id].data() - d);
      hl[id] = (uint32_t)std::min<size_t>(nm.by_id[id].size(), UINT32_MAX);
    }
    slots.resize(cap);
    noff.resize(nn + 1);
    nlen.resize(nn + 1);
    cuda_check(cudaMemsetAsync(slots.ptr, 0, cap * 4, st), "memset");
    cuda_check(cudaMemcpyAsync(noff.ptr, ho.data(), (nn + 1) * 8, cudaMemcpyHostToDevice, st), "upload");
    cuda_check(cudaMemcpyAsync(nlen.ptr, hl.data(), (nn + 1) * 4, cudaMemcpyHostToDevice, st), "upload");
    timed(ctx, "gfa_name_table", 16.0 * nn,
          [&] { launch_name_table(text.ptr, noff.ptr, nlen.ptr, nn, slots.ptr, cap - 1, st); });
    ni = NameIndex{slots.ptr, cap - 1, noff.ptr, nlen.ptr};
    cuda_check(cudaStreamSynchronize(st), "stream sync");  // ho / hl leave scope
  }
  parse_links(d, ls.L, nm, g, threads);

  // P / W steps
  DevVec<uint64_t> offP(st), offW(st);
  DevVec<unsigned long long> err(st);
  cnt.resize(nt);
  cnt2.resize(nt);
  offP.resize(nt + 1);
  offW.resize(nt + 1);
  err.resize(1);
  cuda_check(cudaMemsetAsync(err.ptr, 0xFF, 8, st), "memset");
  timed(ctx, "gfa_tokens", (double)n,
        [&] { launch_token_count(text.ptr, n, nl_off.ptr, nlines, slotoff.ptr, pw.ptr, ni, cnt.ptr, cnt2.ptr,
                                 err.ptr, st); });
  scan_u32(ctx, cnt.ptr, nt, offP.ptr);
  scan_u32(ctx, cnt2.ptr, nt, offW.ptr);
  uint64_t tot[2];
  unsigned long long herr = 0;
  cuda_check(cudaMemcpyAsync(&tot[0], offP.ptr + nt, 8, cudaMemcpyDeviceToHost, st), "download");
  cuda_check(cudaMemcpyAsync(&tot[1], offW.ptr + nt, 8, cudaMemcpyDeviceToHost, st), "download");
  cuda_check(cudaMemcpyAsync(&herr, err.ptr, 8, cudaMemcpyDeviceToHost, st), "download");
  ctx.read_status();
  ctx.check_status("GFA front end");
  std::vector<PWLine> recs(npw);
  if (npw) {
    cuda_check(cudaMemcpyAsync(recs.data(), pw.ptr, npw * sizeof(PWLine), cudaMemcpyDeviceToHost, st), "download");
    cuda_check(cudaStreamSynchronize(st), "stream sync");
  }
  const size_t np = ls.P.size(), nw = ls.W.size();
  size_traversals(g, np, nw);
  // errors: the first P step error, else the first W line with an error
  // (its step error before its start/end error)
  if (herr != ~0ull && !(herr >> 62)) throw std::runtime_error(token_error((uint32_t)(herr & 3)));
  uint64_t wbad = nw;  // W line of the step error
  if (herr != ~0ull) {
    const uint64_t at = (herr & ((1ull << 62) - 1)) >> 2;
    for (uint64_t k = 0; k < nw; ++k) {
      const PWLine &rec = recs[wslot[k]];
      if (at >= rec.fstart && at < rec.fend) {
        wbad = k;
        break;
      }
    }
  }
  for (uint64_t k = 0; k < nw; ++k) {
    if (k == wbad) throw std::runtime_error(token_error((uint32_t)(herr & 3)));
    walk_header(std::string_view(d + ls.W[k].off, ls.W[k].len), g, k);
  }
  if (herr != ~0ull) throw std::runtime_error(token_error((uint32_t)(herr & 3)));
  for (uint64_t k = 0; k < np; ++k)
    path_header(std::string_view(d + ls.P[k].off, ls.P[k].len), recs[pslot[k]].fend - ls.P[k].off, g, k);

  clk.mark("L lines + step count");
  r.steps.resize(tot[0] + tot[1]);
  timed(ctx, "gfa_tokens", (double)n + 4.0 * (tot[0] + tot[1]), [&] {
    launch_token_write(text.ptr, n, nl_off.ptr, nlines, slotoff.ptr, pw.ptr, ni, offP.ptr, offW.ptr, r.steps.ptr,
                       r.steps.ptr + tot[0], err.ptr, st);
  });
  if (npw) cuda_check(cudaMemcpyAsync(recs.data(), pw.ptr, npw * sizeof(PWLine), cudaMemcpyDeviceToHost, st),
                      "download");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
  auto line_offsets = [&](const std::vector<uint64_t> &slot, uint64_t total, std::vector<uint64_t> &off) {
    off.assign(slot.size() + 1, total);
    for (size_t k = 0; k < slot.size(); ++k) {
      const uint64_t o = recs[slot[k]].out;
      off[k] = o == ~0ull ? total : o;
    }
  };
  line_offsets(pslot, tot[0], g.paths.offsets);
  line_offsets(wslot, tot[1], g.walks.offsets);
  r.offsets.assign(np + nw + 1, 0);
  for (size_t k = 0; k < np; ++k) r.offsets[k + 1] = g.paths.offsets[k + 1];
  for (size_t k = 0; k < nw; ++k) r.offsets[np + k + 1] = tot[0] + g.walks.offsets[k + 1];
  parse_jumps_containments(d, ls, nm, g);
  clk.mark("steps + J/C lines");
  return r;
}

void download_steps(Context &ctx, const DeviceParse &r, Graph &g) {
  cudaStream_t st = ctx.stream();
  const uint64_t NP = g.paths.offsets.empty() ? 0 : g.paths.offsets.back();
  const uint64_t NW = g.walks.offsets.empty() ? 0 : g.walks.offsets.back();
  g.paths.steps.resize(NP);
  g.walks.steps.resize(NW);
  if (NP)
    cuda_check(cudaMemcpyAsync(g.paths.steps.data(), r.steps.ptr, NP * 4, cudaMemcpyDeviceToHost, st), "download");
  if (NW)
    cuda_check(cudaMemcpyAsync(g.walks.steps.data(), r.steps.ptr + NP, NW * 4, cudaMemcpyDeviceToHost, st),
               "download");
  cuda_check(cudaStreamSynchronize(st), "stream sync");
}

}  // namespace gfz

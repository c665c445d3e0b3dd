// Host entropy stage (see codec.h).
#include "codec.h"

#include <dlfcn.h>
#include <unistd.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <mutex>
#include <stdexcept>

namespace gfz {

namespace {

// The public zstd entry points used here (names and signatures of the
// documented zstd API; resolved from libzstd.so.1 at run time).
struct ZstdApi {
  void *(*createCCtx)();
  size_t (*freeCCtx)(void *);
  size_t (*setParameter)(void *, int, int);
  size_t (*compressBound)(size_t);
  size_t (*compress2)(void *, void *, size_t, const void *, size_t);
  size_t (*decompress)(void *, size_t, const void *, size_t);
  unsigned (*isError)(size_t);
  const char *(*getErrorName)(size_t);
  unsigned (*versionNumber)();
  bool ok = false;
  std::string why;
};

constexpr int kZstdCompressionLevel = 100;  // ZSTD_c_compressionLevel
constexpr int kZstdNbWorkers = 400;         // ZSTD_c_nbWorkers

ZstdApi &api() {
  static ZstdApi a;
  static std::once_flag once;
  std::call_once(once, [] {
    const char *names[] = {"libzstd.so.1", "libzstd.so"};
    void *h = nullptr;
    for (const char *n : names)
      if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) {
      a.why = "libzstd.so.1 could not be loaded";
      return;
    }
#define GFZ_SYM(field, name)                                  \
  a.field = reinterpret_cast<decltype(a.field)>(dlsym(h, name)); \
  if (!a.field) {                                             \
    a.why = std::string("libzstd lacks ") + name;             \
    return;                                                   \
  }
    GFZ_SYM(createCCtx, "ZSTD_createCCtx");
    GFZ_SYM(freeCCtx, "ZSTD_freeCCtx");
    GFZ_SYM(setParameter, "ZSTD_CCtx_setParameter");
    GFZ_SYM(compressBound, "ZSTD_compressBound");
    GFZ_SYM(compress2, "ZSTD_compress2");
    GFZ_SYM(decompress, "ZSTD_decompress");
    GFZ_SYM(isError, "ZSTD_isError");
    GFZ_SYM(getErrorName, "ZSTD_getErrorName");
    GFZ_SYM(versionNumber, "ZSTD_versionNumber");
#undef GFZ_SYM
    a.ok = true;
  });
  if (!a.ok) throw std::runtime_error("zstd unavailable: " + a.why);
  return a;
}

int zstd_level() {
  static int level = -1;
  if (level == -1) {
    level = 9;
    if (const char *e = std::getenv("GFA_COMPRESSION_ZSTD_LEVEL")) {
      const int v = std::atoi(e);
      if (v >= 1 && v <= 22) level = v;
      else
        std::cerr << "Warning: GFA_COMPRESSION_ZSTD_LEVEL=" << e
                  << " is invalid (must be 1-22), using default 9." << std::endl;
    }
  }
  return level;
}

thread_local int g_zstd_threads = 1;

int zstd_workers() {
  static int env = -1;
  if (env == -1) {
    env = 0;
    if (const char *e = std::getenv("GFA_COMPRESSION_ZSTD_WORKERS")) {
      const int v = std::atoi(e);
      if (v >= 0) env = v;
      else
        std::cerr << "Warning: GFA_COMPRESSION_ZSTD_WORKERS=" << e
                  << " is invalid (must be >= 0), using active thread count." << std::endl;
    }
  }
  return env > 0 ? env : std::max(1, g_zstd_threads);
}

template <typename T>
std::vector<T> unzstd_as(const Block &b) {
  if (b.original_size == 0) return {};
  std::vector<T> out(b.original_size / sizeof(T));
  const size_t r = api().decompress(out.data(), b.original_size, b.payload.data(), b.payload.size());
  if (api().isError(r)) {
    std::cerr << "ZSTD decompression failed: " << api().getErrorName(r) << std::endl;
    return {};
  }
  return out;
}

void put_varint(uint64_t v, std::vector<uint8_t> &out) {
  while (v >= 0x80) {
    out.push_back((uint8_t)((v & 0x7F) | 0x80));
    v >>= 7;
  }
  out.push_back((uint8_t)v);
}

size_t get_varint(const uint8_t *p, size_t n, uint64_t &v, int max_shift) {
  v = 0;
  size_t i = 0;
  int shift = 0;
  while (i < n) {
    const uint8_t b = p[i++];
    if (shift <= max_shift) v |= (uint64_t)(b & 0x7F) << shift;
    if (!(b & 0x80)) break;
    shift += 7;
  }
  return i;
}

}  // namespace

int resolve_threads(int n) {
  if (n > 0) return n;
  const long procs = std::max(1L, sysconf(_SC_NPROCESSORS_ONLN));
  if (n < 0) return (int)procs;
  for (const char *var : {"GFAZ_NUM_THREADS", "OMP_NUM_THREADS"}) {
    if (const char *e = std::getenv(var)) {
      char *end = nullptr;
      const long v = std::strtol(e, &end, 10);
      if (end != e && *end == '\0' && v > 0) return (int)v;
    }
  }
  return (int)std::min<long>(8, std::max<long>(1, procs / 2));
}

void set_zstd_threads(int t) { g_zstd_threads = std::max(1, t); }

unsigned zstd_version() { return api().versionNumber(); }

bool zstd_available(std::string *why) {
  try {
    api();
    return true;
  } catch (const std::exception &e) {
    if (why) *why = e.what();
    return false;
  }
}

Block zstd_bytes(const void *data, size_t n) {
  Block b;
  b.original_size = n;
  if (n == 0) return b;
  ZstdApi &z = api();
  void *cctx = z.createCCtx();
  if (!cctx) {
    std::cerr << "ZSTD compression failed: unable to create compression context" << std::endl;
    return b;
  }
  size_t r = z.setParameter(cctx, kZstdCompressionLevel, zstd_level());
  if (z.isError(r)) {
    std::cerr << "ZSTD parameter setup failed: " << z.getErrorName(r) << std::endl;
    z.freeCCtx(cctx);
    return b;
  }
  r = z.setParameter(cctx, kZstdNbWorkers, zstd_workers());
  if (z.isError(r)) {
    static bool warned = false;
    if (!warned) {
      std::cerr << "Warning: ZSTD multithreaded compression is unavailable (" << z.getErrorName(r)
                << "); falling back to single-threaded ZSTD." << std::endl;
      warned = true;
    }
  }
  b.payload.resize(z.compressBound(n));
  const size_t c = z.compress2(cctx, b.payload.data(), b.payload.size(), data, n);
  z.freeCCtx(cctx);
  if (z.isError(c)) {
    std::cerr << "ZSTD compression failed: " << z.getErrorName(c) << std::endl;
    b.payload.clear();
    return b;
  }
  b.payload.resize(c);
  return b;
}

std::vector<uint8_t> unzstd(const Block &b) { return unzstd_as<uint8_t>(b); }
Block zstd_i32(const std::vector<int32_t> &v) { return zstd_bytes(v.data(), v.size() * 4); }
Block zstd_u32(const std::vector<uint32_t> &v) { return zstd_bytes(v.data(), v.size() * 4); }
Block zstd_str(const std::string &s) { return zstd_bytes(s.data(), s.size()); }
Block zstd_chars(const std::vector<char> &v) { return zstd_bytes(v.data(), v.size()); }
Block zstd_f32(const std::vector<float> &v) { return zstd_bytes(v.data(), v.size() * 4); }
std::vector<int32_t> unzstd_i32(const Block &b) { return unzstd_as<int32_t>(b); }
std::vector<uint32_t> unzstd_u32(const Block &b) { return unzstd_as<uint32_t>(b); }
std::vector<char> unzstd_chars(const Block &b) { return unzstd_as<char>(b); }
std::vector<float> unzstd_f32(const Block &b) { return unzstd_as<float>(b); }
std::string unzstd_str(const Block &b) {
  std::vector<char> v = unzstd_as<char>(b);
  return std::string(v.begin(), v.end());
}

Block delta_varint_u32(const std::vector<uint32_t> &v) {
  if (v.empty()) return Block{};
  std::vector<uint8_t> bytes;
  bytes.reserve(v.size() * 2);
  int32_t prev = 0;
  for (size_t i = 0; i < v.size(); ++i) {
    const int32_t cur = (int32_t)v[i];
    const int32_t d = i == 0 ? cur : (int32_t)((uint32_t)cur - (uint32_t)prev);
    prev = cur;
    const uint32_t zz = ((uint32_t)d << 1) ^ (uint32_t)(d >> 31);
    put_varint(zz, bytes);
  }
  return zstd_bytes(bytes.data(), bytes.size());
}

std::vector<uint32_t> undelta_varint_u32(const Block &b, size_t n) {
  if (b.original_size == 0 || n == 0) return {};
  const std::vector<uint8_t> bytes = unzstd(b);
  std::vector<uint32_t> out;
  out.reserve(n);
  size_t p = 0;
  uint32_t acc = 0;
  while (p < bytes.size() && out.size() < n) {
    uint64_t zz;
    p += get_varint(bytes.data() + p, bytes.size() - p, zz, 31);
    const uint32_t z = (uint32_t)zz;
    const int32_t d = (int32_t)((z >> 1) ^ (~(z & 1u) + 1u));
    acc = out.empty() ? (uint32_t)d : acc + (uint32_t)d;
    out.push_back(acc);
  }
  return out;
}

Block orientations(const std::vector<char> &o) {
  std::vector<uint8_t> packed((o.size() + 7) / 8, 0);
  for (size_t i = 0; i < o.size(); ++i)
    if (o[i] == '-') packed[i >> 3] |= (uint8_t)(1u << (i & 7));
  return zstd_bytes(packed.data(), packed.size());
}

std::vector<char> unorientations(const Block &b, size_t n) {
  std::vector<char> out;
  if (b.original_size == 0 || n == 0) return out;
  const std::vector<uint8_t> packed = unzstd(b);
  out.reserve(n);
  for (size_t i = 0; i < n; ++i) {
    const size_t byte = i >> 3;
    const uint8_t bit = byte < packed.size() ? (packed[byte] >> (i & 7)) & 1u : 0u;
    out.push_back(bit ? '-' : '+');
  }
  return out;
}

Block varint_i64(const std::vector<int64_t> &v) {
  if (v.empty()) return Block{};
  std::vector<uint8_t> bytes;
  bytes.reserve(v.size() * 4);
  for (int64_t x : v) put_varint(((uint64_t)x << 1) ^ (uint64_t)(x >> 63), bytes);
  return zstd_bytes(bytes.data(), bytes.size());
}

std::vector<int64_t> unvarint_i64(const Block &b, size_t n) {
  if (b.original_size == 0 || n == 0) return {};
  const std::vector<uint8_t> bytes = unzstd(b);
  std::vector<int64_t> out;
  out.reserve(n);
  size_t p = 0;
  while (p < bytes.size() && out.size() < n) {
    uint64_t z;
    p += get_varint(bytes.data() + p, bytes.size() - p, z, 63);
    out.push_back((int64_t)((z >> 1) ^ (~(z & 1ULL) + 1ULL)));
  }
  return out;
}

void join_strings(const std::vector<std::string> &v, std::string &cat, std::vector<uint32_t> &lens) {
  size_t total = 0;
  for (const auto &s : v) total += s.size();
  cat.clear();
  cat.reserve(total);
  lens.clear();
  lens.reserve(v.size());
  for (const auto &s : v) {
    cat += s;
    lens.push_back((uint32_t)s.size());
  }
}

std::vector<std::string> split_strings(const std::string &cat, const std::vector<uint32_t> &lens, bool strict,
                                       const char *prefix) {
  std::vector<std::string> out;
  out.reserve(lens.size());
  size_t o = 0;
  for (uint32_t l : lens) {
    if (o + l > cat.size()) {
      if (strict) throw std::runtime_error(std::string(prefix) + "string column is truncated");
      out.emplace_back();
      continue;
    }
    out.push_back(cat.substr(o, l));
    o += l;
  }
  return out;
}

}  // namespace gfz

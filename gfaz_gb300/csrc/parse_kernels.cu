// GFA front end on the device: line index, P/W field bounds and the P/W
// step tokens resolved to signed segment ids.
//
// The rules are the host parser's (host/gfa_parser.cpp), which follow the
// reference's src/io/gfa_parser.cpp:
//  * lines end at '\n' only; a line is typed by its first byte (:353-404);
//  * fields are separated by runs of ' ' / '\t' (next_field, :124-131);
//  * P: name, then the steps field up to the next blank; steps are split on
//    ',' (empty pieces skipped), the last byte of a piece is its orientation
//    ('-' reverse, anything else forward), the rest its segment name
//    (:347-404);
//  * W: sample, hap, seq id, start, end, then the walk field up to the next
//    blank; a step starts at '>' or '<' and runs to the next '>' / '<'; bytes
//    before the first marker are skipped, as are empty names (:405-461);
//  * a name resolves to its number when every segment name is the decimal
//    form of its id (parse_uint32: digits up to the first non-digit; none is
//    an error, as is a value above UINT32_MAX), else through the name table;
//    unresolved names and id 0 drop the step (:881-890, :1210-1218).
//
// Work split: the file is cut into 4 KB tiles, 16 bytes per thread.  Every
// per-byte kernel recovers the line of each byte from a block scan of the
// thread's newline count on top of the tile's exclusive newline count, so
// no kernel searches for line starts.  A token belongs to the thread whose
// bytes hold its first byte; that thread reads the token to its end from
// the block's shared-memory copy of the tile (plus a lookahead), or from
// global memory past it.
#include "common.cuh"
#include "kernels.h"

namespace gfz {

namespace {

constexpr int kPB = 256;                        // threads per block
constexpr int kPBytes = 16;                     // bytes per thread
constexpr uint32_t kPTile = kPB * kPBytes;      // bytes per tile
constexpr uint32_t kPLook = 256;                // lookahead bytes staged after the tile
constexpr uint32_t kPStage = kPTile + kPLook;

__device__ __forceinline__ bool blank(uint32_t c) { return c == ' ' || c == '\t'; }

__device__ __forceinline__ uint32_t nl_count(const uint4 &v) {
  return (__popc(__vcmpeq4(v.x, 0x0A0A0A0Au)) + __popc(__vcmpeq4(v.y, 0x0A0A0A0Au)) +
          __popc(__vcmpeq4(v.z, 0x0A0A0A0Au)) + __popc(__vcmpeq4(v.w, 0x0A0A0A0Au))) >>
         3;
}

__device__ __forceinline__ uint32_t byte_of(const uint4 &v, int k) {
  const uint32_t w = k < 4 ? v.x : k < 8 ? v.y : k < 12 ? v.z : v.w;
  return (w >> (8 * (k & 3))) & 0xFFu;
}

// 16 bytes at p; bytes at or past n read as 0 (the text buffer is padded
// to a multiple of 16 bytes, so the vector load stays inside it).
__device__ __forceinline__ uint4 load16(const char *__restrict__ t, uint64_t p, uint64_t n) {
  uint4 v = make_uint4(0, 0, 0, 0);
  if (p >= n) return v;
  v = *reinterpret_cast<const uint4 *>(t + p);
  if (p + 16 > n) {
    const int keep = (int)(n - p);  // 1..15 bytes are real
    uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int lo = 4 * k;
      if (keep <= lo) w[k] = 0;
      else if (keep < lo + 4) w[k] &= (1u << (8 * (keep - lo))) - 1u;
    }
    v = make_uint4(w[0], w[1], w[2], w[3]);
  }
  return v;
}

// The tile plus lookahead in shared memory; bytes past the staged range
// come from global memory.
struct Staged {
  const uint8_t *s;
  const char *g;
  uint64_t base, len;  // staged file range [base, base + len)
  __device__ __forceinline__ uint32_t at(uint64_t j) const {
    const uint64_t r = j - base;  // wraps for j < base
    return r < len ? (uint32_t)s[r] : (uint32_t)(uint8_t)g[j];
  }
};

__device__ __forceinline__ Staged stage_tile(const char *__restrict__ text, uint64_t n, uint64_t base,
                                             uint4 *smem) {
  const uint64_t end = min(n, base + kPStage);
  for (uint32_t i = threadIdx.x; i < kPStage / 16; i += kPB) smem[i] = load16(text, base + 16ull * i, n);
  __syncthreads();
  return Staged{reinterpret_cast<const uint8_t *>(smem), text, base, end - base};
}

// Line record the per-byte kernels need: whether the line is P/W, its
// record slot and field bounds.
struct LineView {
  bool pw;
  uint32_t kind;
  uint64_t slot, fstart, fend;
};

__device__ __forceinline__ LineView line_view(const uint64_t *slotoff, const PWLine *pw, uint64_t nlines,
                                              uint64_t li) {
  LineView L;
  L.slot = li < nlines ? slotoff[li] : 0;
  L.pw = li < nlines && slotoff[li + 1] != L.slot;
  L.kind = 0;
  L.fstart = L.fend = 0;
  if (L.pw) {  // the write pass stores .out of these records meanwhile
    L.kind = pw[L.slot].kind;
    L.fstart = pw[L.slot].fstart;
    L.fend = pw[L.slot].fend;
  }
  return L;
}

// FNV-1a over the name bytes, then the MurmurHash3 64-bit finalizer.
__device__ __forceinline__ uint64_t name_hash(const Staged &S, uint64_t a, uint64_t b) {
  uint64_t h = 0xcbf29ce484222325ull;
  for (uint64_t j = a; j < b; ++j) h = (h ^ S.at(j)) * 0x100000001b3ull;
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h;
}

__device__ __forceinline__ uint64_t name_hash_global(const char *t, uint64_t a, uint64_t b) {
  uint64_t h = 0xcbf29ce484222325ull;
  for (uint64_t j = a; j < b; ++j) h = (h ^ (uint8_t)t[j]) * 0x100000001b3ull;
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h;
}

// Resolves name bytes [a, b) (b > a) to a segment id; 0 = unresolved.
// Numeric mode errors are reported through *err as the smallest
// (W << 62 | position << 2 | code) over the file.
__device__ __forceinline__ uint32_t resolve(const Staged &S, uint64_t a, uint64_t b, const NameIndex &ni,
                                            uint32_t kind, unsigned long long *err) {
  if (!ni.slots) {
    uint32_t v = 0;
    bool any = false;
    for (uint64_t j = a; j < b; ++j) {
      const uint32_t c = S.at(j);
      if (c < '0' || c > '9') break;
      any = true;
      const uint32_t d = c - '0';
      if (v > 429496729u || (v == 429496729u && d > 5u)) {
        atomicMin(err, ((unsigned long long)kind << 62) | (a << 2) | kParseOverflow);
        return 0;
      }
      v = v * 10u + d;
    }
    if (!any) {
      atomicMin(err, ((unsigned long long)kind << 62) | (a << 2) | kParseNoDigits);
      return 0;
    }
    return v;
  }
  const uint64_t len = b - a;
  uint64_t h = name_hash(S, a, b) & ni.mask;
  for (uint64_t probe = 0; probe <= ni.mask; ++probe) {
    const uint32_t id = ni.slots[h];
    if (id == 0) return 0;
    if (ni.nlen[id] == len) {
      const char *q = S.g + ni.noff[id];
      uint64_t j = 0;
      while (j < len && (uint8_t)q[j] == S.at(a + j)) ++j;
      if (j == len) return id;
    }
    h = (h + 1) & ni.mask;
  }
  return 0;
}

// The token starting at p (a P piece or a W marker) inside its field
// [p, fend): its signed id, 0 when dropped.  prev: the byte before p.
__device__ __forceinline__ int32_t parse_token(const Staged &S, uint64_t p, uint32_t c, uint32_t prev,
                                               const LineView &L, const NameIndex &ni, unsigned long long *err) {
  if (L.kind == 0) {
    if (c == ',' || (p != L.fstart && prev != ',')) return 0;
    uint64_t q = p + 1;
    while (q < L.fend && S.at(q) != ',') ++q;
    if (q - p < 2) return 0;  // empty name
    const uint32_t o = S.at(q - 1);
    const uint32_t id = resolve(S, p, q - 1, ni, 0, err);
    if (!id) return 0;
    return o == '-' ? (int32_t)(0u - id) : (int32_t)id;
  }
  if (c != '>' && c != '<') return 0;
  uint64_t q = p + 1;
  while (q < L.fend) {
    const uint32_t x = S.at(q);
    if (x == '>' || x == '<') break;
    ++q;
  }
  if (q == p + 1) return 0;  // empty name
  const uint32_t id = resolve(S, p + 1, q, ni, 1, err);
  if (!id) return 0;
  return c == '<' ? (int32_t)(0u - id) : (int32_t)id;
}

__global__ void __launch_bounds__(kPB) k_nl_count(const char *__restrict__ text, uint64_t n, uint32_t *cnt) {
  const uint64_t p0 = (uint64_t)blockIdx.x * kPTile + (uint64_t)threadIdx.x * kPBytes;
  unsigned long long total;
  block_excl_sum<kPB>(nl_count(load16(text, p0, n)), total);
  if (threadIdx.x == 0) cnt[blockIdx.x] = (uint32_t)total;
}

__global__ void __launch_bounds__(kPB) k_nl_write(const char *__restrict__ text, uint64_t n,
                                                  const uint64_t *__restrict__ nl_off, uint64_t *eol) {
  const uint64_t p0 = (uint64_t)blockIdx.x * kPTile + (uint64_t)threadIdx.x * kPBytes;
  const uint4 v = load16(text, p0, n);
  unsigned long long total;
  uint64_t at = nl_off[blockIdx.x] + block_excl_sum<kPB>(nl_count(v), total);
#pragma unroll
  for (int k = 0; k < kPBytes; ++k)
    if (byte_of(v, k) == '\n') eol[at++] = p0 + k;
}

// Line i spans [i ? eol[i-1] + 1 : 0, i < nl ? eol[i] : n).
__global__ void k_line_heads(const char *__restrict__ text, uint64_t n, const uint64_t *__restrict__ eol,
                             uint64_t nl, uint64_t nlines, uint8_t *type, uint32_t *ispw) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nlines;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = i ? eol[i - 1] + 1 : 0, e = i < nl ? eol[i] : n;
    const uint8_t t = e > s ? (uint8_t)text[s] : 0;
    type[i] = t;
    ispw[i] = t == 'P' || t == 'W';
  }
}

__global__ void k_line_fields(const char *__restrict__ text, uint64_t n, const uint64_t *__restrict__ eol,
                              uint64_t nl, uint64_t nlines, const uint8_t *__restrict__ type,
                              const uint64_t *__restrict__ slotoff, PWLine *pw) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nlines;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint8_t t = type[i];
    if (t != 'P' && t != 'W') continue;
    const uint64_t s = i ? eol[i - 1] + 1 : 0, e = i < nl ? eol[i] : n;
    uint64_t pos = s + 1;
    const int fields = t == 'P' ? 1 : 5;  // fields before the steps / walk field
    for (int f = 0; f < fields; ++f) {
      while (pos < e && blank((uint8_t)text[pos])) ++pos;
      while (pos < e && !blank((uint8_t)text[pos])) ++pos;
    }
    while (pos < e && blank((uint8_t)text[pos])) ++pos;
    PWLine r;
    r.fstart = pos;
    r.fend = e;
    r.out = ~0ull;
    r.kind = t == 'W';
    r.pad = 0;
    pw[slotoff[i]] = r;
  }
}

// Per-thread line state over its 16 bytes.
struct Walk {
  uint64_t p0, li;
  uint4 v;
};

__device__ __forceinline__ Walk begin_walk(const char *__restrict__ text, uint64_t n,
                                           const uint64_t *__restrict__ nl_off) {
  Walk w;
  w.p0 = (uint64_t)blockIdx.x * kPTile + (uint64_t)threadIdx.x * kPBytes;
  w.v = load16(text, w.p0, n);
  unsigned long long total;
  w.li = nl_off[blockIdx.x] + block_excl_sum<kPB>(nl_count(w.v), total);
  return w;
}

// fend of every P/W line = first blank at or after fstart (or the line end).
__global__ void __launch_bounds__(kPB) k_field_ends(const char *__restrict__ text, uint64_t n,
                                                    const uint64_t *__restrict__ nl_off, uint64_t nlines,
                                                    const uint64_t *__restrict__ slotoff, PWLine *pw) {
  Walk w = begin_walk(text, n, nl_off);
  bool fresh = false;
  LineView L;
#pragma unroll
  for (int k = 0; k < kPBytes; ++k) {
    const uint64_t p = w.p0 + k;
    if (p >= n) break;
    const uint32_t c = byte_of(w.v, k);
    if (blank(c)) {
      if (!fresh) {
        L = line_view(slotoff, pw, nlines, w.li);
        fresh = true;
      }
      if (L.pw && p >= L.fstart && p < L.fend) {
        atomicMin(&pw[L.slot].fend, (unsigned long long)p);
        L.fend = p;
      }
    }
    if (c == '\n') {
      ++w.li;
      fresh = false;
    }
  }
}

// Numeric names, whole window inside one steps / walk field: a straight-
// line lexer over the thread's 16 bytes and the 16 that follow (no
// per-token loops, so the warp does not diverge).  Tokens that start in
// the first 16 bytes and end inside the 32 get their id at the position
// of the byte that ends them (id[j], bit j of *mask); a token still open
// at byte 31 is left for parse_token (*longk = its first byte, else -1).
// The name of a P token excludes its last byte (the orientation), so the
// digit state is also kept as it was before the last digit.
template <bool P>
__device__ __forceinline__ void lex_window(const uint4 &a, const uint4 &b, bool start0, uint64_t p0,
                                           unsigned long long *err, int32_t (&id)[32], uint32_t &mask, int &longk) {
  bool active = false, any = false, pany = false, stopped = false, lastacc = false, rev = false;
  uint64_t v = 0, pv = 0;
  int ts = 0;
  uint32_t prevc = 0;
  mask = 0;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const uint32_t c = j < 16 ? byte_of(a, j) : byte_of(b, j - 16);
    const bool bound = P ? c == ',' : (c == '>' || c == '<');
    id[j] = 0;
    if (bound) {
      if (active) {
        // the token [ts, j): P name = [ts, j - 1) with orientation prevc;
        // W name = (ts, j)
        const bool empty = j - ts < 2;  // P: one byte (the orientation); W: the marker alone
        const uint64_t nv = P && lastacc ? pv : v;
        const bool nany = P && lastacc ? pany : any;
        const uint64_t at = P ? p0 + ts : p0 + ts + 1;
        if (!empty) {
          if (!nany) {
            atomicMin(err, ((unsigned long long)(P ? 0 : 1) << 62) | (at << 2) | kParseNoDigits);
          } else if (nv > 0xFFFFFFFFull) {
            atomicMin(err, ((unsigned long long)(P ? 0 : 1) << 62) | (at << 2) | kParseOverflow);
          } else if (nv) {
            const bool neg = P ? prevc == '-' : rev;
            id[j] = neg ? (int32_t)(0u - (uint32_t)nv) : (int32_t)(uint32_t)nv;
            mask |= 1u << j;
          }
        }
        active = false;
      }
      if (!P && j < 16) {  // a W marker opens the next token
        active = true;
        ts = j;
        rev = c == '<';
        v = pv = 0;
        any = pany = stopped = lastacc = false;
      }
    } else {
      if (P && !active && j < 16 && (j == 0 ? start0 : prevc == ',')) {
        active = true;
        ts = j;
        v = pv = 0;
        any = pany = stopped = lastacc = false;
      }
      if (active) {
        const bool dig = c - '0' < 10u;
        if (!stopped && dig) {
          pv = v;
          pany = any;
          if (v < (1ull << 40)) v = v * 10 + (c - '0');  // beyond 2^40 it overflows anyway
          any = true;
          lastacc = true;
        } else {
          stopped = stopped || !dig;
          lastacc = false;
        }
      }
    }
    prevc = c;
  }
  longk = active ? ts : -1;
}

// Pass 1 (WRITE = false): per-tile counts of kept P and W steps.  Pass 2:
// the steps written at the scanned offsets, and each P/W line's first
// output index.
template <bool WRITE>
__global__ void __launch_bounds__(kPB, 2) k_tokens(const char *__restrict__ text, uint64_t n,
                                                const uint64_t *__restrict__ nl_off, uint64_t nlines,
                                                const uint64_t *__restrict__ slotoff, PWLine *pw, NameIndex ni,
                                                uint32_t *cntP, uint32_t *cntW, const uint64_t *__restrict__ offP,
                                                const uint64_t *__restrict__ offW, int32_t *outP, int32_t *outW,
                                                unsigned long long *err) {
  __shared__ uint4 smem[kPStage / 16];
  const Staged S = stage_tile(text, n, (uint64_t)blockIdx.x * kPTile, smem);
  Walk w = begin_walk(text, n, nl_off);
  const uint64_t li0 = w.li;
  uint32_t prev = w.p0 && w.p0 <= n ? S.at(w.p0 - 1) : 0;
  const LineView L0 = line_view(slotoff, pw, nlines, w.li);
  // fast: numeric names and all 32 bytes from p0 inside the line's field
  const bool fast = !ni.slots && L0.pw && w.p0 >= L0.fstart && w.p0 + 32 <= L0.fend;
  int32_t ids[32];
  // slow: bit k = a kept step starts at byte k (wk: it is a W step);
  // fast: bit j = a kept step ends at byte j
  uint32_t tok = 0, wk = 0;
  int32_t long_id = 0;
  if (fast) {
    const uint4 nx = smem[(w.p0 - S.base) / 16 + 1];
    const bool start0 = L0.kind == 0 && (w.p0 == L0.fstart || prev == ',');
    int longk;
    if (L0.kind == 0) lex_window<true>(w.v, nx, start0, w.p0, err, ids, tok, longk);
    else lex_window<false>(w.v, nx, false, w.p0, err, ids, tok, longk);
    if (longk >= 0) {
      const uint64_t q = w.p0 + longk;
      long_id = parse_token(S, q, S.at(q), S.at(q - 1), L0, ni, err);
    }
    if (L0.kind) wk = tok;
  } else {
    LineView L = L0;
#pragma unroll
    for (int k = 0; k < kPBytes; ++k) {
      ids[k] = 0;
      const uint64_t p = w.p0 + k;
      if (p < n) {
        const uint32_t c = byte_of(w.v, k);
        if (L.pw && p >= L.fstart && p < L.fend) {
          const int32_t id = parse_token(S, p, c, prev, L, ni, err);
          if (id) {
            ids[k] = id;
            tok |= 1u << k;
            wk |= L.kind << k;
          }
        }
        if (c == '\n') L = line_view(slotoff, pw, nlines, ++w.li);
        prev = c;
      }
    }
  }
  const uint32_t nlong = long_id != 0;
  const uint32_t cw = __popc(wk) + (fast && L0.kind ? nlong : 0);
  const uint32_t cp = __popc(tok) - __popc(wk) + (fast && !L0.kind ? nlong : 0);
  unsigned long long total;
  const unsigned long long ex = block_excl_sum<kPB>(((unsigned long long)cp << 32) | cw, total);
  if (!WRITE) {
    if (threadIdx.x == 0) {
      cntP[blockIdx.x] = (uint32_t)(total >> 32);
      cntW[blockIdx.x] = (uint32_t)total;
    }
    return;
  }
  uint64_t ip = offP[blockIdx.x] + (ex >> 32), iw = offW[blockIdx.x] + (uint32_t)ex;
  if (fast) {
    if (w.p0 == L0.fstart) pw[L0.slot].out = L0.kind ? iw : ip;
    int32_t *o = L0.kind ? outW + iw : outP + ip;
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if ((tok >> j) & 1u) *o++ = ids[j];
    if (long_id) *o = long_id;
    return;
  }
  // first output index of every P/W line whose field starts in these bytes
  uint64_t li = li0;
  LineView M = L0;
#pragma unroll
  for (int k = 0; k < kPBytes; ++k) {
    const uint64_t p = w.p0 + k;
    if (p < n) {
      if (M.pw && p == M.fstart) {
        const uint32_t below = (1u << k) - 1u;
        pw[M.slot].out = M.kind ? iw + __popc(wk & below) : ip + __popc(tok & ~wk & below);
      }
      if (byte_of(w.v, k) == '\n') M = line_view(slotoff, pw, nlines, ++li);
    }
  }
#pragma unroll
  for (int k = 0; k < kPBytes; ++k)
    if ((tok >> k) & 1u) {
      if ((wk >> k) & 1u) outW[iw++] = ids[k];
      else outP[ip++] = ids[k];
    }
}

// Name table: slot = id of the name whose hash lands there (linear probing).
__global__ void k_name_table(const char *__restrict__ text, const uint64_t *__restrict__ noff,
                             const uint32_t *__restrict__ nlen, uint64_t nnames, uint32_t *slots, uint64_t mask) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nnames;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t id = (uint32_t)(i + 1);
    uint64_t h = name_hash_global(text, noff[id], noff[id] + nlen[id]) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
      if (atomicCAS(&slots[h], 0u, id) == 0u) break;
      h = (h + 1) & mask;
    }
  }
}

inline unsigned grid_for(uint64_t n, int block, unsigned cap = 152u * 16u) {
  uint64_t g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (unsigned)g;
}

}  // namespace

uint64_t parse_num_tiles(uint64_t n) { return (n + kPTile - 1) / kPTile; }

void launch_nl_count(const char *text, uint64_t n, uint32_t *cnt, cudaStream_t st) {
  const uint64_t nt = parse_num_tiles(n);
  if (nt) k_nl_count<<<(unsigned)nt, kPB, 0, st>>>(text, n, cnt);
}

void launch_nl_write(const char *text, uint64_t n, const uint64_t *nl_off, uint64_t *eol, cudaStream_t st) {
  const uint64_t nt = parse_num_tiles(n);
  if (nt) k_nl_write<<<(unsigned)nt, kPB, 0, st>>>(text, n, nl_off, eol);
}

void launch_line_heads(const char *text, uint64_t n, const uint64_t *eol, uint64_t nl, uint64_t nlines,
                       uint8_t *type, uint32_t *ispw, cudaStream_t st) {
  if (nlines) k_line_heads<<<grid_for(nlines, 256), 256, 0, st>>>(text, n, eol, nl, nlines, type, ispw);
}

void launch_line_fields(const char *text, uint64_t n, const uint64_t *eol, uint64_t nl, uint64_t nlines,
                        const uint8_t *type, const uint64_t *slotoff, PWLine *pw, cudaStream_t st) {
  if (nlines) k_line_fields<<<grid_for(nlines, 256), 256, 0, st>>>(text, n, eol, nl, nlines, type, slotoff, pw);
}

void launch_field_ends(const char *text, uint64_t n, const uint64_t *nl_off, uint64_t nlines, const uint64_t *slotoff,
                       PWLine *pw, cudaStream_t st) {
  const uint64_t nt = parse_num_tiles(n);
  if (nt) k_field_ends<<<(unsigned)nt, kPB, 0, st>>>(text, n, nl_off, nlines, slotoff, pw);
}

void launch_token_count(const char *text, uint64_t n, const uint64_t *nl_off, uint64_t nlines,
                        const uint64_t *slotoff, PWLine *pw, const NameIndex &ni, uint32_t *cntP, uint32_t *cntW,
                        unsigned long long *err, cudaStream_t st) {
  const uint64_t nt = parse_num_tiles(n);
  if (nt)
    k_tokens<false><<<(unsigned)nt, kPB, 0, st>>>(text, n, nl_off, nlines, slotoff, pw, ni, cntP, cntW, nullptr,
                                                  nullptr, nullptr, nullptr, err);
}

void launch_token_write(const char *text, uint64_t n, const uint64_t *nl_off, uint64_t nlines,
                        const uint64_t *slotoff, PWLine *pw, const NameIndex &ni, const uint64_t *offP,
                        const uint64_t *offW, int32_t *outP, int32_t *outW, unsigned long long *err, cudaStream_t st) {
  const uint64_t nt = parse_num_tiles(n);
  if (nt)
    k_tokens<true><<<(unsigned)nt, kPB, 0, st>>>(text, n, nl_off, nlines, slotoff, pw, ni, nullptr, nullptr, offP,
                                                 offW, outP, outW, err);
}

void launch_name_table(const char *text, const uint64_t *noff, const uint32_t *nlen, uint64_t nnames,
                       uint32_t *slots, uint64_t mask, cudaStream_t st) {
  if (nnames) k_name_table<<<grid_for(nnames, 256), 256, 0, st>>>(text, noff, nlen, nnames, slots, mask);
}

}  // namespace gfz

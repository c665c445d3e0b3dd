// Host-callable launchers for the GFAz transform kernels.  Every pointer is a
// device pointer; every launch goes to `stream`.  Launchers never allocate.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gfz {

// Per-context device status block (zeroed by the owner).
struct DevStatus {
  uint32_t err;            // OR of kErr* bits
  uint32_t aux;            // u32 result slot (max |x| of delta coding)
  unsigned long long u64[8];  // kernel result slots (see each launcher)
  unsigned long long pass_open[4];  // rules still open after each pass of a batch of level passes
  uint32_t sticky_err;     // error bits carried past reset_status (a grammar round's sort)
  uint32_t pad;
};

// ---- encode side ----------------------------------------------------------
// out[i] = in[i] - in[i-1] inside each traversal (first element copied);
// atomically max-reduces |out| into *max_abs.  in == out is NOT allowed.
void launch_delta_encode(const int32_t *in, int32_t *out, uint64_t n, const uint64_t *off,
                         uint64_t ntrav, uint32_t *max_abs, cudaStream_t st);
// max |x| of the raw stream (delta_round == 0 seed).
void launch_max_abs(const int32_t *in, uint64_t n, uint32_t *max_abs, cudaStream_t st);

// One hash slot: the canonical key (kEmptyKey when free), its kFlag* bits
// and the final rule id, in one 16-byte word so that a lookup is one load.
struct alignas(16) PairSlot {
  unsigned long long key;
  uint32_t flags;
  uint32_t val;
};
struct PairTable {
  PairSlot *slots;  // cap slots
  uint64_t cap;     // power of two, at most 2^31
};
// dst[0, n) = src[0, n) by a kernel (either side may be page-locked host
// memory); 16-byte words where both ends are 16-byte aligned.
void launch_copy_bytes(const void *src, void *dst, uint64_t n, cudaStream_t st);
// dst[0, n) = 0 by a kernel.
void launch_zero_bytes(void *dst, uint64_t n, cudaStream_t st);
// Sets every slot to {kEmptyKey, 0, val_init} and clears the (cap + 31) / 32
// words of the slot bitmaps given (bits_a, bits_b; either may be null).
void launch_table_clear(PairTable tab, uint32_t val_init, cudaStream_t st, uint32_t *bits_a = nullptr,
                        uint32_t *bits_b = nullptr);

// Traversal-head bitmap of an n-step stream: head_words(n) words (padded
// for tile staging); bit q set <=> some off[t] == q (t <= ntrav, so bit n is
// set).  launch_head_bits sets the bits of a cleared bitmap.
uint64_t head_words(uint64_t n);
void launch_head_bits(const uint64_t *off, uint64_t ntrav, uint32_t *bits, cudaStream_t st);

// Inserts every canonical adjacent pair inside a traversal (heads: the
// stream's head bitmap).  Results: status->u64[0] += new distinct keys,
// u64[1] += keys that became repeated.  The kernels give the same table
// contents (slot placement aside): kTiled stages tiles in shared memory and
// folds runs of equal keys (streams with many repeats); kTiledWarpDedup
// also folds equal keys across a warp; kFlat takes one pair per thread
// without staging or barriers (streams of mostly new pairs); kFlat4 takes
// four and folds their runs, still without barriers.
// With sref (n entries; not with kTiledWarpDedup; tables of at most 2^30
// slots) every position p gets its slot reference: the slot of the pair
// starting at p, bit 31 set when the pair is the reverse of its canonical
// key, 0xFFFFFFFF where no pair starts; with rep_bits (cap bits, zeroed with
// the table) the slot of every key that becomes repeated is set in it.
enum class CountKernel { kTiled = 0, kTiledWarpDedup = 1, kFlat = 2, kFlat4 = 3 };
void launch_count_pairs(const int32_t *s, uint64_t n, const uint32_t *heads, PairTable tab, DevStatus *status,
                        CountKernel kind, cudaStream_t st, uint32_t *sref = nullptr, uint32_t *rep_bits = nullptr);

// Greedy left-to-right replacement of candidate pairs; writes the compacted
// stream with temporary symbols +-(temp_base + slot), the new traversal
// offsets (ntrav + 1 entries) and status->u64[2] = output length.
// heads: the stream's head bitmap; tile_trav: launch_tile_trav's table.
// Scratch: tword (apply_num_tiles(n) * 256 thread words: candidate bits and
// in-tile prefix), tile_agg and state (one u64 per tile), desc (one u64 per
// apply_state_blocks(n) block, zeroed) and a zeroed counter.
struct ApplyScratch {
  uint32_t *tword;
  unsigned long long *tile_agg, *state, *desc;
  uint32_t *counter;
};
// The three passes: candidate bits and tile aggregates (flat: one tile per
// block read straight from global memory, else persistent blocks with
// staged tiles; the same output); carried-in state of every tile; replay
// and compacted output.
void launch_apply_classify(const int32_t *s, uint64_t n, const uint32_t *heads, PairTable tab, const ApplyScratch &w,
                           bool flat, DevStatus *status, cudaStream_t st);
// The classification and emit passes from the count's slot references and
// repeated-slot bitmap (a resident stream; no table probes).  The same
// output as the probing passes.
void launch_apply_classify_sref(const uint32_t *sref, uint64_t n, const uint32_t *rep_bits, const ApplyScratch &w,
                                cudaStream_t st);
void launch_apply_emit_sref(const int32_t *s, const uint32_t *sref, uint64_t n, const uint64_t *off, uint64_t ntrav,
                            const uint64_t *tile_trav, PairTable tab, int32_t temp_base, int32_t *out,
                            uint64_t *new_off, uint32_t *used_bits, const ApplyScratch &w, DevStatus *status,
                            cudaStream_t st);
void launch_apply_states(uint64_t n, const ApplyScratch &w, DevStatus *status, cudaStream_t st);
// Emit also sets bit `slot` of used_bits (cap bits, zeroed) for every slot
// it flags used; flat = one tile per block, read from global memory.
void launch_apply_emit(const int32_t *s, uint64_t n, const uint32_t *heads, const uint64_t *off, uint64_t ntrav,
                       const uint64_t *tile_trav, PairTable tab, int32_t temp_base, int32_t *out, uint64_t *new_off,
                       uint32_t *used_bits, const ApplyScratch &w, bool flat, DevStatus *status,
                       cudaStream_t st);
uint64_t apply_num_tiles(uint64_t n);
constexpr uint64_t kApplyTile = 2048;  // steps per apply tile
// (key with the sign bit flipped, slot) of every slot set in the used bitmap
// (cap bits), in no particular order; count in status->u64[3], entries
// beyond cap_out dropped with kErrLength.
void launch_collect_used(const uint32_t *bits, uint64_t cap, PairTable tab, unsigned long long *keys_out,
                         uint32_t *slots_out, uint64_t cap_out, DevStatus *status, cudaStream_t st);
uint64_t apply_state_blocks(uint64_t n);
// ---- chunks of a stream too long for HBM ---------------------------------
// Head bitmap of positions lo .. lo + span (head_words(span) words, zeroed).
void launch_head_bits_range(const uint64_t *off, uint64_t ntrav, uint64_t lo, uint64_t span, uint32_t *bits,
                            cudaStream_t st);
// One delta round over len steps: in[0] = the step before the chunk,
// in[1 .. len] the chunk; heads chunk-relative; max |out| into *max_abs.
void launch_delta_chunk(const int32_t *in, int32_t *out, uint64_t len, const uint32_t *heads, uint32_t *max_abs,
                        cudaStream_t st);
// Classification of n_pos positions (a whole number of apply tiles unless
// the stream ends) whose words go to tiles tile0 ... of w; s holds n_data
// steps (n_pos + 1 when the stream continues).
void launch_classify_chunk(const int32_t *s, uint64_t n_pos, uint64_t n_data, const uint32_t *heads, PairTable tab,
                           uint64_t tile0, const ApplyScratch &w, DevStatus *status, cudaStream_t st);
// Emit of tiles tile0 .. tile0 + tiles - 1 of the n-step stream: s holds
// the steps from position pos_base on, out the output from output position
// out_shift on; offsets, states and words are the whole stream's.
void launch_emit_chunk(const int32_t *s, uint64_t pos_base, uint64_t tile0, uint64_t tiles, uint64_t n,
                       const uint64_t *off, uint64_t ntrav, const uint64_t *tile_trav, PairTable tab,
                       int32_t temp_base, int32_t *out, uint64_t out_shift, uint64_t *new_off, uint32_t *used_bits,
                       const ApplyScratch &w, DevStatus *status, cudaStream_t st);

// tile_trav[k] = first traversal t with off[t] >= k * (apply tile), for the
// apply_num_tiles(n) tiles.
void launch_tile_trav(const uint64_t *off, uint64_t ntrav, uint64_t n, uint64_t *tile_trav, cudaStream_t st);


// Stable LSD radix sort of (u64 key, u32 value) pairs, one launch per byte.
// launch_sort_hist: hist[b * 256 + d] (8 * 256 entries, zeroed) += keys whose
// byte b is d, for the bytes in byte_mask.  launch_sort_pass: one pass on
// byte `byte` from (keys, vals) into (keys_out, vals_out); desc holds
// sort_tiles(n) * 256 zeroed descriptors and counter one zeroed u32.
uint64_t sort_tiles(uint64_t n);
void launch_sort_hist(const unsigned long long *keys, uint64_t n, uint32_t byte_mask, uint32_t *hist,
                      cudaStream_t st);
void launch_sort_pass(const unsigned long long *keys, const uint32_t *vals, unsigned long long *keys_out,
                      uint32_t *vals_out, uint64_t n, int byte, const uint32_t *hist, unsigned long long *desc,
                      uint32_t *counter, uint32_t *err, cudaStream_t st);

// keys sorted (transformed, ascending signed order): vals[slot] = next_id + rank,
// rulebook[rank] = original key.
void launch_assign_ids(const unsigned long long *sorted_keys, const uint32_t *sorted_slots, uint64_t u,
                       uint32_t next_id, PairTable tab, long long *rulebook, cudaStream_t st);
// Rewrites temporary symbols +-(temp_base + slot) into +-slots[slot].val.
void launch_remap(int32_t *s, uint64_t n, int32_t temp_base, const PairSlot *slots, cudaStream_t st);

// ---- append encoder (add-haplotypes) -------------------------------------
// Builds a key -> rule id table from stored rule columns (rules
// [lo, hi) of the decoded columns get ids start .. start + hi - lo).
void launch_build_rule_table(const int32_t *first, const int32_t *second, uint64_t lo, uint64_t hi,
                             uint32_t start, PairTable tab, DevStatus *status, cudaStream_t st);
// Chunked stack pass (the same result as the stack encoder below): chunk c
// covers [cs[c], ce[c]) of one traversal, bit 63 of cs / ce flags the first
// / last chunk of a traversal.  Writes the stack top after every symbol and
// per-symbol flags (bit 0: the symbol did not pair, bit 1: last symbol of a
// traversal); *nonconv counts chunks whose fix-up did not settle (then the
// result is void).
constexpr uint64_t kChunkEdge = 1ull << 63;
void launch_stack_chunks(const int32_t *s, const uint64_t *cs, const uint64_t *ce, uint64_t nchunks, PairTable tab,
                         int32_t *top, uint8_t *fl, unsigned long long *nonconv, cudaStream_t st);
// keep[p] = 1 for the stack tops that are output symbols.
void launch_stack_keep(const uint8_t *fl, uint64_t n, uint32_t *keep, cudaStream_t st);
// out[pos[p]] = top[p] where keep[p] (pos: exclusive scan of keep).
void launch_stack_scatter(const int32_t *top, const uint32_t *keep, const uint64_t *pos, uint64_t n, int32_t *out,
                          cudaStream_t st);
// Stack encoder, one thread per traversal (sequential within a traversal).
// Encodes s[off[t] .. off[t] + len[t]) in place and updates len[t].
void launch_stack_encode(int32_t *s, const uint64_t *off, uint64_t *len, uint64_t ntrav, PairTable tab,
                         DevStatus *status, cudaStream_t st);

// ---- decode side ------------------------------------------------------------
// Rule expansion lengths: len[i] for rule min_id + i.  One pass resolves the
// rules of [lo, hi) (all by default) whose children are resolved;
// status->pass_open[slot] counts rules still open.
void launch_rule_len_pass(const int32_t *first, const int32_t *second, uint64_t nrules, uint32_t min_id,
                          uint32_t *rlen, DevStatus *status, int slot, cudaStream_t st,
                          uint64_t lo = 0, uint64_t hi = UINT64_MAX);
// Exclusive scan of the expansion length of every encoded symbol into
// pos[0..m] (pos[m] = total); desc/tile_counter zeroed.
void launch_symbol_positions(const int32_t *enc, uint64_t m, uint32_t min_id, uint64_t nrules,
                             const uint32_t *rlen, uint64_t *pos, unsigned long long *desc,
                             uint32_t *tile_counter, DevStatus *status, cudaStream_t st);
uint64_t scan_num_tiles(uint64_t n);
// Expands every encoded symbol into out[pos[i] ..).
void launch_expand(const int32_t *enc, uint64_t m, const uint64_t *pos, const int32_t *first,
                   const int32_t *second, uint64_t nrules, uint32_t min_id, int32_t *out, DevStatus *status,
                   cudaStream_t st);
// In-place inclusive prefix sum inside every traversal (inverse delta).
// It tiles the stream by kInverseDeltaTile steps and needs one look-back
// descriptor per tile: inverse_delta_num_tiles(n) of them.
constexpr uint64_t kInverseDeltaTile = 4096;
uint64_t inverse_delta_num_tiles(uint64_t n);
void launch_inverse_delta(int32_t *x, uint64_t n, const uint64_t *off, uint64_t ntrav,
                          unsigned long long *desc, uint32_t *tile_counter, DevStatus *status,
                          cudaStream_t st);

// GFA text of P-lines (mode 0) or W-lines (mode 1) for traversals whose
// steps are x[off[t] .. off[t+1]).  Every non-empty traversal t emits
// blob[pre_off[t] .. pre_off[t+1]) before its first step and
// blob[suf_off[t] .. suf_off[t+1]) after its last step; `tail` bytes
// (lines of trailing empty traversals) follow the last step.  The total
// text size is written to status->u64[7].  With text == nullptr only the
// size is computed.
struct TextMeta {
  const char *blob;
  const uint64_t *pre_off;  // ntrav + 1
  const uint64_t *suf_off;  // ntrav + 1
  const char *tail;
  uint64_t tail_len;
  int mode;
};
void launch_emit_text(const int32_t *x, uint64_t n, const uint64_t *off, uint64_t ntrav, TextMeta meta,
                      char *text, unsigned long long *desc, uint32_t *tile_counter, DevStatus *status,
                      cudaStream_t st);
uint64_t text_num_tiles(uint64_t n);

// Gathers encoded ranges src[starts[r] .. starts[r] + lens[r]) into dst at
// dst_off[r] (serving batches).
void launch_gather_ranges(const int32_t *src, const uint64_t *starts, const uint64_t *dst_off, uint64_t nr,
                          int32_t *dst, cudaStream_t st);

// ---- prefix-sum expansion decoder (expand_kernels.cu) ----------------------
// Rule r (id min_id + r) expands to rlen[r] steps whose inclusive prefix
// sums are rpre[roff[r] .. roff[r] + rlen[r]).
// rstat[r] = value ranges of the rule's expansion for text lengths: with
// delta_round 1 {min, max} of its prefix values and {min, max} of 0 and all
// prefix values but the last; with delta_round 0 {min, max} of its steps.
struct RulePrefixView {
  const uint32_t *rlen;
  const uint64_t *roff;  // nrules + 1
  const int32_t *rpre;
  const int4 *rstat;
  uint32_t min_id;
  uint64_t nrules;
};
// Encoded symbols expanding to output steps [0, total): symbol i covers
// [pos[i], pos[i + 1]); rec[i] = {symbol, prefix buffer base, rule length
// (0 for a plain step), S_i = sum of the expansions before it in its
// traversal}; tile_sym from launch_tile_symbols.
struct ExpandSource {
  const int4 *rec;
  const uint64_t *pos;  // m + 1
  const uint64_t *tile_sym;
  uint64_t m, total;
  RulePrefixView rules;
};
// Output traversals off[0 .. ntrav] (off[ntrav] = total), their head bitmap
// (launch_head_bits over off) and the text pieces.
struct TextSource {
  const uint64_t *off;
  uint64_t ntrav;
  const uint32_t *heads;
  TextMeta meta;
  uint64_t cap;   // bytes of the text buffer
  uint32_t *err;  // kErrLength when the text would not fit where its lengths say
};
// One build pass over the rule prefix buffer for the rules of [lo, hi) (all
// by default); built[r] = pass of rule r (0 = waiting, zero before pass 1).
// status->pass_open[slot] += rules still waiting.
void launch_rule_prefix_pass(const int32_t *first, const int32_t *second, RulePrefixView rv, int32_t *rpre,
                             int4 *rstat, int delta, uint32_t *built, uint32_t pass, DevStatus *status, int slot,
                             cudaStream_t st, uint64_t lo = 0, uint64_t hi = UINT64_MAX);
// out[0 .. n] = exclusive scan of in[0 .. n) (out[n] = total); desc: one u64
// per excl_scan_tiles(n) tile (at least one), zeroed; tile_counter zeroed.
uint64_t excl_scan_tiles(uint64_t n);
void launch_excl_scan_u32(const uint32_t *in, uint64_t n, uint64_t *out, unsigned long long *desc,
                          uint32_t *tile_counter, DevStatus *status, cudaStream_t st);
void launch_excl_scan_u64(const uint64_t *in, uint64_t n, uint64_t *out, unsigned long long *desc,
                          uint32_t *tile_counter, DevStatus *status, cudaStream_t st);
// rec[i] = {enc[i], base, length, total of its expansion} and, unless tot is
// null, tot[i] = that total; launch_symbol_exclusive then turns rec[i].w
// into incl[i] - total (incl: inclusive segmented sums of tot).
void launch_symbol_records(const int32_t *enc, uint64_t m, RulePrefixView rv, int4 *rec, int32_t *tot,
                           cudaStream_t st);
void launch_symbol_exclusive(int4 *rec, const int32_t *incl, uint64_t m, cudaStream_t st);
// Output tiles of the expansion kernels and the symbol at each tile start
// (expand_num_tiles(total) + 1 entries).
uint64_t expand_num_tiles(uint64_t total);
void launch_tile_symbols(const uint64_t *pos, uint64_t m, uint64_t total, uint64_t *tile_sym, cudaStream_t st);
// Decoded steps (delta = delta_round, 0 or 1) of every output position.
void launch_expand_steps(const ExpandSource &E, int delta, int32_t *out, cudaStream_t st);
// P/W text: slen[i] = text bytes of symbol i (with the line pieces around
// it) and sdig[i] = the digit count all its steps share (0: they differ);
// then, with soff = exclusive scan of slen, the text of every output tile.
void launch_symbol_text(const ExpandSource &E, const TextSource &T, int delta, uint64_t *slen, uint8_t *sdig,
                        cudaStream_t st);
// toff[k]: text offset of output tile k (expand_num_tiles entries), from the
// per-symbol text offsets soff and shared digit counts sdig.
void launch_tile_text_off(const ExpandSource &E, const TextSource &T, int delta, const uint64_t *soff,
                          const uint8_t *sdig, uint64_t *toff, cudaStream_t st);
// The text of output tiles [tile0, tile1) (all by default) at toff[tile];
// T.cap = the body size.
void launch_text_write(const ExpandSource &E, const TextSource &T, int delta, const uint64_t *toff, char *text,
                       cudaStream_t st, uint64_t tile0 = 0, uint64_t tile1 = UINT64_MAX);
// Adds the number of '\n' bytes in text[0, n) (16-byte aligned buffer) to
// out[0] (zero it first); out[1 .. min(count, cap)] = their positions,
// unordered.
void launch_find_newlines(const char *text, uint64_t n, unsigned long long *out, uint64_t cap, cudaStream_t st);

// ---------------------------------------------------------------------------
// GFA front end (parse_kernels.cu).  The text buffer holds the file's n
// bytes padded with zeros to a multiple of 16 bytes; work runs in tiles of
// 4 KB (parse_num_tiles).
// ---------------------------------------------------------------------------
// One P or W line: its steps / walk field [fstart, fend) and the index of
// its first step in the P or W output.
struct PWLine {
  uint64_t fstart;
  unsigned long long fend;
  uint64_t out;
  uint32_t kind;  // 0 = P, 1 = W
  uint32_t pad;
};
// Segment-name lookup: slots == nullptr resolves names as decimal numbers;
// otherwise slots[mask + 1] hold the ids of the names (linear probing) and
// name id sits at text[noff[id] .. + nlen[id]).
struct NameIndex {
  const uint32_t *slots;
  uint64_t mask;
  const uint64_t *noff;
  const uint32_t *nlen;
};
// Error codes in the low two bits of the front end's error word (the
// smallest of W << 62 | byte position << 2 | code over the file).
constexpr uint32_t kParseNoDigits = 1;  // parse_uint32: no digits
constexpr uint32_t kParseOverflow = 2;  // parse_uint32: overflow

// ---------------------------------------------------------------------------
// S and L line text (static_kernels.cu)
// ---------------------------------------------------------------------------
struct StaticTextSource {
  int kind;  // 0 = S lines, 1 = L lines
  uint64_t n;
  // S: sequences back to back; seq_off = exclusive scan of seg_len
  const char *seq;
  const uint64_t *seq_off;
  const uint32_t *seg_len;
  // L: from / to ids and orientations, overlap number and operation (0: '*')
  const uint32_t *lf, *lt, *lnum;
  const char *lfo, *lto, *lop;
  // per-line optional-field text ex[ex_off[i] .. ex_off[i+1]) or none (null)
  const char *ex;
  const uint64_t *ex_off;
};
// len[i] = the byte length of line i.
void launch_static_len(const StaticTextSource &S, uint64_t *len, cudaStream_t st);
// The lines at out[loff[i] ..] (loff: exclusive scan of len, total bytes;
// out 16-byte aligned).
void launch_static_write(const StaticTextSource &S, const uint64_t *loff, uint64_t total, char *out,
                         cudaStream_t st);

// ---------------------------------------------------------------------------
// Pangenome growth (growth_kernels.cu)
// ---------------------------------------------------------------------------
// Bit (g & 63) of word (g >> 6) - w0 of node |x[p]|'s row (rows of w1 - w0
// words, node ids 1 .. num_nodes; others skipped) for every step p of a
// traversal t whose group g = gid[t] has g >> 6 in [w0, w1).
void launch_cover_bits(const int32_t *x, uint64_t n, const uint64_t *off, uint64_t ntrav, const uint32_t *gid,
                       uint64_t num_nodes, uint32_t w0, uint32_t w1, unsigned long long *bits, cudaStream_t st);
// cov[v] += bits set in row v (stride words), v = 1 .. num_nodes.
void launch_cover_count(const unsigned long long *bits, uint64_t num_nodes, uint32_t stride, uint32_t *cov,
                        cudaStream_t st);
// hist[c] += nodes v = 1 .. num_nodes with cov[v] == c, c <= nh (zeroed first).
void launch_cover_hist(const uint32_t *cov, uint64_t num_nodes, uint32_t nh, unsigned long long *hist,
                       cudaStream_t st);

uint64_t parse_num_tiles(uint64_t n);
// cnt[tile] = '\n' bytes in the tile.
void launch_nl_count(const char *text, uint64_t n, uint32_t *cnt, cudaStream_t st);
// eol[nl_off[tile] + j] = position of the tile's j-th '\n' (nl_off: the
// exclusive scan of cnt).
void launch_nl_write(const char *text, uint64_t n, const uint64_t *nl_off, uint64_t *eol, cudaStream_t st);
// Line i = [i ? eol[i-1] + 1 : 0, i < nl ? eol[i] : n): type[i] = its first
// byte (0 when empty), ispw[i] = whether it is a P or W line.
void launch_line_heads(const char *text, uint64_t n, const uint64_t *eol, uint64_t nl, uint64_t nlines,
                       uint8_t *type, uint32_t *ispw, cudaStream_t st);
// pw[slotoff[i]] for every P/W line i (slotoff: exclusive scan of ispw):
// fstart after the leading fields, fend = the line end, out = ~0.
void launch_line_fields(const char *text, uint64_t n, const uint64_t *eol, uint64_t nl, uint64_t nlines,
                        const uint8_t *type, const uint64_t *slotoff, PWLine *pw, cudaStream_t st);
// fend lowered to the first blank at or after fstart.
void launch_field_ends(const char *text, uint64_t n, const uint64_t *nl_off, uint64_t nlines, const uint64_t *slotoff,
                       PWLine *pw, cudaStream_t st);
// Per-tile counts of the kept P and W steps; numeric parse errors to *err
// (set it to ~0 first).
void launch_token_count(const char *text, uint64_t n, const uint64_t *nl_off, uint64_t nlines,
                        const uint64_t *slotoff, PWLine *pw, const NameIndex &ni, uint32_t *cntP, uint32_t *cntW,
                        unsigned long long *err, cudaStream_t st);
// The kept steps at offP / offW (exclusive scans of the counts) and every
// P/W line's pw[].out.
void launch_token_write(const char *text, uint64_t n, const uint64_t *nl_off, uint64_t nlines,
                        const uint64_t *slotoff, PWLine *pw, const NameIndex &ni, const uint64_t *offP,
                        const uint64_t *offW, int32_t *outP, int32_t *outW, unsigned long long *err, cudaStream_t st);
// Inserts names 1 .. nnames (NameIndex layout) into slots (zeroed).
void launch_name_table(const char *text, const uint64_t *noff, const uint32_t *nlen, uint64_t nnames,
                       uint32_t *slots, uint64_t mask, cudaStream_t st);

}  // namespace gfz

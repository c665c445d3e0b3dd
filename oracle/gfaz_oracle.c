/*
 * gfaz_oracle.c - CPU restatement of the GFAz transform hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * path and the timed CPU baseline ("port") of bench.py.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the
 * product library never links, loads or calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks this restatement
 * against golden vectors that the reference CLI (built from its own sources
 * by oracle/build_ref.sh) produced for the fixtures in tests/golden/.
 *
 * What it restates (reference file:line):
 *   delta encode + max |x|   src/codec/codec.cpp:45-76,
 *                            src/workflows/compression_workflow.cpp:217-265
 *   2-mer packing            include/grammar/packed_2mer.hpp:15-48
 *   candidate discovery      src/grammar/rule_generator.cpp:148-260
 *   stack encoder            src/grammar/path_encoder.cpp:13-84
 *   used-rule sort + remap   src/workflows/compression_workflow.cpp:548-700,
 *                            src/workflows/compression_utils.cpp:201-221
 *   rule columns             src/workflows/compression_utils.cpp:165-193
 *   expansion                src/workflows/decompression_workflow.cpp:70-106
 *   inverse delta            src/codec/codec.cpp:29-41
 *   P/W text                 src/io/gfa_write_utils.cpp:238-290
 *   append encoding          src/workflows/add_haplotypes_workflow.cpp:336-379
 *
 * Traversals are passed flattened: steps[offsets[t] .. offsets[t+1]).  The
 * reference counts pairs over P traversals then W traversals into one set
 * and encodes each traversal independently, so one concatenated traversal
 * list (paths first) is equivalent.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* 2-mer helpers (packed_2mer.hpp:15-48).  Negation wraps like int32. */

static inline int32_t neg32(int32_t x) { return (int32_t)(0u - (uint32_t)x); }
static inline uint32_t abs32(int32_t x) { return x < 0 ? (uint32_t)0u - (uint32_t)x : (uint32_t)x; }
static inline int64_t pack2(int32_t a, int32_t b) {
  return (int64_t)(((uint64_t)(uint32_t)a << 32) | (uint64_t)(uint32_t)b);
}
static inline int32_t first_of(int64_t k) { return (int32_t)(uint32_t)((uint64_t)k >> 32); }
static inline int32_t second_of(int64_t k) { return (int32_t)(uint32_t)(uint64_t)k; }
static inline int64_t rev2(int64_t k) { return pack2(neg32(second_of(k)), neg32(first_of(k))); }
static inline int64_t canon2(int64_t k) { int64_t r = rev2(k); return k < r ? k : r; }

/* pack(1,1) is never canonical (its reverse pack(-1,-1) is smaller), so it
 * can mark empty slots of tables that only ever hold canonical keys. */
#define ORC_EMPTY ((int64_t)0x0000000100000001LL)

static inline uint64_t mix64(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33; return x;
}

/* ------------------------------------------------------------------ */
/* Growable open-addressed set / map of canonical int64 keys.          */

typedef struct {
  int64_t *keys;
  uint32_t *vals;
  uint64_t cap, size;
} orc_table;

static void tab_init(orc_table *t, uint64_t cap_hint) {
  uint64_t cap = 1024;
  while (cap < cap_hint * 2) cap <<= 1;
  t->cap = cap; t->size = 0;
  t->keys = (int64_t *)malloc(cap * sizeof(int64_t));
  t->vals = (uint32_t *)calloc(cap, sizeof(uint32_t));
  for (uint64_t i = 0; i < cap; ++i) t->keys[i] = ORC_EMPTY;
}
static void tab_free(orc_table *t) { free(t->keys); free(t->vals); t->keys = NULL; t->vals = NULL; }

static int64_t tab_find(const orc_table *t, int64_t k) {
  /* forward lookups of non-canonical pairs may equal the empty marker */
  if (k == ORC_EMPTY) return -1;
  uint64_t m = t->cap - 1, h = mix64((uint64_t)k) & m;
  for (;;) {
    if (t->keys[h] == k) return (int64_t)h;
    if (t->keys[h] == ORC_EMPTY) return -1;
    h = (h + 1) & m;
  }
}
static void tab_grow(orc_table *t);
/* returns slot; *inserted=1 when the key was new */
static uint64_t tab_insert(orc_table *t, int64_t k, int *inserted) {
  if ((t->size + 1) * 10 > t->cap * 7) tab_grow(t);
  uint64_t m = t->cap - 1, h = mix64((uint64_t)k) & m;
  for (;;) {
    if (t->keys[h] == k) { *inserted = 0; return h; }
    if (t->keys[h] == ORC_EMPTY) { t->keys[h] = k; t->size++; *inserted = 1; return h; }
    h = (h + 1) & m;
  }
}
static void tab_grow(orc_table *t) {
  orc_table n; tab_init(&n, t->cap);
  for (uint64_t i = 0; i < t->cap; ++i)
    if (t->keys[i] != ORC_EMPTY) { int ins; uint64_t s = tab_insert(&n, t->keys[i], &ins); n.vals[s] = t->vals[i]; }
  tab_free(t); *t = n;
}

static int resolve_threads(int threads) {
#ifdef _OPENMP
  if (threads > 0) return threads;
  return omp_get_max_threads();
#else
  (void)threads; return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* Delta encoding (codec.cpp:45-76; compression_workflow.cpp:217-265). */

/* One delta round over every traversal, back to front; returns the max |x|
 * over all elements after the round, first elements included. */
static uint32_t delta_round_once(int32_t *steps, const uint64_t *off, uint64_t ntrav, int threads) {
  uint32_t mx = 0;
#pragma omp parallel for schedule(dynamic) reduction(max : mx) num_threads(threads)
  for (int64_t t = 0; t < (int64_t)ntrav; ++t) {
    uint64_t b = off[t], e = off[t + 1];
    if (e == b) continue;
    uint32_t local = abs32(steps[b]);
    for (uint64_t i = e - 1; i > b; --i) {
      steps[i] = (int32_t)((uint32_t)steps[i] - (uint32_t)steps[i - 1]);
      uint32_t a = abs32(steps[i]);
      if (a > local) local = a;
    }
    if (local > mx) mx = local;
  }
  return mx;
}

/* Applies delta_round rounds in place and returns the seed for rule IDs
 * (next_id = max_abs + 1, or max |raw| + 1 when delta_round == 0).
 * Returns 0 (an impossible seed) when max_abs == UINT32_MAX, where the
 * reference throws. */
uint32_t orc_delta_encode(int32_t *steps, const uint64_t *off, uint64_t ntrav, int delta_round, int threads) {
  threads = resolve_threads(threads);
  uint32_t max_abs = 0;
  if (delta_round < 0) delta_round = 0;
  if (delta_round == 0) {
#pragma omp parallel for schedule(static) reduction(max : max_abs) num_threads(threads)
    for (int64_t i = 0; i < (int64_t)off[ntrav]; ++i) {
      uint32_t a = abs32(steps[i]);
      if (a > max_abs) max_abs = a;
    }
  }
  for (int r = 0; r < delta_round; ++r) {
    uint32_t m = delta_round_once(steps, off, ntrav, threads);
    if (m > max_abs) max_abs = m;
  }
  if (max_abs == UINT32_MAX) return 0;
  return max_abs + 1;
}

/* Inverse delta (codec.cpp:29-41), delta_round times. */
void orc_delta_decode(int32_t *steps, const uint64_t *off, uint64_t ntrav, int delta_round, int threads) {
  threads = resolve_threads(threads);
  for (int r = 0; r < delta_round; ++r) {
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (int64_t t = 0; t < (int64_t)ntrav; ++t)
      for (uint64_t i = off[t] + 1; i < off[t + 1]; ++i)
        steps[i] = (int32_t)((uint32_t)steps[i] + (uint32_t)steps[i - 1]);
  }
}

/* ------------------------------------------------------------------ */
/* Candidate discovery (rule_generator.cpp:148-260): canonical pairs seen
 * twice or more, overlapping occurrences counted, never across traversals.
 * Per-thread seen/repeated sets, then a serial merge, like the reference. */

static void find_candidates(const int32_t *s, const uint64_t *off, uint64_t ntrav, int threads,
                            orc_table *cand /* out: keys of candidates, vals = temp id */) {
  orc_table *seen = (orc_table *)malloc(sizeof(orc_table) * threads);
  orc_table *rep = (orc_table *)malloc(sizeof(orc_table) * threads);
  for (int i = 0; i < threads; ++i) { tab_init(&seen[i], 1 << 12); tab_init(&rep[i], 1 << 12); }
#pragma omp parallel num_threads(threads)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    orc_table *ls = &seen[tid], *lr = &rep[tid];
#pragma omp for schedule(dynamic)
    for (int64_t t = 0; t < (int64_t)ntrav; ++t) {
      uint64_t b = off[t], e = off[t + 1];
      if (e - b < 2) continue;
      for (uint64_t i = b; i + 1 < e; ++i) {
        int64_t k = canon2(pack2(s[i], s[i + 1]));
        if (tab_find(lr, k) >= 0) continue;
        if (tab_find(ls, k) >= 0) { int ins; tab_insert(lr, k, &ins); }
        else { int ins; tab_insert(ls, k, &ins); }
      }
    }
  }
  orc_table gseen; tab_init(&gseen, 1 << 12);
  tab_init(cand, 1 << 12);
  for (int t = 0; t < threads; ++t) {
    for (uint64_t i = 0; i < rep[t].cap; ++i)
      if (rep[t].keys[i] != ORC_EMPTY) { int ins; tab_insert(cand, rep[t].keys[i], &ins); }
    for (uint64_t i = 0; i < seen[t].cap; ++i) {
      int64_t k = seen[t].keys[i];
      if (k == ORC_EMPTY) continue;
      if (tab_find(cand, k) >= 0) continue;
      if (tab_find(&gseen, k) >= 0) { int ins; tab_insert(cand, k, &ins); }
      else { int ins; tab_insert(&gseen, k, &ins); }
    }
  }
  for (int i = 0; i < threads; ++i) { tab_free(&seen[i]); tab_free(&rep[i]); }
  free(seen); free(rep); tab_free(&gseen);
}

/* ------------------------------------------------------------------ */
/* Stack encoder (path_encoder.cpp:13-84).  Pushes each symbol; when the
 * top two form a rule key (forward -> +id, else reverse -> -id) they are
 * replaced by the rule symbol and the rule is marked used.  The top pair
 * is re-checked after every push, so a rule symbol can cascade into a
 * later layer's rule when the table holds several layers (append path). */

static uint64_t stack_encode(int32_t *seq, uint64_t n, const orc_table *rules, uint32_t rules_start,
                             uint8_t *used, uint64_t nrules) {
  uint64_t top = 0; /* stack lives in seq[0..top) since top <= i always */
  for (uint64_t i = 0; i < n; ++i) {
    seq[top++] = seq[i];
    if (top >= 2) {
      int32_t a = seq[top - 2], b = seq[top - 1];
      int64_t k = pack2(a, b);
      int64_t slot = tab_find(rules, k);
      int32_t sym = 0; int found = 0;
      if (slot >= 0) { sym = (int32_t)rules->vals[slot]; found = 1; }
      else {
        slot = tab_find(rules, rev2(k));
        if (slot >= 0) { sym = neg32((int32_t)rules->vals[slot]); found = 1; }
      }
      if (found) {
        top -= 2;
        seq[top++] = sym;
        uint32_t id = rules->vals[slot];
        if (used && (uint64_t)(id - rules_start) < nrules) used[id - rules_start] = 1;
      }
    }
  }
  return top;
}

static int cmp_i64(const void *x, const void *y) {
  int64_t a = *(const int64_t *)x, b = *(const int64_t *)y;
  return (a > b) - (a < b);
}

/* ------------------------------------------------------------------ */
/* Full grammar stage on already delta-coded traversals
 * (compression_workflow.cpp:548-700).
 *
 * steps/off: delta-coded traversals (paths then walks).  On return the
 * encoded traversals are compacted back to back in steps[] and
 * out_off[0..ntrav] holds their offsets.  rules_out receives the packed
 * rulebook (index = id - layer_start) and the function returns the number
 * of rules, or -1 when rules_cap is too small.  next_id is the seed on
 * entry and the high-water mark on exit. */
int64_t orc_grammar(int32_t *steps, const uint64_t *off, uint64_t ntrav, int rounds,
                    uint32_t *next_id, uint64_t *out_off, int64_t *rules_out, uint64_t rules_cap,
                    int *rounds_done, int threads) {
  threads = resolve_threads(threads);
  uint64_t *cur = (uint64_t *)malloc((ntrav + 1) * sizeof(uint64_t));
  memcpy(cur, off, (ntrav + 1) * sizeof(uint64_t));
  uint64_t *lens = (uint64_t *)malloc((ntrav + 1) * sizeof(uint64_t));
  uint64_t nrules = 0;
  int done = 0;
  for (int round = 0; round < rounds; ++round) {
    orc_table cand;
    find_candidates(steps, cur, ntrav, threads, &cand);
    if (cand.size == 0) { tab_free(&cand); break; }
    done++;
    /* temp ids in slot order: start + rank in table order (any order works;
     * final ids come from the sort below) */
    uint32_t start = *next_id;
    int64_t *tmp_key = (int64_t *)malloc(cand.size * sizeof(int64_t));
    uint64_t ti = 0;
    for (uint64_t i = 0; i < cand.cap; ++i)
      if (cand.keys[i] != ORC_EMPTY) { cand.vals[i] = start + (uint32_t)ti; tmp_key[ti++] = cand.keys[i]; }
    uint64_t nc = cand.size;
    uint8_t *used = (uint8_t *)calloc(nc, 1);
#pragma omp parallel for schedule(dynamic) num_threads(threads)
    for (int64_t t = 0; t < (int64_t)ntrav; ++t) {
      uint64_t n = cur[t + 1] - cur[t];
      lens[t] = stack_encode(steps + cur[t], n, &cand, start, used, nc);
    }
    /* keep used rules, sort by signed key, id_map temp -> final */
    uint64_t nu = 0;
    for (uint64_t i = 0; i < nc; ++i) nu += used[i];
    if (nu == 0) {
      /* traversals are unchanged when nothing was used */
      free(tmp_key); free(used); tab_free(&cand);
      break;
    }
    int64_t *uk = (int64_t *)malloc(nu * sizeof(int64_t));
    uint64_t u = 0;
    for (uint64_t i = 0; i < nc; ++i) if (used[i]) uk[u++] = tmp_key[i];
    qsort(uk, nu, sizeof(int64_t), cmp_i64);
    uint32_t *id_map = (uint32_t *)calloc(nc, sizeof(uint32_t));
    for (uint64_t r = 0; r < nu; ++r) {
      int64_t slot = tab_find(&cand, uk[r]);
      id_map[cand.vals[slot] - start] = *next_id + (uint32_t)r;
    }
    /* compact traversals and remap temp ids (compression_utils.cpp:201-221) */
    uint64_t *noff = (uint64_t *)malloc((ntrav + 1) * sizeof(uint64_t));
    noff[0] = 0;
    for (uint64_t t = 0; t < ntrav; ++t) noff[t + 1] = noff[t] + lens[t];
    for (uint64_t t = 0; t < ntrav; ++t) {
      int32_t *src = steps + cur[t];
      int32_t *dst = steps + noff[t];
      for (uint64_t i = 0; i < lens[t]; ++i) {
        int32_t x = src[i];
        uint32_t a = abs32(x);
        if (a >= start && (uint64_t)(a - start) < nc && id_map[a - start] != 0) {
          int32_t y = (int32_t)id_map[a - start];
          x = x > 0 ? y : neg32(y);
        }
        dst[i] = x;
      }
    }
    if (nrules + nu > rules_cap) {
      free(uk); free(id_map); free(noff); free(tmp_key); free(used); tab_free(&cand);
      free(cur); free(lens);
      return -1;
    }
    memcpy(rules_out + nrules, uk, nu * sizeof(int64_t));
    nrules += nu;
    *next_id += (uint32_t)nu;
    memcpy(cur, noff, (ntrav + 1) * sizeof(uint64_t));
    free(uk); free(id_map); free(noff); free(tmp_key); free(used); tab_free(&cand);
  }
  memcpy(out_off, cur, (ntrav + 1) * sizeof(uint64_t));
  if (rounds_done) *rounds_done = done;
  free(cur); free(lens);
  return (int64_t)nrules;
}

/* Rule columns (compression_utils.cpp:165-193 + codec.cpp:79-86): split the
 * packed keys into first/second and delta-code each column. */
void orc_rule_columns(const int64_t *rules, uint64_t n, int32_t *first, int32_t *second) {
  for (uint64_t i = 0; i < n; ++i) { first[i] = first_of(rules[i]); second[i] = second_of(rules[i]); }
  for (uint64_t i = n; i-- > 1;) {
    first[i] = (int32_t)((uint32_t)first[i] - (uint32_t)first[i - 1]);
    second[i] = (int32_t)((uint32_t)second[i] - (uint32_t)second[i - 1]);
  }
}

/* ------------------------------------------------------------------ */
/* Append encoding with an existing rulebook
 * (add_haplotypes_workflow.cpp:336-379, 447-465): one stack-encoder pass
 * per stored layer over each delta-coded traversal.  The layers are given
 * as [start_id, end_id) ranges over the decoded rule columns. */
int orc_append_encode(int32_t *steps, const uint64_t *off, uint64_t ntrav, uint64_t *out_len,
                      const int32_t *first, const int32_t *second, uint64_t nrules,
                      const uint32_t *layer_start, const uint32_t *layer_end,
                      const uint64_t *layer_flat_off, const int32_t *layer_k, int nlayers) {
  for (uint64_t t = 0; t < ntrav; ++t) out_len[t] = off[t + 1] - off[t];
  for (int l = 0; l < nlayers; ++l) {
    orc_table tab; uint32_t cnt = layer_end[l] - layer_start[l];
    tab_init(&tab, cnt + 16);
    uint64_t base = layer_k[l] == 0 ? 0 : layer_flat_off[l] / (uint64_t)layer_k[l];
    for (uint32_t i = 0; i < cnt; ++i) {
      uint64_t idx = base + i;
      if (idx >= nrules) { tab_free(&tab); return -1; }
      int ins; uint64_t s = tab_insert(&tab, pack2(first[idx], second[idx]), &ins);
      /* emplace keeps the first mapping when keys repeat */
      if (ins) tab.vals[s] = layer_start[l] + i;
    }
    for (uint64_t t = 0; t < ntrav; ++t)
      out_len[t] = stack_encode(steps + off[t], out_len[t], &tab, layer_start[l], NULL, 0);
    tab_free(&tab);
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* Expansion (decompression_workflow.cpp:70-106) + inverse delta.       */

static uint64_t expand_sym(int32_t v, const int32_t *first, const int32_t *second, uint32_t min_id,
                           uint32_t max_id, int32_t *out, uint64_t pos) {
  uint32_t a = abs32(v);
  if (!(a >= min_id && a < max_id)) { out[pos] = v; return pos + 1; }
  int rev = v < 0;
  int32_t x = first[a - min_id], y = second[a - min_id];
  if (!rev) {
    pos = expand_sym(x, first, second, min_id, max_id, out, pos);
    pos = expand_sym(y, first, second, min_id, max_id, out, pos);
  } else {
    pos = expand_sym(neg32(y), first, second, min_id, max_id, out, pos);
    pos = expand_sym(neg32(x), first, second, min_id, max_id, out, pos);
  }
  return pos;
}

/* Expands every traversal into out[] at out_off[t] (taken from the stored
 * original lengths) and applies delta_round inverse deltas.  Returns -1 if
 * a traversal expands to a different length than out_off gives. */
int orc_expand(const int32_t *enc, const uint64_t *enc_off, uint64_t ntrav, const int32_t *first,
               const int32_t *second, uint64_t nrules, uint32_t min_id, int delta_round,
               int32_t *out, const uint64_t *out_off, int threads) {
  threads = resolve_threads(threads);
  uint32_t max_id = min_id + (uint32_t)nrules;
  int bad = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : bad) num_threads(threads)
  for (int64_t t = 0; t < (int64_t)ntrav; ++t) {
    uint64_t pos = out_off[t];
    for (uint64_t i = enc_off[t]; i < enc_off[t + 1]; ++i) {
      if (pos > out_off[t + 1]) { bad = 1; break; }
      pos = expand_sym(enc[i], first, second, min_id, max_id, out, pos);
    }
    if (pos != out_off[t + 1]) bad = 1;
  }
  if (bad) return -1;
  orc_delta_decode(out, out_off, ntrav, delta_round, threads);
  return 0;
}

/* ------------------------------------------------------------------ */
/* P/W line text (gfa_write_utils.cpp:238-290).  With out == NULL only the
 * size is returned.  Strings are given as concatenated bytes + offsets. */

static inline int u32_to_dec(uint32_t v, char *buf) {
  char tmp[16]; int n = 0;
  do { tmp[n++] = (char)('0' + v % 10); v /= 10; } while (v);
  for (int i = 0; i < n; ++i) buf[i] = tmp[n - 1 - i];
  return n;
}
static inline int i64_to_dec(int64_t v, char *buf) {
  char tmp[24]; int n = 0; uint64_t u; int neg = v < 0;
  u = neg ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
  do { tmp[n++] = (char)('0' + u % 10); u /= 10; } while (u);
  int k = 0;
  if (neg) buf[k++] = '-';
  for (int i = 0; i < n; ++i) buf[k++] = tmp[n - 1 - i];
  return k;
}

static uint64_t put(char *out, uint64_t pos, const char *s, uint64_t n) {
  if (out) memcpy(out + pos, s, n);
  return pos + n;
}

uint64_t orc_format_p_lines(const int32_t *steps, const uint64_t *off, uint64_t ntrav,
                            const char *names, const uint64_t *name_off,
                            const char *overlaps, const uint64_t *ov_off, char *out) {
  uint64_t pos = 0; char buf[24];
  for (uint64_t t = 0; t < ntrav; ++t) {
    pos = put(out, pos, "P\t", 2);
    pos = put(out, pos, names + name_off[t], name_off[t + 1] - name_off[t]);
    pos = put(out, pos, "\t", 1);
    for (uint64_t i = off[t]; i < off[t + 1]; ++i) {
      if (i > off[t]) pos = put(out, pos, ",", 1);
      int32_t v = steps[i];
      int n = u32_to_dec(abs32(v), buf);
      buf[n++] = v < 0 ? '-' : '+';
      pos = put(out, pos, buf, (uint64_t)n);
    }
    pos = put(out, pos, "\t", 1);
    if (ov_off[t + 1] == ov_off[t]) pos = put(out, pos, "*", 1);
    else pos = put(out, pos, overlaps + ov_off[t], ov_off[t + 1] - ov_off[t]);
    pos = put(out, pos, "\n", 1);
  }
  return pos;
}

uint64_t orc_format_w_lines(const int32_t *steps, const uint64_t *off, uint64_t ntrav,
                            const char *samples, const uint64_t *sample_off,
                            const uint32_t *haps, const char *seqids, const uint64_t *seqid_off,
                            const int64_t *starts, const int64_t *ends, char *out) {
  uint64_t pos = 0; char buf[32];
  for (uint64_t t = 0; t < ntrav; ++t) {
    int n;
    pos = put(out, pos, "W\t", 2);
    pos = put(out, pos, samples + sample_off[t], sample_off[t + 1] - sample_off[t]);
    pos = put(out, pos, "\t", 1);
    n = u32_to_dec(haps[t], buf); pos = put(out, pos, buf, (uint64_t)n);
    pos = put(out, pos, "\t", 1);
    pos = put(out, pos, seqids + seqid_off[t], seqid_off[t + 1] - seqid_off[t]);
    pos = put(out, pos, "\t", 1);
    if (starts[t] >= 0) { n = i64_to_dec(starts[t], buf); pos = put(out, pos, buf, (uint64_t)n); }
    else pos = put(out, pos, "*", 1);
    pos = put(out, pos, "\t", 1);
    if (ends[t] >= 0) { n = i64_to_dec(ends[t], buf); pos = put(out, pos, buf, (uint64_t)n); }
    else pos = put(out, pos, "*", 1);
    pos = put(out, pos, "\t", 1);
    for (uint64_t i = off[t]; i < off[t + 1]; ++i) {
      int32_t v = steps[i];
      buf[0] = v < 0 ? '<' : '>';
      n = 1 + u32_to_dec(abs32(v), buf + 1);
      pos = put(out, pos, buf, (uint64_t)n);
    }
    pos = put(out, pos, "\n", 1);
  }
  return pos;
}

/* ------------------------------------------------------------------ */
/* Whole CPU transform for the baseline timing: delta + grammar + rule
 * columns, then expansion + inverse delta + P-line text, on one batch of
 * traversals.  Returns the text size, or 0 on failure.  Scratch is
 * allocated here and released before returning. */
static double wall_ms(void) {
#ifdef _OPENMP
  return omp_get_wtime() * 1e3;
#else
  return 0.0;
#endif
}

uint64_t orc_roundtrip_p(const int32_t *raw, const uint64_t *off, uint64_t ntrav, int rounds,
                         int delta_round, char *text_out, uint64_t text_cap, int threads,
                         uint64_t *enc_len_out, uint64_t *nrules_out, double *phase_ms,
                         int32_t *enc_out, uint64_t *enc_off_out, int64_t *rules_out) {
  /* phase_ms (optional): [0] delta + grammar + rule columns, [1] expansion +
   * inverse delta + P text, wall-clock milliseconds.  enc_out (n entries),
   * enc_off_out (ntrav + 1) and rules_out (n entries), when given, receive
   * the grammar: encoded stream, its offsets and the packed rulebook. */
  threads = resolve_threads(threads);
  const double t_start = wall_ms();
  uint64_t n = off[ntrav];
  int32_t *s = (int32_t *)malloc((n ? n : 1) * sizeof(int32_t));
  memcpy(s, raw, n * sizeof(int32_t));
  uint32_t next_id = orc_delta_encode(s, off, ntrav, delta_round, threads);
  if (next_id == 0) { free(s); return 0; }
  uint32_t layer_start = next_id;
  uint64_t *eoff = (uint64_t *)malloc((ntrav + 1) * sizeof(uint64_t));
  uint64_t cap = n + 1;
  int64_t *rules = (int64_t *)malloc(cap * sizeof(int64_t));
  int rd = 0;
  int64_t nr = orc_grammar(s, off, ntrav, rounds, &next_id, eoff, rules, cap, &rd, threads);
  if (nr < 0) { free(s); free(eoff); free(rules); return 0; }
  int32_t *f = (int32_t *)malloc((nr ? nr : 1) * sizeof(int32_t));
  int32_t *g = (int32_t *)malloc((nr ? nr : 1) * sizeof(int32_t));
  orc_rule_columns(rules, (uint64_t)nr, f, g);
  const double t_mid = wall_ms();
  /* decode side: undo the column deltas, expand, inverse delta, text */
  for (int64_t i = 1; i < nr; ++i) {
    f[i] = (int32_t)((uint32_t)f[i] + (uint32_t)f[i - 1]);
    g[i] = (int32_t)((uint32_t)g[i] + (uint32_t)g[i - 1]);
  }
  int32_t *x = (int32_t *)malloc((n ? n : 1) * sizeof(int32_t));
  int rc = orc_expand(s, eoff, ntrav, f, g, (uint64_t)nr, layer_start, delta_round, x, off, threads);
  uint64_t size = 0;
  if (rc == 0) {
    /* text per traversal in parallel, then placed in order */
    uint64_t *tsz = (uint64_t *)malloc((ntrav + 1) * sizeof(uint64_t));
    char nm[32];
    uint64_t zero2[2] = {0, 0};
#pragma omp parallel for schedule(dynamic) num_threads(threads) private(nm)
    for (int64_t t = 0; t < (int64_t)ntrav; ++t) {
      int k = snprintf(nm, sizeof nm, "p%lld", (long long)t);
      uint64_t no[2] = {0, (uint64_t)k};
      uint64_t o2[2] = {0, off[t + 1] - off[t]};
      tsz[t] = orc_format_p_lines(x + off[t], o2, 1, nm, no, "", zero2, NULL);
    }
    uint64_t acc = 0;
    for (uint64_t t = 0; t < ntrav; ++t) { uint64_t v = tsz[t]; tsz[t] = acc; acc += v; }
    tsz[ntrav] = acc;
    /* the text is always produced (into a scratch buffer when the caller
     * passes none) so the timed work matches a real decompression */
    char *dst = text_out;
    if (!dst || acc > text_cap) dst = (char *)malloc(acc ? acc : 1);
    {
#pragma omp parallel for schedule(dynamic) num_threads(threads) private(nm)
      for (int64_t t = 0; t < (int64_t)ntrav; ++t) {
        int k = snprintf(nm, sizeof nm, "p%lld", (long long)t);
        uint64_t no[2] = {0, (uint64_t)k};
        uint64_t o2[2] = {0, off[t + 1] - off[t]};
        orc_format_p_lines(x + off[t], o2, 1, nm, no, "", zero2, dst + tsz[t]);
      }
    }
    if (dst != text_out) free(dst);
    size = acc;
    free(tsz);
  }
  if (phase_ms) {
    phase_ms[0] = t_mid - t_start;
    phase_ms[1] = wall_ms() - t_mid;
  }
  if (enc_len_out) *enc_len_out = eoff[ntrav];
  if (nrules_out) *nrules_out = (uint64_t)nr;
  if (enc_out) memcpy(enc_out, s, eoff[ntrav] * sizeof(int32_t));
  if (enc_off_out) memcpy(enc_off_out, eoff, (ntrav + 1) * sizeof(uint64_t));
  if (rules_out) memcpy(rules_out, rules, (uint64_t)nr * sizeof(int64_t));
  free(s); free(eoff); free(rules); free(f); free(g); free(x);
  return size;
}

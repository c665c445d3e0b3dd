/*
 * gfaz_gb300.h - C ABI of the GB300 GFAz transform library (libgfaz_gb300.so).
 *
 * Plain C: opaque handles, plain pointers and sizes, integer status codes.
 * No exception crosses the boundary; on failure a function returns a
 * negative gfz_status and gfz_last_error() gives the message (thread-local),
 * which carries the same prefixes as the reference's exceptions
 * ("GFAZ serialization error: ", "Extraction workflow error: ", ...).
 *
 * Each entry point names the reference interface it replaces (file:line in
 * the babyplutokurt/GFAz sources).  Traversal transforms (delta coding,
 * grammar rounds, expansion, inverse delta, P/W text) run on the GPU; there
 * is no CPU fallback and calls fail with GFZ_ERR_CUDA when no GPU is usable.
 * Host-only entry points (container I/O, inspection) work without a GPU.
 *
 * Buffers returned through `char **out` / `void **out` are allocated by the
 * library and released with gfz_free().
 */
#ifndef GFAZ_GB300_H
#define GFAZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GFZ_OK = 0,
  GFZ_ERR_INVALID = -1,   /* bad argument */
  GFZ_ERR_IO = -2,        /* file cannot be opened / read / written */
  GFZ_ERR_FORMAT = -3,    /* malformed .gfaz / GFA / append file */
  GFZ_ERR_CUDA = -4,      /* CUDA runtime failure or no usable GPU */
  GFZ_ERR_DEVICE = -5,    /* a kernel reported an error (table full, timeout ...) */
  GFZ_ERR_NOT_FOUND = -6, /* requested path / walk does not exist */
  GFZ_ERR_BUFFER = -7,    /* caller buffer too small (*size holds the need) */
  GFZ_ERR_INTERNAL = -8
} gfz_status;

#define GFZ_WHERE_HOST 0
#define GFZ_WHERE_DEVICE 1
#define GFZ_P_LINES 0
#define GFZ_W_LINES 1

typedef struct gfz_context gfz_context;       /* one GPU + one CUDA stream */
typedef struct gfz_compressed gfz_compressed; /* a .gfaz container (host) */
typedef struct gfz_grammar gfz_grammar;       /* device-resident grammar */
typedef struct gfz_graph gfz_graph;           /* decompressed graph (host) */

/* ---- library ------------------------------------------------------------ */
const char *gfz_last_error(void);
const char *gfz_version(void);
void gfz_free(void *p);
/* 1 when a CUDA device is usable (gfa_compression.has_gpu_backend,
 * src/python/bindings.cpp:94-100). */
int gfz_has_gpu(void);
/* zstd library version in use (entropy stage), 0 if unavailable. */
unsigned gfz_zstd_version(void);

/* ---- contexts ------------------------------------------------------------ */
/* cuda_stream may be NULL (the context creates its own stream, one step
 * above the lowest priority).  Text that gfz_decode_text puts into host
 * memory is bound by the chip-to-chip link: its copies (or, with
 * "host_text" 0, its kernel) run on a stream of the lowest priority
 * ordered after the context's stream.  Every other transfer of a context
 * is made by kernels, so that it never waits behind another stream's
 * copy-engine transfer.  Grammars
 * free their device memory on the stream of the context that made them:
 * free them before that context, and keep a caller's stream alive until
 * the context is destroyed. */
gfz_status gfz_context_create(int device, void *cuda_stream, gfz_context **out);
void gfz_context_destroy(gfz_context *ctx);
/* Records CUDA events around every kernel launch when enabled. */
gfz_status gfz_context_set_timing(gfz_context *ctx, int enabled);
/* JSON object {"kernel": {"ms": .., "launches": .., "bytes": ..}, ...} plus
 * "_launches": total kernels launched since the last reset. */
gfz_status gfz_context_kernel_stats(gfz_context *ctx, int reset, char **json, size_t *len);
/* Tuning switches: "warp_dedup" = warp-level de-duplication of pair inserts
 * (default 0); "first_table_cap" = pair-table slots of the first grammar
 * round, a power of two (default 0 = sized automatically; the table grows
 * when it fills either way); "append_chunk" = steps per chunk of the
 * chunked append encoder (default 0 = 256, then 2048 and 16384 where a
 * chunk's fix-up does not settle, then one thread per traversal; any other
 * value tries that size, then one thread per traversal); "count_kernel" =
 * the pair-count kernel of the grammar rounds: -1 (default) = the fastest of
 * the tiled and the flat kernels, timed the first time the context meets a
 * stream class (length, repeat density) and remembered, 0 = tiled, 1 =
 * tiled with warp folding, 2 = flat (one pair per thread), 3 = flat with
 * four pairs per thread and run folding; "slot_refs" = 1 (default): the
 * count records each position's table slot, and the candidate
 * classification and the replacement read it instead of probing the table
 * again (0 = probe; the same result); "classify_kernel" = the candidate
 * classification pass when it probes the table (slot references off),
 * tuned alike: -1 (default), 0 = persistent with staged tiles, 1 = flat
 * (one tile per block);
 * "hbm_budget" = device bytes that compression of host-resident input may
 * use (default 0 = no limit): above it the stream stays in host memory and
 * passes through HBM in chunks, with identical output; "encode_chunk" =
 * steps per such chunk, forcing chunked compression (default 0);
 * "decode_chunk" = expanded steps per device pass of the full-file writer
 * (gfz_write_gfa, gfz_gfa_text): P and W lines are written in traversal
 * groups of at most that many steps (a longer traversal alone), each group
 * downloaded before the next decodes (default 0 = one pass; the same
 * bytes; the CLI's --gpu-rolling-output-chunk-mb sets it);
 * "front_end" = the GFA parse of file compression: 1 (default) = the
 * device front end (line index and P/W steps on the GPU), 0 = the host
 * parser; both give the same graph, and the host parser also runs when the
 * file does not fit "hbm_budget" three times over; "static_text" = the S and
 * L lines of the full-file writer: 1 (default) = written on the device,
 * 0 = on the host; the same bytes; "table_tuner" = 1 (default): the pair
 * table's size (hash load factor) is tuned per stream class (the count
 * timed with tables for load <= 3/4, 1/2, 1/4 and at the estimate's size,
 * the fastest kept), 0 = sized from the estimate alone; results are the
 * same either way; "host_text" = how gfz_decode_text fills a page-locked
 * host buffer: 1 (default) = the text is written to HBM and moved by a copy
 * engine in pieces, each copied while the next is written, 0 = the text
 * kernel writes host memory directly (its stores then slow uploads of
 * other contexts running at the same time); the same bytes. */
gfz_status gfz_context_set_option(gfz_context *ctx, const char *name, int64_t value);

/* ---- workflows (ctx may be NULL: a default context on device 0) ---------- */
/* compress_gfa, include/workflows/compression_workflow.hpp:7-9;
 * python compress_file, src/python/bindings.cpp:661-667.  threshold is
 * accepted and, as in the reference, only warns when > 2. */
gfz_status gfz_compress_file(gfz_context *ctx, const char *gfa_path, int rounds, uint64_t threshold,
                             int delta_round, int threads, int show_stats, gfz_compressed **out);
/* serialize_compressed_data, include/codec/serialization.hpp:13-14 */
gfz_status gfz_serialize(const gfz_compressed *c, const char *path);
gfz_status gfz_serialize_buffer(const gfz_compressed *c, void **out, size_t *len);
/* deserialize_compressed_data, include/codec/serialization.hpp:15-16 */
gfz_status gfz_deserialize(const char *path, gfz_compressed **out);
gfz_status gfz_deserialize_buffer(const void *data, size_t len, gfz_compressed **out);
void gfz_compressed_free(gfz_compressed *c);
/* write_gfa_from_compressed_data, include/io/gfa_writer.hpp:9-11 and the
 * GPU writer write_gfa_from_compressed_data_gpu,
 * include/gpu/io/gfa_writer_gpu.hpp:9-12 (streaming order H,S,L,J,C,P,W). */
gfz_status gfz_write_gfa(gfz_context *ctx, const gfz_compressed *c, const char *out_path, int threads);
gfz_status gfz_gfa_text(gfz_context *ctx, const gfz_compressed *c, int threads, char **out, size_t *len);
/* extract_path_lines_by_name, include/workflows/extraction_workflow.hpp:19-21:
 * lines concatenated in request order. */
gfz_status gfz_extract_path_lines(gfz_context *ctx, const gfz_compressed *c, const char *const *names, size_t n,
                                  int threads, char **out, size_t *len);
typedef struct {
  const char *sample_id;
  uint32_t hap_index;
  const char *seq_id;
  int64_t seq_start; /* -1 prints '*' */
  int64_t seq_end;
} gfz_walk_key;
/* extract_walk_lines, extraction_workflow.hpp:35-38 */
gfz_status gfz_extract_walk_lines(gfz_context *ctx, const gfz_compressed *c, const gfz_walk_key *keys, size_t n,
                                  int threads, char **out, size_t *len);
/* extract_walk_lines_by_name, extraction_workflow.hpp:40-43 */
gfz_status gfz_extract_walk_lines_by_name(gfz_context *ctx, const gfz_compressed *c, const char *const *names,
                                          size_t n, int threads, char **out, size_t *len);
/* add_haplotypes, include/workflows/add_haplotypes_workflow.hpp:9-10 (in place) */
gfz_status gfz_add_haplotypes(gfz_context *ctx, gfz_compressed *c, const char *path, int threads);
/* parse_gfa_file, src/python/bindings.cpp:659-660 (GfaParser::parse,
 * src/io/gfa_parser.cpp:306-590): device != 0 parses with the device front
 * end on ctx (NULL: the default context), device == 0 with the host parser
 * (ctx unused; no GPU needed).  Parse errors are "GFA parser error: ..." or
 * the value parser's own message, as in the reference. */
gfz_status gfz_parse_gfa(gfz_context *ctx, const char *path, int threads, int device, gfz_graph **out);
/* compute_growth, include/workflows/growth_workflow.hpp:36-41 (`gfaz growth`,
 * src/cli/growth_command.cpp): group_by 0 = every P/W line ("path"), 1 =
 * PanSN sample#hap#seq ("sample-hap-seq"), 2 = sample#hap ("sample-hap"),
 * 3 = sample.  *hist gets num_haplotypes + 1 counts (nodes covered by
 * exactly c groups) and *growth num_haplotypes + 1 values (growth[0] = 0),
 * both released with gfz_free (NULL when num_haplotypes is 0). */
gfz_status gfz_growth(gfz_context *ctx, const gfz_compressed *c, int threads, int group_by, uint32_t *num_haplotypes,
                      uint32_t *num_nodes, uint64_t **hist, double **growth);
/* compute_pav, include/workflows/pav_workflow.hpp:35 (`gfaz pav`,
 * src/cli/pav_command.cpp): group_by 0 = every traversal name, 2 =
 * sample#hap (-H), 3 = sample (-S).  Outputs, released with gfz_free: the
 * BED ranges as "chrom\tstart\tend\tname\n" lines, the group names
 * newline-joined, denominators[nranges] and numerators[nranges * ngroups]
 * (row = range), in bases. */
gfz_status gfz_pav(gfz_context *ctx, const gfz_compressed *c, const char *bed_path, int threads, int group_by,
                   char **ranges, size_t *ranges_len, char **groups, size_t *groups_len, uint64_t *nranges,
                   uint64_t *ngroups, uint64_t **denominators, uint64_t **numerators);
/* decompress_gfa, include/workflows/decompression_workflow.hpp:8-9 */
gfz_status gfz_decompress_graph(gfz_context *ctx, const gfz_compressed *c, int threads, gfz_graph **out);
void gfz_graph_free(gfz_graph *g);

/* ---- container / graph inspection (host only) ---------------------------- */
typedef struct {
  uint64_t num_paths, num_walks, num_links, num_jumps, num_containments, num_layers, total_rules;
  uint32_t min_rule_id, reserved;
  int32_t delta_round;
  int32_t reserved2;
} gfz_container_info;
gfz_status gfz_compressed_info(const gfz_compressed *c, gfz_container_info *info);
/* Layer ranges as rows (k, start_id, end_id, flattened_offset, element_count). */
gfz_status gfz_compressed_layers(const gfz_compressed *c, int64_t *rows, size_t max_rows);
/* Named u32 vectors: "sequence_lengths", "original_path_lengths",
 * "walk_lengths", "original_walk_lengths". */
gfz_status gfz_compressed_u32(const gfz_compressed *c, const char *field, const uint32_t **data, size_t *n);
/* zstd-decoded bytes of a named block ("rules_first", "rules_second",
 * "paths", "walks", "names", "name_lengths", ...). */
gfz_status gfz_compressed_block(const gfz_compressed *c, const char *field, void **out, size_t *len);
/* Steps (paths then walks share no buffer): kind 0 = paths, 1 = walks. */
gfz_status gfz_graph_traversals(const gfz_graph *g, int kind, const int32_t **steps, const uint64_t **offsets,
                                uint64_t *ntrav);
/* Newline-joined string fields: "path_names", "path_overlaps",
 * "walk_sample_ids", "walk_seq_ids", "segment_names", "segment_sequences"
 * (segments in id order), "header". */
gfz_status gfz_graph_strings(const gfz_graph *g, const char *field, char **out, size_t *len);
gfz_status gfz_graph_walk_numbers(const gfz_graph *g, const uint32_t **haps, const int64_t **starts,
                                  const int64_t **ends, uint64_t *n);
gfz_status gfz_graph_counts(const gfz_graph *g, uint64_t *segments, uint64_t *links, uint64_t *jumps,
                            uint64_t *containments);

/* ---- the transform hot path (device-resident) ---------------------------- */
/* Replaces the reference GPU compressor's compress_gpu_graph /
 * run_path_compression_gpu (include/gpu/compression/compression_workflow_gpu.hpp:84-99)
 * with CPU-identical semantics: delta_round rounds of per-traversal delta
 * coding, then up to `rounds` grammar rounds.  steps / offsets describe
 * traversals steps[offsets[t] .. offsets[t+1]) (paths first, then walks);
 * offsets are host memory (ntrav + 1 entries); steps live where `where`
 * says.  threshold is accepted and ignored beyond a warning, as in the
 * reference (src/grammar/rule_generator.cpp:242-246). */
gfz_status gfz_encode(gfz_context *ctx, const int32_t *steps, const uint64_t *offsets, uint64_t ntrav, int rounds,
                      uint64_t threshold, int delta_round, int where, gfz_grammar **out);
typedef struct {
  uint64_t ntrav, encoded_len, num_rules;
  uint32_t layer_start, next_id;
  int32_t rounds_done, delta_round;
} gfz_grammar_info;
gfz_status gfz_grammar_info_get(const gfz_grammar *g, gfz_grammar_info *info);
/* Copies the encoded stream (encoded_len), its offsets (ntrav + 1, host) and
 * the packed rulebook (num_rules int64 keys, index = id - layer_start).  Any
 * pointer may be NULL. */
gfz_status gfz_grammar_copy(gfz_context *ctx, const gfz_grammar *g, int32_t *encoded, uint64_t *offsets,
                            int64_t *rules, int where);
/* Rule columns as stored in the container: first/second halves of each key,
 * each delta coded over the rulebook (compression_utils.cpp:165-193). */
gfz_status gfz_grammar_rule_columns(gfz_context *ctx, const gfz_grammar *g, int32_t *first, int32_t *second,
                                    int where);
/* Decompression side: loads a stored rulebook (delta-coded columns) and
 * encoded traversals.  Replaces prepare_gpu_traversal_rulebook /
 * decompress_to_gpu_layout (include/gpu/decompression/decompression_workflow_gpu.hpp:46-48). */
gfz_status gfz_grammar_load(gfz_context *ctx, const int32_t *encoded, const uint64_t *offsets, uint64_t ntrav,
                            const int32_t *rules_first, const int32_t *rules_second, uint64_t num_rules,
                            uint32_t min_rule_id, int delta_round, int where, gfz_grammar **out);
void gfz_grammar_free(gfz_grammar *g);
/* Expansion + inverse delta of traversals [t0, t1).  out receives the steps
 * (capacity `cap` elements), offsets_out (host, t1 - t0 + 1 entries) their
 * offsets; *n_out is the number of steps.  GFZ_ERR_BUFFER when cap is too
 * small. */
gfz_status gfz_decode(gfz_context *ctx, gfz_grammar *g, uint64_t t0, uint64_t t1, int32_t *out, uint64_t cap,
                      uint64_t *n_out, uint64_t *offsets_out, int where);
/* Line metadata for text emission.  P: names + overlaps (NULL entry or NULL
 * array = ""); W: names are sample ids, plus hap/seq_id/start/end. */
typedef struct {
  int mode; /* GFZ_P_LINES or GFZ_W_LINES */
  const char *const *names;
  const char *const *overlaps;
  const uint32_t *hap_indices;
  const char *const *seq_ids;
  const int64_t *seq_starts;
  const int64_t *seq_ends;
} gfz_line_meta;
/* Expansion + inverse delta + GFA text of traversals [t0, t1) (the rolling
 * writer's path, src/gpu/decompression/path_decompression_gpu_rolling.cpp:215-370
 * and format_*_line_numeric, src/io/gfa_write_utils.cpp:238-290).  With
 * out == NULL the text stays in a device buffer owned by `g`
 * (gfz_grammar_text gives its address); otherwise it goes to out (capacity
 * cap bytes, host or device per `where`).  When out is device memory the
 * kernels write the text there directly; page-locked host memory gets it
 * as "host_text" says (staged in HBM and copied in pieces by default, or
 * written by the kernel); either way `g` keeps no copy: gfz_grammar_text
 * then fails until the next decode without out. */
gfz_status gfz_decode_text(gfz_context *ctx, gfz_grammar *g, uint64_t t0, uint64_t t1, const gfz_line_meta *meta,
                           char *out, uint64_t cap, uint64_t *size, int where);
gfz_status gfz_grammar_text(const gfz_grammar *g, const char **device_text, uint64_t *size);

/* ---- resident extraction server ------------------------------------------ */
/* No counterpart in the reference, which decodes the whole file for each
 * extraction (src/workflows/extraction_workflow.cpp:207-357) and rewrites
 * the container for each append (add_haplotypes_workflow.cpp:579).  The
 * server keeps the rules, their prefix buffers and all encoded traversals
 * of `c` in HBM and serves extract-path / extract-walk / append requests
 * with continuous batching: `workers` threads, one CUDA stream each, take
 * the queued extractions whose expanded output fits the free part of
 * `hbm_budget` bytes and decode them in one launch; requests arriving
 * meanwhile join the next batch.  An append waits for the batches in flight
 * and is seen by every later request.  Returned lines are byte-identical to
 * gfz_extract_path_lines / gfz_extract_walk_lines on the same container. */
typedef struct gfz_server gfz_server;
gfz_status gfz_server_create(int device, const gfz_compressed *c, uint64_t hbm_budget, int workers,
                             gfz_server **out);
gfz_status gfz_server_submit_path(gfz_server *s, const char *name, uint64_t *ticket);
gfz_status gfz_server_submit_walk(gfz_server *s, const gfz_walk_key *key, uint64_t *ticket);
/* P or W lines to append, as GFA text (the add-haplotypes input format). */
gfz_status gfz_server_submit_append(gfz_server *s, const char *gfa_text, size_t len, uint64_t *ticket);
/* Blocks until request `ticket` is done: its line (empty for an append)
 * and the time from submission to completion.  The line lives in the
 * server's pinned host memory, valid until gfz_server_release(s, ticket);
 * a request that failed returns its error and is released already. */
gfz_status gfz_server_wait(gfz_server *s, uint64_t ticket, const char **line, size_t *len, double *latency_ms);
/* For a finished request before its release: the time it waited in the
 * queue (submission to the start of its batch), the time in service (batch
 * start to completion) and the number of requests in its batch. */
gfz_status gfz_server_request_times(gfz_server *s, uint64_t ticket, double *queue_ms, double *service_ms,
                                    uint32_t *batch_size);
gfz_status gfz_server_release(gfz_server *s, uint64_t ticket);
/* Wait, request times and release in one call, for clients that consume
 * only the size of the line (load generators, health checks). */
gfz_status gfz_server_collect(gfz_server *s, uint64_t ticket, size_t *len, double *latency_ms, double *queue_ms,
                              double *service_ms, uint32_t *batch_size);
gfz_status gfz_server_stats(gfz_server *s, uint64_t *batches, uint64_t *requests, uint64_t *max_batch);
void gfz_server_destroy(gfz_server *s);

/* Allocation-free inverse delta.  This entry point has no counterpart in the
 * reference.  It is for callers that may not allocate device memory: hosts
 * whose own pool allocator holds nearly all of HBM, plug-ins that such a host
 * forbids to allocate, and latency-bound loops that cannot afford the device
 * synchronisation cudaMalloc/cudaFree can cause.  It undoes `delta_round`
 * rounds of per-traversal delta coding (the inverse-delta step of
 * gfz_decode) of `n` steps from `steps_in` into `steps_out` on `cuda_stream`
 * (NULL = legacy default stream), with `offsets` (ntrav + 1 entries, from 0
 * to n) marking the traversals.  All three buffers are the caller's device
 * memory on the current device (managed and mapped host memory are refused
 * with GFZ_ERR_INVALID); steps_in == steps_out decodes in place.
 * The call allocates nothing: its scratch is a fixed 131,328-byte device
 * array that every GPU loading this library holds until exit, so n is
 * limited to GFZ_NOALLOC_MAX_STEPS (67,108,864); larger n fails with
 * GFZ_ERR_INVALID.  The first call on each device does a one-time set-up
 * (it looks up the array's device address) and should come before any
 * stream capture.  All calls on a device share the array, which keeps the
 * last call's contents (each call clears what must start at zero); calls
 * whose GPU work overlaps race on it and must be serialised by the caller.
 * Returns after `cuda_stream` has finished the work. */
#define GFZ_NOALLOC_MAX_STEPS 67108864ull
gfz_status gfz_inverse_delta_noalloc(const int32_t *steps_in, int32_t *steps_out, uint64_t n, const uint64_t *offsets,
                                     uint64_t ntrav, int delta_round, void *cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* GFAZ_GB300_H */

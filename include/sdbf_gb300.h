/*
 * sdbf_gb300.h -- C ABI of the GB300 SDBF engine (libsdbf_gb300.so).
 *
 * Plain pointers and sizes only.  Every entry point names the reference
 * sdhash interface (file:line in the sdhash source tree) whose work it
 * performs; the C++ compatibility classes (sdbf / sdbf_set with the
 * reference's signatures) and the Python binding sit on top of this ABI.
 *
 * Results are bit-exact with sdhash 4.0: digests byte-identical (SDBF v3
 * text), scores integer-identical.
 *
 * Error convention: functions return SDBFG_OK (0) or a negative status;
 * sdbfg_last_error() describes the last failure on that context.  Nothing
 * here exits the process (the reference exits on allocation failure,
 * sdbf/error.cc:33-39).
 */
#ifndef SDBF_GB300_H
#define SDBF_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDBFG_OK 0
#define SDBFG_ERR_ARG -1        /* bad argument */
#define SDBFG_ERR_CUDA -2       /* CUDA runtime error (see sdbfg_last_error) */
#define SDBFG_ERR_NOMEM -3      /* device or host allocation failed */
#define SDBFG_ERR_FORMAT -4     /* malformed SDBF text */
#define SDBFG_ERR_CAPACITY -5   /* output buffer too small */

/* Per-input digest status, mirroring the reference constructors' throws
 * (sdbf/sdbf_class.cc:37,81,117). */
#define SDBFG_DIGEST_OK 0
#define SDBFG_DIGEST_TOO_SMALL -3 /* fewer than 512 bytes (MIN_FILE_SIZE) */

typedef struct sdbfg_ctx sdbfg_ctx;
typedef struct sdbfg_set sdbfg_set;
typedef struct sdbfg_index sdbfg_index;

/* ---------------------------------------------------------------- context
 * One context = one device + one CUDA stream + reusable device buffers.
 * Replaces the process-global `sdbf::config` (sdbf/sdbf_class.cc:25) for the
 * GPU path.  A context is not thread-safe; use one per host thread. */
int sdbfg_ctx_create(int device, sdbfg_ctx **out);
void sdbfg_ctx_destroy(sdbfg_ctx *ctx);
const char *sdbfg_last_error(const sdbfg_ctx *ctx);
/* Launch on a caller-owned cudaStream_t (NULL = the context's own stream). */
int sdbfg_ctx_set_stream(sdbfg_ctx *ctx, void *cuda_stream);
int sdbfg_ctx_synchronize(sdbfg_ctx *ctx);
/* Kernel launches issued on this context so far (instrumentation). */
uint64_t sdbfg_ctx_launch_count(const sdbfg_ctx *ctx);
/* Per-kernel timing with CUDA events recorded on the launch stream around
 * every launch (off by default; enabling clears previous totals).
 * sdbfg_ctx_kernel_time reports the accumulated milliseconds and launch
 * count of one kernel ("k_stream_tiles", "k_stream_check", "k_stream_fix",
 * "k_stream_commit", "k_pack_filters", "k_block_digest", "k_compare_pairs",
 * "k_scan_offsets").  While profiling, the stream kernels also count SM
 * cycles per phase; the names "k_stream_tiles.{load,ranks,fres,walk,link,
 * compact,sha1}" and "k_stream_commit.{wait,busy,max_file}" report those
 * cycles in *total_ms (and the tile count in *launches); ".count",
 * ".groups", ".loops" report counts.  The tensor-core comparison kernel
 * reports "k_matrix_tc.{compose,fill,fetch_wait,stage_wait,widen,issue,
 * producer_step,acc_wait,score,mark,walk,fold,consumer_step,step_barrier,
 * tmem_ld}" in SM cycles and ".tiles" as a count.
 * Instrumentation without a counterpart in the reference. */
int sdbfg_ctx_profile(sdbfg_ctx *ctx, int enable);
int sdbfg_ctx_kernel_time(sdbfg_ctx *ctx, const char *kernel, double *total_ms, uint64_t *launches);
/* Speculative lead-in of the parallel popularity-score walk, in window steps
 * (default 64, maximum 128).  Results are exact for every value -- shorter
 * lead-ins only make the re-walk path run more often; tests use this to
 * exercise it.  No counterpart in the reference (its walk is sequential). */
int sdbfg_ctx_set_lead(sdbfg_ctx *ctx, uint32_t steps);
/* Stream-mode launch groups (<= 2 GiB of input each) kept in flight on
 * separate streams, 1..8 (default 4): the ordered commit of one group
 * overlaps the next groups' tile kernels.  Depth 1 runs groups one after
 * another (used to time kernels without overlap).  Tuning knob without a
 * counterpart in the reference. */
int sdbfg_ctx_set_pipeline_depth(sdbfg_ctx *ctx, int depth);
/* The current pipeline depth (no counterpart in the reference). */
int sdbfg_ctx_pipeline_depth(const sdbfg_ctx *ctx);
/* Tiles whose speculative popularity chain was re-walked (instrumentation). */
uint64_t sdbfg_ctx_relinked_tiles(sdbfg_ctx *ctx);
/* Stream-mode index build (sdbfg_digest_batch_index with dd == 0): the
 * number of parallel fixed-point rounds tried per launch group before the
 * one-warp sequential commit takes over (default 16; 0 = sequential only).
 * Results are exact either way.  sdbfg_ctx_index_rounds: rounds the last
 * launch group took (0 = it ran the sequential commit).  No counterpart in
 * the reference (its index build is sequential). */
int sdbfg_ctx_set_index_rounds(sdbfg_ctx *ctx, uint32_t max_rounds);
uint32_t sdbfg_ctx_index_rounds(sdbfg_ctx *ctx);

/* ----------------------------------------------------- digest generation */
typedef struct {
    uint32_t bf_count;      /* filters in the digest */
    uint32_t last_count;    /* stream: elements in the last filter; block: 0 */
    int32_t status;         /* SDBFG_DIGEST_OK or SDBFG_DIGEST_TOO_SMALL */
    uint32_t reserved;
    uint64_t filter_offset; /* index of the digest's first filter in out_filters */
} sdbfg_digest_result;

/* Filter slots a batch needs in out_filters: per input (len>>11)+1 for stream
 * mode (the reference's own allocation bound, sdbf/sdbf_core.cc:202-204) or
 * len/B + (len%B >= 512) for block mode. */
uint64_t sdbfg_digest_capacity(const uint64_t *lens, uint32_t n, uint32_t dd_block_size);

/* Digest n inputs.  dd_block_size == 0: stream mode, as
 *   sdbf::sdbf(name, char *str, 0, length, NULL)        sdbf/sdbf_class.cc:115
 *   -> gen_chunk_sdbf                                      sdbf/sdbf_core.cc:196
 * dd_block_size > 0 (<= 16384): block mode, as the same constructor with
 * dd_block_size -> gen_block_sdbf_mt (sdbf/sdbf_core.cc:287).
 * The file / istream constructors (sdbf_class.cc:34,71) read the bytes and
 * then do exactly this.
 * host_data + offsets[i] holds input i (lens[i] bytes) in HOST memory
 * (pinned memory is copied directly, pageable memory through a staging
 * buffer).  Filters land in out_filters (host, 256 bytes per slot,
 * capacity out_cap filter slots, see sdbfg_digest_capacity); block-mode
 * element counts in out_elem_counts (one uint16 per slot; may be NULL for
 * stream mode). */
int sdbfg_digest_batch(sdbfg_ctx *ctx, const uint8_t *host_data, const uint64_t *offsets, const uint64_t *lens,
                       uint32_t n, uint32_t dd_block_size, uint8_t *out_filters, uint64_t out_cap,
                       uint16_t *out_elem_counts, sdbfg_digest_result *results);

/* Same with inputs already in DEVICE memory (offsets must be multiples of
 * 16) and outputs written to DEVICE memory; results[] is host memory. */
int sdbfg_digest_batch_device(sdbfg_ctx *ctx, const uint8_t *dev_data, const uint64_t *offsets,
                              const uint64_t *lens, uint32_t n, uint32_t dd_block_size, uint8_t *dev_out_filters,
                              uint64_t out_cap, uint16_t *dev_out_elem_counts, sdbfg_digest_result *results);

/* ------------------------------------------- digests without allocation
 * No counterpart in the reference.  For callers that cannot allocate GPU
 * memory -- code inside a framework that owns every device allocation, a
 * fixed memory budget reserved up front, or a path that may not enter the
 * allocator -- this stream-mode digest (same results as
 * sdbfg_digest_batch_device with dd_block_size 0) allocates nothing, on the
 * device or on the host heap.  Its scratch is one fixed device array of
 * SDBFG_NOALLOC_SCRATCH_BYTES compiled into the library: every GPU that
 * loads the library holds it until the process exits.
 *   Limits: at most SDBFG_NOALLOC_MAX_INPUTS inputs and
 *   SDBFG_NOALLOC_MAX_INPUT_BYTES input bytes per call; larger requests are
 *   rejected with SDBFG_ERR_CAPACITY (and a message on stderr), as is an
 *   output smaller than the digests need.
 * Inputs: device memory, offsets multiples of 16; outputs: packed filters in
 * dev_out_filters (out_cap filter slots), results[] in host memory.  Runs on
 * the current device and on cuda_stream (NULL = default stream), and
 * returns after the work is complete.
 * The first call on a device resolves the scratch array's device address
 * and loads the digest tables into it; make that first call before any
 * stream capture.  That set-up is not repeated: after cudaDeviceReset on a
 * device this entry point must not be used on it again in the process.
 * All calls share the one array: calls whose work overlaps on the GPU race
 * and corrupt each other's results -- serialise them. */
#define SDBFG_NOALLOC_MAX_INPUTS 256u
#define SDBFG_NOALLOC_MAX_INPUT_BYTES (8ull << 20)
#define SDBFG_NOALLOC_SCRATCH_BYTES (14ull << 20)
int sdbfg_digest_stream_noalloc(const uint8_t *dev_data, const uint64_t *offsets, const uint64_t *lens, uint32_t n,
                                uint8_t *dev_out_filters, uint64_t out_cap, sdbfg_digest_result *results,
                                void *cuda_stream);

/* ------------------------------------------------------------ comparison */
/* A digest as the reference's sdbf object holds it (sdbf/sdbf_class.h:95-119). */
typedef struct {
    const char *name;             /* hashname; used by the swap tie-break */
    const uint8_t *filters;       /* bf_count * 256 bytes (host) */
    const uint16_t *elem_counts;  /* block digests: per filter; NULL for stream */
    uint32_t bf_count;
    uint32_t last_count;          /* stream digests */
    uint32_t max_elem;            /* 160 stream / 192 block */
    uint32_t dd_block_size;       /* 0 for stream digests */
    uint64_t orig_size;
} sdbfg_digest_desc;

/* Upload digests to the device once (the resident form of sdbf_set,
 * sdbf/sdbf_set.h:15-96); hamming weights are computed on upload
 * (sdbf::compute_hamming, sdbf_class.cc:388-401). */
int sdbfg_set_upload(sdbfg_ctx *ctx, const sdbfg_digest_desc *digests, uint32_t n, sdbfg_set **out);
void sdbfg_set_free(sdbfg_set *set);
/* Bulk load of SDBF v3 text (one digest per line) into a resident set:
 * sdbf_set(const char* fname) (sdbf/sdbf_set.cc:51-74) over
 * sdbf(const std::string&) (sdbf/sdbf_class.cc:144-215) for every line.
 * The host reads the line headers; the base64 payloads are decoded, checked
 * and their hamming weights computed on the device.  Loading stops at the
 * first empty line, as the reference's does.  A malformed line returns
 * SDBFG_ERR_FORMAT with *bad_line = its index (0-based) and *bad_code = the
 * value the reference constructor throws for it (-1: shorter than 344
 * characters, -2: any other format error); no set is created.  Either
 * pointer may be NULL. */
int sdbfg_set_load_text(sdbfg_ctx *ctx, const char *text, uint64_t len, sdbfg_set **out, int64_t *bad_line,
                        int32_t *bad_code);
/* ------------------------------------------------------------ indexes
 * An index is one large Bloom filter (bloom_filter, sdbf/bloom_filter.cc),
 * resident on the device.  sdbfg_index_load_file reads an index file as
 * bloom_filter(string indexfilename) does (bloom_filter.cc:87-118): the
 * header "sdbf-idx:<bf_size>:<elem_count>:<hash_count>:<bit_mask>:<compressed
 * size>:<set name>" and the LZ4-compressed filter.  An unreadable file
 * returns SDBFG_ERR_ARG (the reference throws -1), a malformed one
 * SDBFG_ERR_FORMAT (-2).  sdbfg_index_create makes one from raw filter
 * bytes (bloom_filter(size, hash_count, 0, 0) plus its contents; size a
 * power of two >= 64, bit mask size*8-1). */
int sdbfg_index_load_file(sdbfg_ctx *ctx, const char *path, sdbfg_index **out);
int sdbfg_index_create(sdbfg_ctx *ctx, const uint8_t *bits, uint64_t bf_size, uint32_t hash_count, const char *name,
                       sdbfg_index **out);
void sdbfg_index_free(sdbfg_index *index);
int sdbfg_index_info(const sdbfg_index *index, uint64_t *bf_size, uint64_t *elem_count, uint32_t *hash_count,
                     uint64_t *bit_mask, const char **name);
/* Block-mode digests (as sdbfg_digest_batch with dd_block_size > 0) with
 * the index search of sdhash --index-search (sdbf::gen_block_hash with an
 * index list, sdbf/sdbf_core.cc:141-191; check_indexes :482-493): every
 * fourth counted feature of each block is looked up in every index, and
 * out_hits[slot * nidx + i] receives how many of them index i holds (all
 * hash bits set) for the filter in output slot `slot`.  The reference
 * prints "<name> [<block>] |<index set name>|<hits>" for hits > 4
 * (print_indexes :458-472); out_hits has out_cap * nidx bytes. */
int sdbfg_digest_batch_search(sdbfg_ctx *ctx, const uint8_t *host_data, const uint64_t *offsets,
                              const uint64_t *lens, uint32_t n, uint32_t dd_block_size, uint8_t *out_filters,
                              uint64_t out_cap, uint16_t *out_counts, sdbfg_digest_result *results,
                              const sdbfg_index *const *indexes, uint32_t nidx, uint8_t *out_hits);
/* Digests (as sdbfg_digest_batch) with an index being built, as sdhash
 * --index builds one per group of files (sdhash-src/sdhash_threads.cc:
 * 376-470).  index_bits (index_bytes, a power of two, host memory) is the
 * index before the batch and receives it after; *elem_count is increased by
 * the inserts that set a new bit (bloom_filter::insert_sha1,
 * bloom_filter.cc:333-359).  Stream mode (dd_block_size 0): every feature
 * whose filter insert set a new bit is inserted into the index and is
 * skipped unless that set a new index bit (sdbf_core.cc:108-114), so each
 * digest depends on the inputs before it: inputs are taken in order, as
 * sdhash -p 1 does.  Block mode: every counted feature is inserted
 * (sdbf_core.cc:164-167) and the digests are those of sdbfg_digest_batch. */
int sdbfg_digest_batch_index(sdbfg_ctx *ctx, const uint8_t *host_data, const uint64_t *offsets, const uint64_t *lens,
                             uint32_t n, uint32_t dd_block_size, uint8_t *out_filters, uint64_t out_cap,
                             uint16_t *out_elem_counts, sdbfg_digest_result *results, uint8_t *index_bits,
                             uint64_t index_bytes, uint64_t *elem_count);
/* bloom_filter::write_out (bloom_filter.cc:190-216): the index file header
 * and the filter as one LZ4 block (this library's own encoder: any LZ4
 * decoder, the reference's included, reads it; the bytes differ from the
 * reference's compressor's).  Host-only; SDBFG_ERR_ARG when the file cannot
 * be written. */
int sdbfg_index_write_file(const char *path, const uint8_t *bits, uint64_t bf_size, uint64_t elem_count,
                           uint32_t hash_count, const char *set_name);
/* LZ4 block encode (the encoder of sdbfg_index_write_file): returns the
 * encoded size; writes it to out when it fits out_cap.  Host-only. */
int64_t sdbfg_lz4_encode(const uint8_t *in, uint64_t in_len, uint8_t *out, uint64_t out_cap);
/* LZ4 block decode of in_len bytes into exactly out_len bytes (the index
 * file payload, LZ4_uncompress in bloom_filter::decompress,
 * bloom_filter.cc:185-190); returns the input bytes used or
 * SDBFG_ERR_FORMAT.  Host-only. */
int64_t sdbfg_lz4_decode(const uint8_t *in, uint64_t in_len, uint8_t *out, uint64_t out_len);

/* Header fields of digest i (name owned by the set; filters and
 * elem_counts are NULL): the sdbf accessors name(), input_size(),
 * filter_count() (sdbf/sdbf_class.h:23-121). */
int sdbfg_set_digest_info(const sdbfg_set *set, uint32_t i, sdbfg_digest_desc *out);
/* Copies digest i's filters (bf_count*256 bytes; the folded bytes after
 * sdbfg_set_fast) and, if elem_counts is not NULL, its per-filter element
 * counts (sdbf::get_elem_count, sdbf_class.cc:406-415) back to the host. */
int sdbfg_set_read_digest(sdbfg_ctx *ctx, const sdbfg_set *set, uint32_t i, uint8_t *filters,
                          uint16_t *elem_counts);
/* sdbf::fast (sdbf/sdbf_class.cc:425-439) on digests [first, first+count)
 * of a resident set: every filter's 256 bytes are folded into its first 64
 * (bloom_filter::fold(2), bloom_filter.cc:262-288; the other bytes are left
 * as they were), its hamming weight becomes that of the folded 64 bytes, and
 * the digest is scored in fast mode (CUTOFFS64, 64-byte one-stage count)
 * whenever it is the reference side of a pair -- the reference's fastmode
 * rule (sdbf_core.cc:422-440).  Folding twice changes nothing. */
int sdbfg_set_fast(sdbfg_ctx *ctx, sdbfg_set *set, uint32_t first, uint32_t count);
uint32_t sdbfg_set_size(const sdbfg_set *set);

/* Scores of explicit pairs (a[ia[k]], b[ib[k]]) as sdbf::compare(other, 0)
 * (sdbf/sdbf_class.cc:266 -> sdbf_score, sdbf/sdbf_core.cc:330-389),
 * including the swap rule and the -1 result.  b may equal a. */
int sdbfg_score_pairs(sdbfg_ctx *ctx, const sdbfg_set *a, const sdbfg_set *b, const uint32_t *ia,
                      const uint32_t *ib, uint64_t npairs, int32_t *out_scores);

/* All pairs i<j of one set in set order (sdbf_set::compare_all /
 * compare_all_quiet, sdbf/sdbf_set.cc:239-308): out has n*(n-1)/2 scores in
 * row order (0,1),(0,2),...,(1,2),... */
int sdbfg_compare_all(sdbfg_ctx *ctx, const sdbfg_set *set, int32_t *out_scores);

/* Every query against every target (sdbf_set::compare_to /
 * compare_to_quiet with sample_size 0, sdbf/sdbf_set.cc:317-394):
 * out[i*nt + j] = score(query i, target j). */
int sdbfg_compare_to(sdbfg_ctx *ctx, const sdbfg_set *queries, const sdbfg_set *targets, int32_t *out_scores);

/* sdbfg_compare_all / sdbfg_compare_to run on the batched engine: one
 * persistent launch over work units (a reference digest against a run of
 * target digests, largest units first), replayed as a CUDA graph when the
 * same sets are compared again.  The _device forms write the scores to a
 * device array (same layout) and return without waiting: the work is
 * queued on the context stream.  Batched forms of the reference's
 * OpenMP loops (sdbf/sdbf_set.cc:249-265, 330-346); no single counterpart. */
int sdbfg_compare_all_device(sdbfg_ctx *ctx, const sdbfg_set *set, int32_t *dev_scores);
int sdbfg_compare_to_device(sdbfg_ctx *ctx, const sdbfg_set *queries, const sdbfg_set *targets,
                            int32_t *dev_scores);
/* The pairs whose score is >= threshold, in pair order, as the rows
 * sdbf_set::compare_all / compare_to print them (sdbf/sdbf_set.cc:249-265,
 * 330-346; i < j for all pairs, (query, target) for compare_to).  Returns
 * SDBFG_ERR_CAPACITY with *count = the number of matches when cap is too
 * small (call again with room for *count). */
typedef struct {
    uint32_t i, j;
    int32_t score;
} sdbfg_match;
int sdbfg_compare_all_matches(sdbfg_ctx *ctx, const sdbfg_set *set, int32_t threshold, sdbfg_match *out,
                              uint64_t cap, uint64_t *count);
int sdbfg_compare_to_matches(sdbfg_ctx *ctx, const sdbfg_set *queries, const sdbfg_set *targets, int32_t threshold,
                             sdbfg_match *out, uint64_t cap, uint64_t *count);
/* Filter pairs the comparison scores (sum of n_ref * n_target over pairs). */
uint64_t sdbfg_compare_filter_pairs(sdbfg_ctx *ctx, const sdbfg_set *a, const sdbfg_set *b_or_null);
/* Engine tuning: kernel variant 0..4 (rows per CTA x target filters per
 * shared-memory tile: 128x32, 128x16, 128x64, 64x32, 256x32), unit work
 * budget in filter pairs, CUDA-graph replay on/off.  The autotuner times
 * every variant and budget 2^20, 2^22, 2^24 on a sample of about
 * sample_pairs filter pairs of the given job (b NULL: all pairs of a) and
 * keeps the fastest in the context.  No counterpart in the reference. */
int sdbfg_ctx_set_compare_tuning(sdbfg_ctx *ctx, int variant, uint64_t unit_work, int use_graphs);
int sdbfg_ctx_get_compare_tuning(const sdbfg_ctx *ctx, int *variant, uint64_t *unit_work);
int sdbfg_compare_autotune(sdbfg_ctx *ctx, const sdbfg_set *a, const sdbfg_set *b_or_null, uint64_t sample_pairs,
                           int *out_variant, uint64_t *out_unit_work, double *out_pairs_per_s);

/* ------------------------------------------------------------- serving
 * A serving loop over a device-resident target set (the resident form of
 * sdhash's compare_to of query digests against a reference set,
 * sdbf/sdbf_set.cc:318-346; no counterpart as a service in the reference).
 * A worker thread admits queued query digests into batch slots (one CUDA
 * stream each) as slots free up, in arrival order, while their filters fit
 * the slot's share of memory_budget and the batch's filter pairs stay within
 * max_batch_pairs (a bound on the batch's GPU time, hence on latency); a
 * query larger than that runs in a batch of its own.  Every query is scored against every
 * target exactly as sdbfg_compare_to would score it.  The context must not
 * be used from other threads while its server runs; the target set must
 * outlive the server. */
typedef struct sdbfg_server sdbfg_server;
typedef struct {
    uint32_t slots;              /* batches in flight, 1..8 (default 3) */
    uint32_t max_batch_queries;  /* queries per batch (default 256) */
    uint64_t memory_budget;      /* device bytes for batches in flight (default 256 MiB) */
    int32_t threshold;           /* a target matches at score >= threshold (default 1) */
    uint32_t pad;
    uint64_t max_batch_pairs;    /* filter pairs per batch, i.e. GPU work per batch (0: 2^31) */
} sdbfg_server_config;
typedef struct {
    uint64_t tag;                /* as submitted */
    int32_t status;              /* SDBFG_OK */
    int32_t best_score;          /* highest score over the targets (-1: none) */
    uint32_t best_target;        /* its index in the target set */
    uint32_t matches;            /* targets with score >= threshold */
    uint32_t batch_queries;      /* queries in the batch it was scored in */
    uint32_t pad;
    uint64_t submit_ns, start_ns, done_ns;  /* steady clock: queued, admitted, scores on the host */
} sdbfg_server_result;
/* cfg NULL: defaults. */
int sdbfg_server_create(sdbfg_ctx *ctx, const sdbfg_set *targets, const sdbfg_server_config *cfg,
                        sdbfg_server **out);
/* Copies the query digest; thread-safe.  SDBFG_ERR_CAPACITY if the digest
 * alone exceeds a slot's memory share. */
int sdbfg_server_submit(sdbfg_server *srv, const sdbfg_digest_desc *query, uint64_t tag);
/* Up to max finished queries, oldest first; scores (max * n_targets, may
 * be NULL) receives each query's score row.  timeout_ms: 0 = do not wait,
 * < 0 = wait for at least one. */
int sdbfg_server_poll(sdbfg_server *srv, sdbfg_server_result *out, int32_t *scores, uint32_t max, uint32_t *n,
                      int timeout_ms);
int sdbfg_server_stats(const sdbfg_server *srv, uint64_t *pending, uint64_t *served, uint64_t *batches,
                       uint64_t *launches);
/* Finishes queued and running queries, then frees the server. */
void sdbfg_server_destroy(sdbfg_server *srv);

/* ------------------------------------------------------------ SDBF text */
/* sdbf::to_string (sdbf/sdbf_class.cc:293-334): one SDBF v3 line with
 * trailing newline.  Writes at most cap bytes (NUL-terminated); returns the
 * length needed (excluding NUL) or a negative status. */
int64_t sdbfg_to_string(const sdbfg_digest_desc *d, char *out, uint64_t cap);

/* sdbf::sdbf(const std::string&) (sdbf/sdbf_class.cc:144-215).  Parses one
 * line into caller-provided buffers (filters: bf_count*256 bytes, elem_counts:
 * bf_count entries for sdbf-dd).  Call first with filters == NULL to learn
 * bf_count / name length via *d.  name_buf receives the NUL-terminated name.
 * Returns SDBFG_OK, -1 (shorter than 344 chars) or SDBFG_ERR_FORMAT. */
int sdbfg_parse(const char *line, uint64_t len, sdbfg_digest_desc *d, char *name_buf, uint64_t name_cap,
                uint8_t *filters, uint16_t *elem_counts);

#ifdef __cplusplus
}
#endif
#endif

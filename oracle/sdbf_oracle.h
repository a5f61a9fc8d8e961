/*
 * sdbf_oracle.h -- CPU restatement of sdhash's digest-generation and
 * digest-comparison hot paths, in plain C.
 *
 * THIS IS TEST INFRASTRUCTURE (the oracle), not the product.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
 * only as the checker or as the timed CPU baseline.  The product path lives
 * in sdhash_gb300/ and never calls into this file.
 *
 * Every function cites the reference file:line it restates.  Parity of this
 * restatement against the reference itself (compiled from its own sources by
 * oracle/Makefile.ref) is pinned by tests/test_oracle_vs_reference.py and the
 * committed fixtures under tests/golden/.
 */
#ifndef SDBF_ORACLE_H
#define SDBF_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One similarity digest (fields of class sdbf, sdbf/sdbf_class.h:95-119). */
typedef struct {
    char     *name;           /* owned copy */
    uint64_t  orig_size;      /* orig_file_size */
    uint32_t  bf_count;       /* number of 256-byte filters */
    uint32_t  last_count;     /* stream mode: elements in the last filter */
    uint32_t  max_elem;       /* 160 stream / 192 block */
    uint32_t  dd_block_size;  /* 0 = stream digest */
    uint8_t  *filters;        /* bf_count * 256 bytes */
    uint16_t *elem_counts;    /* block mode only (NULL for stream) */
    uint16_t *hamming;        /* popcount per filter */
    int32_t   fastmode;       /* filters folded to 64 bytes (sdbf::fast) */
} orc_digest;

/* sdbf::fast (sdbf_class.cc:425-439): fold every filter 256 -> 64 bytes
 * (bloom_filter::fold(2), bloom_filter.cc:262-288) into its first 64 bytes,
 * hamming of the folded bytes, fastmode on. */
void orc_fast(orc_digest *d);

/* FIPS 180-4 SHA-1 of an arbitrary message. */
void orc_sha1(const uint8_t *msg, uint64_t len, uint8_t out[20]);

/* entr64_table_init_int (sdbf/entr64.cc:13-21), computed with libm log(). */
void orc_entropy_table(uint64_t table[65]);

/* gen_chunk_ranks (sdbf/sdbf_core.cc:21-45). ranks has n entries. */
void orc_ranks(const uint8_t *x, uint64_t n, uint16_t *ranks);

/* gen_chunk_scores (sdbf/sdbf_core.cc:50-89); histo (66 entries) may be NULL. */
void orc_scores(const uint16_t *ranks, uint64_t n, uint16_t *scores, int32_t *histo);

/* Stream-mode digest (sdbf/sdbf_core.cc:93-136,196-246).  Returns 0, or -3
 * when len < 512 (sdbf/sdbf_class.cc:79-82,116-117). */
int orc_digest_stream(const char *name, const uint8_t *x, uint64_t len, orc_digest *out);

/* Block-mode digest (sdbf/sdbf_core.cc:141-191,251-324; sdbf_class.cc:124-134). */
int orc_digest_block(const char *name, const uint8_t *x, uint64_t len,
                     uint32_t dd_block_size, orc_digest *out);

void orc_digest_free(orc_digest *d);

/* get_elem_count (sdbf/sdbf_class.cc:406-415). */
int32_t orc_elem_count(const orc_digest *d, uint64_t idx);

/* Staged AND-popcount (sdbf/bf_utils.cc:114-206) as used by
 * sdbf_max_score (sdbf/sdbf_core.cc:430-440): 0 when an early stage cuts. */
uint32_t orc_match_cut(const uint8_t *f1, const uint8_t *f2, uint32_t cut_off);

/* sdbf_max_score (sdbf/sdbf_core.cc:395-455). */
double orc_max_score(const orc_digest *ref, uint32_t ref_index, const orc_digest *tgt);

/* sdbf_score with sample == 0 (sdbf/sdbf_core.cc:330-389). */
int32_t orc_score(const orc_digest *a, const orc_digest *b);

/* sdbf::to_string (sdbf/sdbf_class.cc:293-334).  Returns malloc'd text. */
char *orc_to_string(const orc_digest *d);

/* sdbf(const std::string&) (sdbf/sdbf_class.cc:144-215).  0 / -1 / -2. */
int orc_from_string(const char *line, size_t len, orc_digest *out);

/* compare_all_quiet / compare_to_quiet output text (sdbf/sdbf_set.cc:239-394)
 * in set order (single thread).  sep is '|' by default.  Returns malloc'd. */
char *orc_compare_all(const orc_digest *set, uint32_t n, int32_t threshold, char sep);
char *orc_compare_to(const orc_digest *q, uint32_t nq, const orc_digest *t, uint32_t nt,
                     int32_t threshold, char sep);

/* Score matrices (no text): out[i*n+j] for i<j (compare_all orientation) and
 * out[i*nt+j] (compare_to orientation).  nthreads<=0 uses all cores. */
void orc_score_all_matrix(const orc_digest *set, uint32_t n, int32_t *out, int nthreads);
void orc_score_cross_matrix(const orc_digest *q, uint32_t nq, const orc_digest *t,
                            uint32_t nt, int32_t *out, int nthreads);
/* Scores of an explicit list of (i, j) pairs (set order), multithreaded. */
void orc_score_pairs(const orc_digest *set, const uint32_t *pi, const uint32_t *pj,
                     uint64_t npairs, int32_t *out, int nthreads);

/* Digest many buffers on nthreads host threads (file-parallel, as
 * sdhash-src/sdhash_threads.cc:152-186 assigns files round-robin). */
/* Block-mode digest with an index search (gen_block_hash with an index list,
 * sdbf/sdbf_core.cc:141-191): hits[b * nidx + x] = sampled features (counted
 * features 0, 4, 8, ...) of block b that index x holds.  hits must hold
 * bf_count * nidx zeroed bytes.  orc_index_search_many runs it over n inputs
 * on nthreads threads (hits[i] per input, digests discarded). */
int orc_index_search_block(const char *name, const uint8_t *x, uint64_t len, uint32_t B,
                           const uint8_t *const *bits, const uint32_t *masks, const uint32_t *hash_counts,
                           uint32_t nidx, orc_digest *d, uint8_t *hits);
void orc_index_search_many(const uint8_t *const *bufs, const uint64_t *lens, uint32_t n, uint32_t dd,
                           const uint8_t *const *bits, const uint32_t *masks, const uint32_t *hash_counts,
                           uint32_t nidx, int nthreads, uint8_t *const *hits, int *status);
/* Stream-mode digests of one sdhash --index group (files in order, one
 * shared index of bit mask index_mask; *elem_count counts the inserts that
 * set a new bit).  status[i] as orc_digest_stream returns it. */
int orc_index_build_stream(const uint8_t *const *bufs, const uint64_t *lens, const char *const *names, uint32_t n,
                           uint8_t *index_bits, uint32_t index_mask, uint64_t *elem_count, orc_digest *outs,
                           int *status);
void orc_digest_many(const uint8_t *const *bufs, const uint64_t *lens, const char *const *names, uint32_t n,
                     uint32_t dd_block_size, int nthreads, orc_digest *outs, int *status);

/* Base64 (RFC 4648, '=' padding) as produced by base64/modp_b64.cc. */
size_t orc_b64_encode(const uint8_t *in, size_t len, char *out);

#ifdef __cplusplus
}
#endif
#endif

/*
 * sdbf_oracle.c -- plain-C restatement of sdhash's hot paths (the ORACLE).
 *
 * Test infrastructure only: tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py load it as a checker / baseline.  The product
 * (sdhash_gb300/) never links or calls it.
 *
 * Parity: pinned against the reference sdhash compiled from its own sources
 * (oracle/Makefile.ref -> oracle/_ref/libsdbf_ref.so) by
 * tests/test_oracle_vs_reference.py and the fixtures in tests/golden/.
 *
 * SHA-1 is the third-party piece: the reference calls OpenSSL's SHA1()
 * (sdbf/sdbf_core.cc:105,160; OpenSSL version not pinned by the reference,
 * 3.0.13 in the build container).  It is restated here from FIPS 180-4 and
 * checked against the FIPS known-answer vectors and Python's hashlib.
 */
#include "sdbf_oracle.h"
#include "../sdhash_gb300/csrc/sdbf_tables.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define ORC_WIN 64                 /* entr_win_size / pop_win_size, sdbf_conf.cc:22,25 */
#define ORC_SYNC 4096              /* entropy resync period, sdbf_conf.cc:24 */
#define ORC_THRESHOLD 16           /* selection threshold, sdbf_conf.cc:29 */
#define ORC_MAX_ELEM 160           /* sdbf_defines.h:34 */
#define ORC_MAX_ELEM_DD 192        /* sdbf_defines.h:35 */
#define ORC_MIN_FILE 512           /* sdbf_defines.h:56 */
#define ORC_MIN_ELEM 16            /* sdbf_defines.h:58 */
#define ORC_BIG_BYTES 16384        /* sdbf_defines.h:64 */
#define ORC_BIG_ELEM 8738          /* sdbf_defines.h:65 */
#define ORC_BIG_MASK 0x1FFFFu      /* bloom_filter.cc:59-63 for 16 KiB */
#define ORC_BF_MASK 0x7FFu         /* BF_CLASS_MASKS[0], sdbf_conf.cc:143 */
#define ORC_CHUNK (32ull << 20)    /* stream chunk, sdbf_class.cc:43,88,123 */

/* ------------------------------------------------------------------ SHA-1 */
static uint32_t rol32(uint32_t v, int s) { return (v << s) | (v >> (32 - s)); }

static void sha1_block(uint32_t h[5], const uint8_t *p) {
    uint32_t w[80];
    for (int t = 0; t < 16; t++)
        w[t] = ((uint32_t)p[4 * t] << 24) | ((uint32_t)p[4 * t + 1] << 16) |
               ((uint32_t)p[4 * t + 2] << 8) | (uint32_t)p[4 * t + 3];
    for (int t = 16; t < 80; t++) w[t] = rol32(w[t - 3] ^ w[t - 8] ^ w[t - 14] ^ w[t - 16], 1);
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4];
    for (int t = 0; t < 80; t++) {
        uint32_t f, k;
        if (t < 20) { f = (b & c) | (~b & d); k = 0x5A827999u; }
        else if (t < 40) { f = b ^ c ^ d; k = 0x6ED9EBA1u; }
        else if (t < 60) { f = (b & c) | (b & d) | (c & d); k = 0x8F1BBCDCu; }
        else { f = b ^ c ^ d; k = 0xCA62C1D6u; }
        uint32_t tmp = rol32(a, 5) + f + e + k + w[t];
        e = d; d = c; c = rol32(b, 30); b = a; a = tmp;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e;
}

void orc_sha1(const uint8_t *msg, uint64_t len, uint8_t out[20]) {
    uint32_t h[5] = {0x67452301u, 0xEFCDAB89u, 0x98BADCFEu, 0x10325476u, 0xC3D2E1F0u};
    uint64_t full = len / 64;
    for (uint64_t i = 0; i < full; i++) sha1_block(h, msg + 64 * i);
    uint8_t tail[128];
    uint64_t rem = len % 64;
    memset(tail, 0, sizeof tail);
    memcpy(tail, msg + 64 * full, rem);
    tail[rem] = 0x80;
    uint64_t tl = (rem < 56) ? 64 : 128;
    uint64_t bits = len * 8;
    for (int i = 0; i < 8; i++) tail[tl - 1 - i] = (uint8_t)(bits >> (8 * i));
    sha1_block(h, tail);
    if (tl == 128) sha1_block(h, tail + 64);
    for (int i = 0; i < 5; i++) {
        out[4 * i] = (uint8_t)(h[i] >> 24);
        out[4 * i + 1] = (uint8_t)(h[i] >> 16);
        out[4 * i + 2] = (uint8_t)(h[i] >> 8);
        out[4 * i + 3] = (uint8_t)h[i];
    }
}

/* The reference reads the 20-byte digest as five native (little-endian on
 * every platform it targets) uint32 words: bf_utils.cc:32-43 casts it. */
static void sha1_words(const uint8_t *x, uint32_t w[5]) {
    uint8_t d[20];
    orc_sha1(x, ORC_WIN, d);
    for (int i = 0; i < 5; i++)
        w[i] = (uint32_t)d[4 * i] | ((uint32_t)d[4 * i + 1] << 8) |
               ((uint32_t)d[4 * i + 2] << 16) | ((uint32_t)d[4 * i + 3] << 24);
}

/* --------------------------------------------------------------- entropy */
void orc_entropy_table(uint64_t table[65]) {
    /* entr64.cc:13-21 */
    table[0] = 0;
    for (int i = 1; i <= 64; i++) {
        double p = (double)i / 64;
        table[i] = (uint64_t)((-p * (log(p) / log((double)2)) / 6) * 1024000);
    }
}

static uint64_t window_entropy(const uint8_t *x, uint8_t cnt[256], const uint64_t *tab) {
    /* entr64_init_int, entr64.cc:27-41 */
    memset(cnt, 0, 256);
    for (int i = 0; i < ORC_WIN; i++) cnt[x[i]]++;
    uint64_t e = 0;
    for (int v = 0; v < 256; v++)
        if (cnt[v]) e += tab[cnt[v]];
    return e;
}

static uint64_t roll_entropy(uint64_t e, const uint8_t *x, uint8_t cnt[256], const uint64_t *tab) {
    /* entr64_inc_int, entr64.cc:47-71: x[0] leaves, x[64] enters. */
    if (x[0] == x[64]) return e;
    uint32_t out_c = cnt[x[0]], in_c = cnt[x[64]];
    cnt[x[0]]--;
    cnt[x[64]]++;
    if (out_c == in_c + 1) return e;
    int64_t d_out = (int64_t)tab[out_c] - (int64_t)tab[out_c - 1];
    int64_t d_in = (int64_t)tab[in_c + 1] - (int64_t)tab[in_c];
    int64_t r = (int64_t)e - d_out + d_in;
    if (r < 0) r = 0;
    else if (r > 1024000) r = 1024000;
    return (uint64_t)r;
}

static uint64_t T[65];
static pthread_once_t entropy_once = PTHREAD_ONCE_INIT;
static void init_entropy(void) { orc_entropy_table(T); }

void orc_ranks(const uint8_t *x, uint64_t n, uint16_t *ranks) {
    /* gen_chunk_ranks, sdbf_core.cc:21-45: rank of every window start o with
     * o < n-64; the last 64 positions (and everything when n <= 64) stay 0. */
    pthread_once(&entropy_once, init_entropy);
    memset(ranks, 0, n * sizeof(uint16_t));
    if (n <= ORC_WIN) return;
    uint8_t cnt[256];
    uint64_t e = 0;
    for (uint64_t o = 0; o < n - ORC_WIN; o++) {
        if (o % ORC_SYNC == 0) e = window_entropy(x + o, cnt, T);
        else e = roll_entropy(e, x + o - 1, cnt, T);
        ranks[o] = SDBF_ENTR64_RANKS[e >> 10];
    }
}

/* ------------------------------------------------------- popularity score */
void orc_scores(const uint16_t *r, uint64_t n, uint16_t *score, int32_t *histo) {
    /* gen_chunk_scores, sdbf_core.cc:50-89, restated step for step including
     * its quirks: the "cheap slide" tests r[i+64] (not r[i+63]) and may credit
     * a position just outside the window; a full rescan picks the leftmost
     * smallest non-zero rank and extends it over an equal right neighbour run. */
    memset(score, 0, n * sizeof(uint16_t));
    if (n <= ORC_WIN) return;
    const uint64_t last = n - ORC_WIN;
    uint64_t mpos = 0;
    uint16_t mrank = r[0];
    for (uint64_t i = 0; i < last; i++) {
        if (i > 0 && mrank > 0) {
            while (r[i + ORC_WIN] >= mrank && i < mpos && i < last + 1) {
                if (r[i + ORC_WIN] == mrank) mpos = i + ORC_WIN;
                score[mpos]++;
                i++;
            }
        }
        mpos = i;
        mrank = r[i];
        for (uint64_t j = i + 1; j < i + ORC_WIN; j++) {
            if (r[j] != 0 && r[j] < mrank) {
                mrank = r[j];
                mpos = j;
            } else if (mpos + 1 == j && r[j] == mrank) {
                mpos = j;
            }
        }
        if (r[mpos] > 0) score[mpos]++;
    }
    if (histo)
        for (uint64_t i = 0; i < last; i++) histo[score[i]]++;
}

/* ------------------------------------------------------------ Bloom bits */
static uint32_t bf_insert5(uint8_t *bf, const uint32_t h[5]) {
    /* bf_sha1_insert, bf_utils.cc:32-43: number of bits newly set. */
    uint32_t added = 0;
    for (int i = 0; i < 5; i++) {
        uint32_t pos = h[i] & ORC_BF_MASK;
        uint8_t bit = (uint8_t)(1u << (pos & 7));
        if (!(bf[pos >> 3] & bit)) added++;
        bf[pos >> 3] |= bit;
    }
    return added;
}

static int big_insert5(uint8_t *big, const uint32_t h[5]) {
    /* bloom_filter::query_and_set(mode_set=true), bloom_filter.cc:333-359:
     * true iff fewer than 5 probed bits were already set. */
    int already = 0;
    for (int i = 0; i < 5; i++) {
        uint32_t pos = h[i] & ORC_BIG_MASK;
        uint8_t bit = (uint8_t)(1u << (pos & 7));
        if (big[pos >> 3] & bit) already++;
        else big[pos >> 3] |= bit;
    }
    return already < 5;
}

static void compute_hamming(orc_digest *d) {
    /* compute_hamming, sdbf_class.cc:388-401 */
    d->hamming = (uint16_t *)calloc(d->bf_count ? d->bf_count : 1, sizeof(uint16_t));
    for (uint32_t i = 0; i < d->bf_count; i++) {
        uint32_t c = 0;
        for (int k = 0; k < 256; k++) c += (uint32_t)__builtin_popcount(d->filters[256u * i + k]);
        d->hamming[i] = (uint16_t)c;
    }
}

static char *dup_name(const char *name) {
    size_t l = strlen(name);
    char *s = (char *)malloc(l + 1);
    memcpy(s, name, l + 1);
    return s;
}

static int index_insert5(uint8_t *bits, uint32_t mask, const uint32_t h[5]) {
    /* bloom_filter::insert_sha1 = query_and_set(mode_set=true),
     * bloom_filter.cc:311-359: sets the probed bits; true iff one was new. */
    int fresh = 0;
    for (int i = 0; i < 5; i++) {
        uint32_t pos = h[i] & mask;
        uint8_t bit = (uint8_t)(1u << (pos & 7));
        if (!(bits[pos >> 3] & bit)) fresh = 1;
        bits[pos >> 3] |= bit;
    }
    return fresh;
}

/* ----------------------------------------------------------- stream mode */
static int digest_stream(const char *name, const uint8_t *x, uint64_t len, uint8_t *index_bits, uint32_t index_mask,
                         uint64_t *elem_count, orc_digest *d);

int orc_digest_stream(const char *name, const uint8_t *x, uint64_t len, orc_digest *d) {
    return digest_stream(name, x, len, NULL, 0, NULL, d);
}

int orc_index_build_stream(const uint8_t *const *bufs, const uint64_t *lens, const char *const *names, uint32_t n,
                           uint8_t *index_bits, uint32_t index_mask, uint64_t *elem_count, orc_digest *outs,
                           int *status) {
    /* hash_index_stringlist's stream path for one group (sdhash_threads.cc:
     * 402-416 with -p 1: sdbf_hash_files, :249-270): files in order, one
     * shared index */
    for (uint32_t i = 0; i < n; i++)
        status[i] = digest_stream(names[i], bufs[i], lens[i], index_bits, index_mask, elem_count, &outs[i]);
    return 0;
}

static int digest_stream(const char *name, const uint8_t *x, uint64_t len, uint8_t *index_bits, uint32_t index_mask,
                         uint64_t *elem_count, orc_digest *d) {
    memset(d, 0, sizeof *d);
    if (len < ORC_MIN_FILE) return -3;
    d->name = dup_name(name);
    d->orig_size = len;
    d->max_elem = ORC_MAX_ELEM;
    d->bf_count = 1;
    d->last_count = 0;
    /* buffer estimate, sdbf_core.cc:202-204 (never exceeded: at most one
     * counted feature per 17 credited window steps) */
    uint64_t cap = ((len >> 11) + 1) << 8;
    if (cap < 256) cap = 256;
    d->filters = (uint8_t *)calloc(cap, 1);
    uint64_t chunk = len < ORC_CHUNK ? len : ORC_CHUNK;
    uint16_t *ranks = (uint16_t *)malloc(chunk * sizeof(uint16_t));
    uint16_t *scores = (uint16_t *)malloc(chunk * sizeof(uint16_t));
    uint8_t *big = (uint8_t *)calloc(ORC_BIG_BYTES, 1);
    uint8_t *cur = d->filters;
    for (uint64_t pos = 0; pos < len; pos += ORC_CHUNK) {
        /* full 32 MiB chunks, then the remainder (sdbf_core.cc:214-232) */
        uint64_t n = len - pos < ORC_CHUNK ? len - pos : ORC_CHUNK;
        orc_ranks(x + pos, n, ranks);
        orc_scores(ranks, n, scores, NULL);
        /* gen_chunk_hash, sdbf_core.cc:93-136; the big-filter element counter
         * is local to each chunk (:100), the big filter itself is not. */
        uint32_t bigfi = 0;
        if (n <= ORC_WIN) continue;
        for (uint64_t i = 0; i < n - ORC_WIN; i++) {
            if (scores[i] <= ORC_THRESHOLD) continue;
            uint32_t h[5];
            sha1_words(x + pos + i, h);
            if (bf_insert5(cur, h) == 0) continue;
            /* with an index being built (sdbf_core.cc:108-114) */
            if (index_bits) {
                if (!index_insert5(index_bits, index_mask, h)) continue;
                (*elem_count)++;
            }
            if (!big_insert5(big, h)) continue;
            d->last_count++;
            bigfi++;
            if (d->last_count == ORC_MAX_ELEM) {
                cur += 256;
                d->bf_count++;
                d->last_count = 0;
            }
            if (bigfi == ORC_BIG_ELEM) {
                memset(big, 0, ORC_BIG_BYTES);
                bigfi = 0;
            }
        }
    }
    /* drop a nearly empty last filter, sdbf_core.cc:235-238 */
    if (d->bf_count > 1 && d->last_count < ORC_MAX_ELEM / 8) {
        d->bf_count--;
        d->last_count = ORC_MAX_ELEM;
    }
    free(ranks);
    free(scores);
    free(big);
    compute_hamming(d);
    return 0;
}

/* ------------------------------------------------------------ block mode */
/* The index list of an index search (index_info::setlist, sdbf/index_info.h). */
typedef struct {
    const uint8_t *const *bits;
    const uint32_t *masks;
    const uint32_t *hash_counts;
    uint32_t n;
} orc_index_list;

static void block_hash(const uint8_t *data, uint64_t n, const uint16_t *scores, uint32_t k,
                       int32_t allowed, uint8_t *bf, uint16_t *count, const orc_index_list *idx,
                       uint8_t *hits) {
    /* gen_block_hash, sdbf_core.cc:141-191; with an index list, counted
     * features 0, 4, 8, ... are looked up in every index (check_indexes,
     * :482-493; bloom_filter::query_sha1 = all hash bits set) */
    uint32_t hashed = 0;
    for (uint64_t i = 0; i < n - ORC_WIN && hashed < ORC_MAX_ELEM_DD; i++) {
        if (scores[i] > k || (scores[i] == k && allowed > 0)) {
            uint32_t h[5];
            sha1_words(data + i, h);
            if (bf_insert5(bf, h) == 0) continue;
            if (idx && hashed % 4 == 0) {
                for (uint32_t x = 0; x < idx->n; x++) {
                    uint32_t all = 1;
                    for (uint32_t z = 0; z < idx->hash_counts[x] && all; z++) {
                        const uint32_t pos = h[z] & idx->masks[x];
                        all = (idx->bits[x][pos >> 3] >> (pos & 7)) & 1u;
                    }
                    hits[x] += (uint8_t)all;
                }
            }
            hashed++;
            if (scores[i] == k) allowed--;
        }
    }
    *count = (uint16_t)hashed;
}

static int digest_block_idx(const char *name, const uint8_t *x, uint64_t len, uint32_t B, orc_digest *d,
                            const orc_index_list *idx, uint8_t *hits);

int orc_digest_block(const char *name, const uint8_t *x, uint64_t len, uint32_t B,
                     orc_digest *d) {
    return digest_block_idx(name, x, len, B, d, NULL, NULL);
}

int orc_index_search_block(const char *name, const uint8_t *x, uint64_t len, uint32_t B,
                           const uint8_t *const *bits, const uint32_t *masks, const uint32_t *hash_counts,
                           uint32_t nidx, orc_digest *d, uint8_t *hits) {
    const orc_index_list idx = {bits, masks, hash_counts, nidx};
    return digest_block_idx(name, x, len, B, d, &idx, hits);
}

static int digest_block_idx(const char *name, const uint8_t *x, uint64_t len, uint32_t B, orc_digest *d,
                            const orc_index_list *idx, uint8_t *hits) {
    memset(d, 0, sizeof *d);
    if (len < ORC_MIN_FILE) return -3;
    d->name = dup_name(name);
    d->orig_size = len;
    d->max_elem = ORC_MAX_ELEM_DD;
    d->dd_block_size = B;
    uint64_t qt = len / B, rem = len % B;
    d->bf_count = (uint32_t)(qt + (rem >= ORC_MIN_FILE ? 1 : 0));
    d->filters = (uint8_t *)calloc((size_t)d->bf_count * 256 + 256, 1);
    d->elem_counts = (uint16_t *)calloc(d->bf_count + 1, sizeof(uint16_t));
    uint16_t *ranks = (uint16_t *)malloc((size_t)B * sizeof(uint16_t));
    uint16_t *scores = (uint16_t *)malloc((size_t)B * sizeof(uint16_t));
    for (uint64_t b = 0; b < qt; b++) {
        /* thread_gen_block_sdbf, sdbf_core.cc:266-277 */
        int32_t histo[66];
        memset(histo, 0, sizeof histo);
        orc_ranks(x + b * B, B, ranks);
        orc_scores(ranks, B, scores, histo);
        uint32_t k = 65, sum = 0;
        for (; k >= ORC_THRESHOLD; k--) {
            if (sum <= ORC_MAX_ELEM_DD && sum + (uint32_t)histo[k] > ORC_MAX_ELEM_DD) break;
            sum += (uint32_t)histo[k];
        }
        block_hash(x + b * B, B, scores, k, (int32_t)(ORC_MAX_ELEM_DD - sum),
                   d->filters + 256 * b, &d->elem_counts[b], idx, idx ? hits + b * idx->n : NULL);
    }
    if (rem >= ORC_MIN_FILE) {
        /* tail block, sdbf_core.cc:309-319: threshold 16, allowed 192 */
        orc_ranks(x + qt * B, rem, ranks);
        orc_scores(ranks, rem, scores, NULL);
        block_hash(x + qt * B, rem, scores, ORC_THRESHOLD, ORC_MAX_ELEM_DD,
                   d->filters + 256 * qt, &d->elem_counts[qt], idx, idx ? hits + qt * idx->n : NULL);
    }
    free(ranks);
    free(scores);
    compute_hamming(d);
    return 0;
}

void orc_digest_free(orc_digest *d) {
    free(d->name);
    free(d->filters);
    free(d->elem_counts);
    free(d->hamming);
    memset(d, 0, sizeof *d);
}

/* ------------------------------------------------------------- comparing */
int32_t orc_elem_count(const orc_digest *d, uint64_t idx) {
    if (!d->elem_counts) return idx < d->bf_count - 1 ? (int32_t)d->max_elem : (int32_t)d->last_count;
    return d->elem_counts[idx];
}

static uint32_t pc64(const uint8_t *a, const uint8_t *b, int w0, int w1) {
    uint32_t c = 0;
    for (int w = w0; w < w1; w++) {
        uint64_t x, y;
        memcpy(&x, a + 8 * w, 8);
        memcpy(&y, b + 8 * w, 8);
        c += (uint32_t)__builtin_popcountll(x & y);
    }
    return c;
}

uint32_t orc_match_cut(const uint8_t *f1, const uint8_t *f2, uint32_t cut) {
    /* bf_bitcount_cut_256_asm, bf_utils.cc:114-206, slack 48, followed by the
     * full recount of sdbf_core.cc:435-437 (which returns the same total). */
    const uint32_t slack = 48;
    uint32_t c = pc64(f1, f2, 0, 4);
    if (cut > 0 && 8 * c + slack < cut) return 0;
    c += pc64(f1, f2, 4, 8);
    if (cut > 0 && 4 * c + slack < cut) return 0;
    c += pc64(f1, f2, 8, 16);
    if (cut > 0 && 2 * c + slack < cut) return 0;
    c += pc64(f1, f2, 16, 32);
    return c;
}

static uint32_t orc_match_cut_64(const uint8_t *f1, const uint8_t *f2, uint32_t cut) {
    /* bf_bitcount_cut_64_asm, bf_utils.cc:78-110 (first 64 bytes, one stage:
     * 2c + slack < cut after 32 bytes), then the full recount */
    const uint32_t slack = 48;
    uint32_t c = pc64(f1, f2, 0, 4);
    if (cut > 0 && 2 * c + slack < cut) return 0;
    c += pc64(f1, f2, 4, 8);
    return c;
}

void orc_fast(orc_digest *d) {
    for (uint32_t i = 0; i < d->bf_count; i++) {
        uint8_t *f = d->filters + 256ull * i;
        uint64_t w[32], h = 0;
        memcpy(w, f, 256);
        for (int j = 0; j < 16; j++) w[j] |= w[j + 16];  /* fold 1: 256 -> 128 bytes */
        for (int j = 0; j < 8; j++) w[j] |= w[j + 8];    /* fold 2: 128 -> 64 bytes */
        memcpy(f, w, 64);                                /* only the folded 64 bytes are copied back */
        for (int j = 0; j < 8; j++) h += (uint64_t)__builtin_popcountll(w[j]);
        d->hamming[i] = (uint16_t)h;
    }
    d->fastmode = 1;
}

double orc_max_score(const orc_digest *ref, uint32_t ri, const orc_digest *tgt) {
    /* sdbf_max_score, sdbf_core.cc:395-455; the reference digest's fastmode
     * selects CUTOFFS64 and the 64-byte count (:422-440) */
    uint32_t s1 = (uint32_t)orc_elem_count(ref, ri);
    if (s1 < ORC_MIN_ELEM) return 0;
    const uint8_t *f1 = ref->filters + 256ull * ri;
    uint32_t e1 = ref->hamming[ri];
    double best = -1;
    for (uint32_t j = 0; j < tgt->bf_count; j++) {
        uint32_t s2 = (uint32_t)orc_elem_count(tgt, j);
        if (s2 < ORC_MIN_ELEM) continue;
        uint32_t e2 = tgt->hamming[j];
        uint32_t max_est = e1 < e2 ? e1 : e2;
        uint32_t cut, match;
        if (!ref->fastmode) {
            cut = SDBF_CUTOFFS256[4096 / (s1 + s2)];
            match = orc_match_cut(f1, tgt->filters + 256ull * j, cut);
        } else {
            cut = SDBF_CUTOFFS64[1024 / (s1 + s2)];
            match = orc_match_cut_64(f1, tgt->filters + 256ull * j, cut);
        }
        double s = (match <= cut) ? 0 : (double)(match - cut) / (double)(max_est - cut);
        if (s > best) best = s;
    }
    return best;
}

static double round_half_away(double v) { return v < 0 ? -floor(-v + 0.5) : floor(v + 0.5); }

int32_t orc_score(const orc_digest *a, const orc_digest *b) {
    /* sdbf_score, sdbf_core.cc:330-389 with sample == 0 */
    uint32_t n1 = a->bf_count;
    if (n1 > b->bf_count ||
        (n1 == b->bf_count &&
         (orc_elem_count(a, n1 - 1) > orc_elem_count(b, b->bf_count - 1) ||
          strcmp(a->name, b->name) > 0))) {
        const orc_digest *t = a;
        a = b;
        b = t;
        n1 = a->bf_count;
    }
    double sum = -1;
    uint32_t sparse = 0;
    for (uint32_t i = 0; i < n1; i++) {
        double m = orc_max_score(a, i, b);
        sum = (sum < 0) ? m : sum + m;
        if (orc_elem_count(a, i) < ORC_MIN_ELEM) sparse++;
    }
    uint64_t denom = n1;
    if (n1 > 1) denom -= sparse;
    if (denom == 0) sum = -1;
    if (sum < 0) return -1;
    /* boost::math::round: half away from zero (sdbf_core.cc:387) */
    return (int32_t)round_half_away(100.0 * sum / (double)denom);
}

/* ----------------------------------------------------------- SDBF text */
static const char B64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

size_t orc_b64_encode(const uint8_t *in, size_t len, char *out) {
    size_t o = 0, i = 0;
    for (; i + 2 < len; i += 3) {
        uint32_t v = ((uint32_t)in[i] << 16) | ((uint32_t)in[i + 1] << 8) | in[i + 2];
        out[o++] = B64[v >> 18];
        out[o++] = B64[(v >> 12) & 63];
        out[o++] = B64[(v >> 6) & 63];
        out[o++] = B64[v & 63];
    }
    if (i < len) {
        uint32_t v = (uint32_t)in[i] << 16;
        if (i + 1 < len) v |= (uint32_t)in[i + 1] << 8;
        out[o++] = B64[v >> 18];
        out[o++] = B64[(v >> 12) & 63];
        out[o++] = (i + 1 < len) ? B64[(v >> 6) & 63] : '=';
        out[o++] = '=';
    }
    out[o] = 0;
    return o;
}

static int b64_val(char c) {
    if (c >= 'A' && c <= 'Z') return c - 'A';
    if (c >= 'a' && c <= 'z') return c - 'a' + 26;
    if (c >= '0' && c <= '9') return c - '0' + 52;
    if (c == '+') return 62;
    if (c == '/') return 63;
    return -1;
}

static long b64_decode(const char *in, size_t len, uint8_t *out) {
    /* strict decode of a '='-padded block; returns bytes or -1 */
    if (len % 4) return -1;
    size_t o = 0;
    for (size_t i = 0; i < len; i += 4) {
        int v[4], pad = 0;
        for (int k = 0; k < 4; k++) {
            if (in[i + k] == '=' && i + 4 == len && k >= 2) { v[k] = 0; pad++; }
            else if ((v[k] = b64_val(in[i + k])) < 0) return -1;
        }
        uint32_t x = ((uint32_t)v[0] << 18) | ((uint32_t)v[1] << 12) | ((uint32_t)v[2] << 6) | (uint32_t)v[3];
        out[o++] = (uint8_t)(x >> 16);
        if (pad < 2) out[o++] = (uint8_t)(x >> 8);
        if (pad < 1) out[o++] = (uint8_t)x;
    }
    return (long)o;
}

char *orc_to_string(const orc_digest *d) {
    size_t nlen = strlen(d->name);
    size_t cap = 256 + nlen + (size_t)d->bf_count * (344 + 8) + 16;
    char *s = (char *)malloc(cap);
    size_t o;
    if (!d->elem_counts) {
        o = (size_t)sprintf(s, "sdbf:03:%d:%s:%llu:sha1:256:5:7ff:%u:%u:%u:", (int)nlen, d->name,
                            (unsigned long long)d->orig_size, d->max_elem, d->bf_count, d->last_count);
        o += orc_b64_encode(d->filters, (size_t)d->bf_count * 256, s + o);
    } else {
        o = (size_t)sprintf(s, "sdbf-dd:03:%d:%s:%llu:sha1:256:5:7ff:%u:%u:%u", (int)nlen, d->name,
                            (unsigned long long)d->orig_size, d->max_elem, d->bf_count, d->dd_block_size);
        for (uint32_t i = 0; i < d->bf_count; i++) {
            o += (size_t)sprintf(s + o, ":%02x:", d->elem_counts[i]);
            o += orc_b64_encode(d->filters + 256ull * i, 256, s + o);
        }
    }
    s[o++] = '\n';
    s[o] = 0;
    return s;
}

static const char *field(const char *p, const char *end, const char **f, size_t *flen) {
    const char *q = p;
    while (q < end && *q != ':') q++;
    *f = p;
    *flen = (size_t)(q - p);
    return q < end ? q + 1 : end;
}

int orc_from_string(const char *line, size_t len, orc_digest *d) {
    /* sdbf(const std::string&), sdbf_class.cc:144-215 (well-formed input) */
    memset(d, 0, sizeof *d);
    while (len && (line[len - 1] == '\n' || line[len - 1] == '\r')) len--;
    if (len < 344) return -1;
    const char *p = line, *end = line + len, *f;
    size_t fl;
    char tmp[64];
    p = field(p, end, &f, &fl);
    if (fl < 4 || strncmp(f, "sdbf", 4)) return -2;
    int dd = (fl == 7 && !strncmp(f, "sdbf-dd", 7));
    p = field(p, end, &f, &fl); /* version */
    p = field(p, end, &f, &fl); /* name length */
    p = field(p, end, &f, &fl); /* name */
    d->name = (char *)malloc(fl + 1);
    memcpy(d->name, f, fl);
    d->name[fl] = 0;
#define NUMF(dst)                                      \
    p = field(p, end, &f, &fl);                        \
    if (fl == 0 || fl >= sizeof tmp) goto bad;         \
    memcpy(tmp, f, fl);                                \
    tmp[fl] = 0;                                       \
    dst = strtoull(tmp, NULL, 10);
    unsigned long long v;
    NUMF(v); d->orig_size = v;
    p = field(p, end, &f, &fl); /* sha1 */
    NUMF(v); if (v != 256) goto bad;
    NUMF(v); /* hash count */
    p = field(p, end, &f, &fl); /* mask */
    NUMF(v); d->max_elem = (uint32_t)v;
    NUMF(v); d->bf_count = (uint32_t)v;
    d->filters = (uint8_t *)calloc((size_t)d->bf_count * 256 + 4, 1);
    if (dd) {
        NUMF(v); d->dd_block_size = (uint32_t)v;
        d->elem_counts = (uint16_t *)calloc(d->bf_count + 1, sizeof(uint16_t));
        for (uint32_t i = 0; i < d->bf_count; i++) {
            p = field(p, end, &f, &fl);
            if (fl == 0 || fl >= sizeof tmp) goto bad;
            memcpy(tmp, f, fl);
            tmp[fl] = 0;
            d->elem_counts[i] = (uint16_t)strtoul(tmp, NULL, 16);
            p = field(p, end, &f, &fl);
            if (fl != 344 || b64_decode(f, 344, d->filters + 256ull * i) != 256) goto bad;
        }
    } else {
        NUMF(v); d->last_count = (uint32_t)v;
        size_t need = 4 * (((size_t)d->bf_count * 256 + 2) / 3);
        if ((size_t)(end - p) < need) goto bad;
        if (b64_decode(p, need, d->filters) != (long)d->bf_count * 256) goto bad;
    }
#undef NUMF
    compute_hamming(d);
    return 0;
bad:
    orc_digest_free(d);
    return -2;
}

/* --------------------------------------------------------- set drivers */
typedef struct {
    char *buf;
    size_t len, cap;
} sbuf;

static void sb_put(sbuf *b, const char *s, size_t n) {
    if (b->len + n + 1 > b->cap) {
        b->cap = (b->cap + n + 1) * 2;
        b->buf = (char *)realloc(b->buf, b->cap);
    }
    memcpy(b->buf + b->len, s, n);
    b->len += n;
    b->buf[b->len] = 0;
}

static void put_line(sbuf *b, const char *n1, const char *n2, int32_t score, char sep) {
    /* sdbf_set.cc:257-261: "%03d" via setw(3)+fill('0'), -1 unpadded */
    char tail[32];
    int k = (score != -1) ? snprintf(tail, sizeof tail, "%c%03d\n", sep, score)
                          : snprintf(tail, sizeof tail, "%c%d\n", sep, score);
    sb_put(b, n1, strlen(n1));
    sb_put(b, &sep, 1);
    sb_put(b, n2, strlen(n2));
    sb_put(b, tail, (size_t)k);
}

char *orc_compare_all(const orc_digest *set, uint32_t n, int32_t threshold, char sep) {
    sbuf b = {0, 0, 0};
    sb_put(&b, "", 0);
    for (uint32_t i = 0; i < n; i++)
        for (uint32_t j = i + 1; j < n; j++) {
            int32_t s = orc_score(&set[i], &set[j]);
            if (s >= threshold) put_line(&b, set[i].name, set[j].name, s, sep);
        }
    return b.buf;
}

char *orc_compare_to(const orc_digest *q, uint32_t nq, const orc_digest *t, uint32_t nt,
                     int32_t threshold, char sep) {
    sbuf b = {0, 0, 0};
    sb_put(&b, "", 0);
    for (uint32_t i = 0; i < nq; i++)
        for (uint32_t j = 0; j < nt; j++) {
            int32_t s = orc_score(&q[i], &t[j]);
            if (s >= threshold) put_line(&b, q[i].name, t[j].name, s, sep);
        }
    return b.buf;
}

/* ------------------------------------------------------ threaded drivers */
static int resolve_threads(int n) {
    if (n > 0) return n;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

typedef struct {
    int tid, nt;
    const orc_digest *a, *b;
    uint32_t na, nb;
    int32_t *out;
    int all;
    const uint32_t *pi, *pj;
    uint64_t np;
} score_task;

static void *score_worker(void *arg) {
    score_task *t = (score_task *)arg;
    if (t->pi) {
        for (uint64_t k = (uint64_t)t->tid; k < t->np; k += (uint64_t)t->nt)
            t->out[k] = orc_score(&t->a[t->pi[k]], &t->a[t->pj[k]]);
    } else if (t->all) {
        for (uint32_t i = (uint32_t)t->tid; i < t->na; i += (uint32_t)t->nt)
            for (uint32_t j = i + 1; j < t->na; j++) t->out[(uint64_t)i * t->na + j] = orc_score(&t->a[i], &t->a[j]);
    } else {
        for (uint32_t i = (uint32_t)t->tid; i < t->na; i += (uint32_t)t->nt)
            for (uint32_t j = 0; j < t->nb; j++) t->out[(uint64_t)i * t->nb + j] = orc_score(&t->a[i], &t->b[j]);
    }
    return NULL;
}

static void run_scores(score_task proto, int nthreads) {
    int nt = resolve_threads(nthreads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
    score_task *ts = (score_task *)malloc(sizeof(score_task) * (size_t)nt);
    for (int i = 0; i < nt; i++) {
        ts[i] = proto;
        ts[i].tid = i;
        ts[i].nt = nt;
        pthread_create(&th[i], NULL, score_worker, &ts[i]);
    }
    for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
    free(th);
    free(ts);
}

void orc_score_all_matrix(const orc_digest *set, uint32_t n, int32_t *out, int nthreads) {
    score_task p;
    memset(&p, 0, sizeof p);
    p.a = set; p.na = n; p.out = out; p.all = 1;
    run_scores(p, nthreads);
}

void orc_score_cross_matrix(const orc_digest *q, uint32_t nq, const orc_digest *t, uint32_t nt,
                            int32_t *out, int nthreads) {
    score_task p;
    memset(&p, 0, sizeof p);
    p.a = q; p.na = nq; p.b = t; p.nb = nt; p.out = out;
    run_scores(p, nthreads);
}

void orc_score_pairs(const orc_digest *set, const uint32_t *pi, const uint32_t *pj, uint64_t np,
                     int32_t *out, int nthreads) {
    score_task p;
    memset(&p, 0, sizeof p);
    p.a = set; p.pi = pi; p.pj = pj; p.np = np; p.out = out;
    run_scores(p, nthreads);
}

typedef struct {
    int tid, nt;
    const uint8_t *const *bufs;
    const uint64_t *lens;
    const char *const *names;
    uint32_t n, dd;
    orc_digest *outs;
    int *status;
} digest_task;

static void *digest_worker(void *arg) {
    digest_task *t = (digest_task *)arg;
    char name[32];
    for (uint32_t i = (uint32_t)t->tid; i < t->n; i += (uint32_t)t->nt) {
        snprintf(name, sizeof name, "f%u", i);
        const char *nm = t->names ? t->names[i] : name;
        t->status[i] = t->dd ? orc_digest_block(nm, t->bufs[i], t->lens[i], t->dd, &t->outs[i])
                             : orc_digest_stream(nm, t->bufs[i], t->lens[i], &t->outs[i]);
    }
    return NULL;
}

typedef struct {
    int id, nt;
    const uint8_t *const *bufs;
    const uint64_t *lens;
    uint32_t n, dd;
    orc_index_list idx;
    uint8_t *const *hits;
    int *status;
} search_task;

static void *search_worker(void *arg) {
    search_task *t = (search_task *)arg;
    for (uint32_t i = (uint32_t)t->id; i < t->n; i += (uint32_t)t->nt) {
        orc_digest d;
        t->status[i] = digest_block_idx("", t->bufs[i], t->lens[i], t->dd, &d, &t->idx, t->hits[i]);
        if (t->status[i] == 0) orc_digest_free(&d);
    }
    return NULL;
}

void orc_index_search_many(const uint8_t *const *bufs, const uint64_t *lens, uint32_t n, uint32_t dd,
                           const uint8_t *const *bits, const uint32_t *masks, const uint32_t *hash_counts,
                           uint32_t nidx, int nthreads, uint8_t *const *hits, int *status) {
    int nt = resolve_threads(nthreads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
    search_task *ts = (search_task *)malloc(sizeof(search_task) * (size_t)nt);
    for (int i = 0; i < nt; i++) {
        search_task d = {i, nt, bufs, lens, n, dd, {bits, masks, hash_counts, nidx}, hits, status};
        ts[i] = d;
        pthread_create(&th[i], NULL, search_worker, &ts[i]);
    }
    for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
    free(th);
    free(ts);
}

void orc_digest_many(const uint8_t *const *bufs, const uint64_t *lens, const char *const *names, uint32_t n,
                     uint32_t dd, int nthreads, orc_digest *outs, int *status) {
    int nt = resolve_threads(nthreads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
    digest_task *ts = (digest_task *)malloc(sizeof(digest_task) * (size_t)nt);
    for (int i = 0; i < nt; i++) {
        digest_task d = {i, nt, bufs, lens, names, n, dd, outs, status};
        ts[i] = d;
        pthread_create(&th[i], NULL, digest_worker, &ts[i]);
    }
    for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
    free(th);
    free(ts);
}

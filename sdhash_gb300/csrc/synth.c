/*
 * synth.c -- seeded synthetic inputs for the digest / compare workloads.
 *
 * The reference measures on no public dataset; every workload here is made
 * of seeded synthetic bytes with the shapes the benchmark configurations ask
 * for (uniform random files, derived "partner" files, and a content mixture of
 * random regions, low-entropy runs and order-1 Markov text).  Deterministic on
 * every platform: a xoshiro256** stream per (seed, stream id), no libc rand.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { uint64_t s[4]; } rng_t;

static uint64_t splitmix(uint64_t *x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void rng_seed(rng_t *r, uint64_t seed, uint64_t stream) {
    uint64_t x = seed * 0x2545F4914F6CDD1Dull + stream * 0x9E3779B97F4A7C15ull + 0x1234567ull;
    for (int i = 0; i < 4; i++) r->s[i] = splitmix(&x);
}

static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }

static uint64_t rng_next(rng_t *r) {
    uint64_t *s = r->s;
    uint64_t out = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return out;
}

/* uniform in [lo, hi] */
static uint64_t rng_range(rng_t *r, uint64_t lo, uint64_t hi) {
    return lo + rng_next(r) % (hi - lo + 1);
}

static void fill_random(rng_t *r, uint8_t *out, uint64_t n) {
    uint64_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t v = rng_next(r);
        memcpy(out + i, &v, 8);
    }
    if (i < n) {
        uint64_t v = rng_next(r);
        memcpy(out + i, &v, (size_t)(n - i));
    }
}

void synth_fill_random(uint64_t seed, uint64_t stream, uint8_t *out, uint64_t n) {
    rng_t r;
    rng_seed(&r, seed, stream);
    fill_random(&r, out, n);
}

/* Partner of a base file: a seeded 30% of its aligned 4 KiB blocks replaced
 * by fresh random bytes, then one insertion of 1..63 random bytes at 90% of
 * the length (so the last 10% of the bytes are shifted), truncated back to n. */
void synth_partner(uint64_t seed, uint64_t stream, const uint8_t *base, uint8_t *out, uint64_t n) {
    rng_t r;
    rng_seed(&r, seed, stream ^ 0xABCDEF0123ull);
    memcpy(out, base, (size_t)n);
    uint64_t nblocks = n / 4096;
    uint64_t nrep = (uint64_t)floor(0.3 * (double)nblocks + 0.5);
    uint8_t *picked = (uint8_t *)calloc(nblocks ? nblocks : 1, 1);
    for (uint64_t k = 0; k < nrep && nblocks; k++) {
        uint64_t b;
        do { b = rng_range(&r, 0, nblocks - 1); } while (picked[b]);
        picked[b] = 1;
        fill_random(&r, out + 4096 * b, 4096);
    }
    free(picked);
    uint64_t at = n - n / 10;
    uint64_t ins = rng_range(&r, 1, 63);
    if (at < n) {
        uint64_t keep = n - at - ins > n ? 0 : n - at - ins;
        memmove(out + at + ins, out + at, (size_t)keep);
        uint8_t tmp[64];
        fill_random(&r, tmp, ins);
        uint64_t w = ins < n - at ? ins : n - at;
        memcpy(out + at, tmp, (size_t)w);
    }
}

/* Per-file content mixture: segments of U[64, 65536] bytes, each one of
 *   50% uniform random bytes,
 *   25% low-entropy runs (alphabet of 1..4 random symbols, runs U[16,4096]),
 *   25% order-1 Markov text over printable ASCII 0x20..0x7E with seeded
 *       transition weights (one weight table per file). */
void synth_fill_mixture(uint64_t seed, uint64_t stream, uint8_t *out, uint64_t n) {
    rng_t r;
    rng_seed(&r, seed, stream);
    /* Transition table: for each current symbol, 256 slots of next symbols in
     * proportion to Dirichlet(1)-like weights sharpened by a cube, which gives
     * text-like (moderate) entropy. */
    uint8_t *trans = (uint8_t *)malloc(95 * 256);
    for (int c = 0; c < 95; c++) {
        uint64_t w[95], tot = 0;
        for (int k = 0; k < 95; k++) {
            uint64_t v = rng_range(&r, 1, 64);
            w[k] = v * v * v; /* heavy-tailed weights -> text-like entropy */
            tot += w[k];
        }
        int slot = 0;
        uint64_t acc = 0;
        for (int k = 0; k < 95; k++) {
            acc += w[k];
            int upto = (int)((acc * 256 + tot / 2) / tot);
            if (k == 94) upto = 256;
            while (slot < upto && slot < 256) trans[c * 256 + slot++] = (uint8_t)k;
        }
    }
    uint64_t pos = 0;
    uint8_t cur = (uint8_t)rng_range(&r, 0, 94);
    while (pos < n) {
        uint64_t len = rng_range(&r, 64, 65536);
        if (len > n - pos) len = n - pos;
        uint64_t kind = rng_range(&r, 0, 3);
        if (kind <= 1) {
            fill_random(&r, out + pos, len);
        } else if (kind == 2) {
            uint8_t alpha[4];
            int na = (int)rng_range(&r, 1, 4);
            for (int k = 0; k < na; k++) alpha[k] = (uint8_t)rng_next(&r);
            uint64_t p = 0;
            while (p < len) {
                uint64_t run = rng_range(&r, 16, 4096);
                if (run > len - p) run = len - p;
                memset(out + pos + p, alpha[rng_range(&r, 0, (uint64_t)na - 1)], (size_t)run);
                p += run;
            }
        } else {
            uint64_t bits = 0;
            int have = 0;
            for (uint64_t p = 0; p < len; p++) {
                if (have == 0) { bits = rng_next(&r); have = 8; }
                cur = trans[cur * 256 + (bits & 0xFF)];
                bits >>= 8;
                have--;
                out[pos + p] = (uint8_t)(0x20 + cur);
            }
        }
        pos += len;
    }
    free(trans);
}

/* sizes = round(lo * (hi/lo)^u), u uniform in [0,1) with 24-bit resolution.
 * (hi/lo)^u is a product of repeated square roots selected by the bits of u:
 * only correctly rounded IEEE operations, so every platform gets the same
 * sizes (libm exp/log are not bit-identical across libraries). */
void synth_log_uniform_sizes(uint64_t seed, uint32_t count, uint64_t lo, uint64_t hi, uint64_t *out) {
    rng_t r;
    rng_seed(&r, seed, 0x51AE5ull);
    double root[24];
    double q = (double)hi / (double)lo;
    for (int i = 0; i < 24; i++) {
        q = sqrt(q);
        root[i] = q;
    }
    for (uint32_t i = 0; i < count; i++) {
        uint32_t u = (uint32_t)(rng_next(&r) >> 40); /* 24 bits */
        double v = (double)lo;
        for (int b = 0; b < 24; b++)
            if (u & (1u << (23 - b))) v *= root[b];
        uint64_t s = (uint64_t)floor(v + 0.5);
        if (s < lo) s = lo;
        if (s > hi) s = hi;
        out[i] = s;
    }
}

typedef struct {
    int tid, nt, kind;
    uint64_t seed;
    uint32_t n;
    const uint64_t *offs, *sizes;
    uint8_t *out;
} fill_task;

static void *fill_worker(void *arg) {
    fill_task *t = (fill_task *)arg;
    for (uint32_t i = (uint32_t)t->tid; i < t->n; i += (uint32_t)t->nt) {
        if (t->kind == 0) synth_fill_random(t->seed, i, t->out + t->offs[i], t->sizes[i]);
        else synth_fill_mixture(t->seed, i, t->out + t->offs[i], t->sizes[i]);
    }
    return NULL;
}

/* Fill n files (file i at out+offs[i], sizes[i] bytes) on nthreads threads.
 * kind 0 = uniform random, 1 = mixture.  Content of file i depends only on
 * (seed, i), never on the thread count. */
void synth_fill_many(uint64_t seed, int kind, uint32_t n, const uint64_t *offs,
                     const uint64_t *sizes, uint8_t *out, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    pthread_t th[256];
    fill_task ts[256];
    if (nthreads > 256) nthreads = 256;
    for (int i = 0; i < nthreads; i++) {
        fill_task f = {i, nthreads, kind, seed, n, offs, sizes, out};
        ts[i] = f;
        pthread_create(&th[i], NULL, fill_worker, &ts[i]);
    }
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
}

// gen_kernels.cu -- SDBF digest generation on sm_103a.
//
// Restates sdhash's generation path (sdbf/sdbf_core.cc:21-324) as three
// kernels over a batch of files resident in HBM:
//
//  k_stream_tiles   one CTA per tile of kTileL window steps of a 32 MiB
//                   stream chunk: bytes -> ranks (rolling 64-byte entropy,
//                   gen_chunk_ranks :21-45) -> popularity scores
//                   (gen_chunk_scores :50-89, parallelised below) ->
//                   selection score > 16 -> SHA-1 of every selected 64-byte
//                   feature.  Writes the ordered feature digests of the tile.
//  k_stream_check   one warp per chunk: finds the first tile whose
//                   speculative entry state differs from its predecessor's
//                   exit state.
//  k_stream_fix     one CTA per chunk with such a tile (others exit at
//                   once): recomputes tiles in place from the true state.
//  k_stream_commit  one warp per file: the ordered filter fill of
//                   gen_chunk_hash (:93-136) -- 256-byte filter insert with
//                   zero-new-bit suppression, the 16 KiB "big filter"
//                   dedupe (bloom_filter.cc:333-359), roll-over at 160
//                   elements, big-filter roll-over at 8738 per chunk, and the
//                   final chop (:235-238).
//  k_block_digest   one CTA per dd block (gen_block_sdbf_mt :251-324,
//                   gen_block_hash :141-191): histogram threshold, <=192
//                   ordered inserts.
//
// Popularity scores in parallel.  gen_chunk_scores is a sequential state
// machine over window steps i with state (P, M) = (min_pos, min_rank).  A
// step is either a "cheap slide" (depends on (P, M) and rank[i+64]) or a full
// rescan of window [i, i+63], whose result depends on i only.  Hence two
// walks that reach the same state at the same step agree from then on.  Each
// thread walks one segment of steps, starting kLead steps early with an
// assumed full rescan; the state it reaches at its segment start is compared
// with the state its left neighbour reaches at the same step.  Equal states
// prove the segment exact (induction from step 0, which is always a full
// rescan); a mismatch is re-walked from the neighbour's state.  The same
// check links consecutive tiles of a chunk (k_stream_check / k_stream_fix).
#include <cstdint>
#include <cuda_runtime.h>

#include "gen_kernels.h"
#include "sdbf_device.cuh"

namespace sdbfg {

// ------------------------------------------------------------ smem layout
struct TileGeom {
    uint32_t n;      // chunk length
    uint32_t t0;     // first step owned by the tile
    uint32_t S0;     // first step whose credits the tile needs (t0-64, or 0)
    uint32_t SE;     // end of steps (exclusive), <= n-64
    uint32_t Q0;     // first step simulated (lead-in), multiple of 64 rel. chunk
    uint32_t RE;     // end of rank positions (exclusive)
    uint32_t BE;     // end of bytes (exclusive)
    uint32_t L;      // positions owned: [t0, t0+L)
};

// Shared-memory carve-up for a tile of at most Lmax owned positions.
struct TileSmem {
    uint32_t* bytes32;     // chunk bytes [Q0, BE) (+pad)
    uint16_t* ranks;       // ranks [Q0, RE)
    uint8_t* hist;         // per-thread byte histograms (phase 2 only)
    uint16_t* fres;        // full-rescan result per step [Q0, SE)
    uint32_t* score32;     // u8 scores of [t0, t0+L) packed 4 per word
    uint32_t* list;        // selected positions (relative to t0)
    uint64_t* sig;         // per-segment entry state
    uint64_t* tau;         // per-segment exit state
    uint32_t* own;         // block mode, insert phase: 2,048 owner masks over dead space
    uint32_t* misc;        // scalars
};

__host__ __device__ constexpr uint32_t align_up(uint32_t v, uint32_t a) { return (v + a - 1) / a * a; }

// Padded index of the per-position uint16 arrays (ranks, full-rescan
// results): one spare word after every 64 entries, so 32 lanes that each
// scan their own aligned 64-position block address 32 different banks.
__host__ __device__ constexpr uint32_t pidx(uint32_t o) { return o + 2 * (o >> 6); }
__host__ __device__ constexpr uint32_t padded_len(uint32_t n) { return pidx(n) + 2; }

// Byte address of thread t's counter for byte value v in the histogram area:
// each lane's 256 counters occupy 64 words of its own bank.
static_assert(kRankThreads % 32 == 0, "histogram layout assumes full warps");
__device__ __forceinline__ uint32_t hist_off(uint32_t t, uint32_t v) {
    return ((((t >> 5) * 64 + (v >> 2)) * 32 + (t & 31)) << 2) | (v & 3);
}

// Layout: bytes | ranks | union { histograms (ranks phase) ;
//                                 fres | scores | list | sig | tau } | misc
__host__ __device__ inline uint32_t phase3_bytes(uint32_t Lmax) {
    return align_up(padded_len(Lmax + 64 + kLead) * 2, 16) + align_up(Lmax + 16, 16) +
           align_up(((Lmax + 64) / 15 + 8) * 4, 16) + 2 * kSegs * 8;
}

// Offset in the union of the block-mode insert's owner table (8 KiB): the
// full-rescan table when it is that large (dead once the scores are
// known), else past the phase-3 layout.
constexpr uint32_t kOwnBytes = 2048 * 4;
__host__ __device__ inline uint32_t own_offset(uint32_t Lmax) {
    return align_up(padded_len(Lmax + 64 + kLead) * 2, 16) >= kOwnBytes ? 0u : phase3_bytes(Lmax);
}

__host__ __device__ inline uint32_t union_bytes(uint32_t Lmax) {
    const uint32_t hist = 256 * kRankThreads, p3 = phase3_bytes(Lmax), own = own_offset(Lmax) + kOwnBytes;
    return max(max(hist, p3), own);
}

__host__ __device__ inline uint32_t tile_smem_bytes(uint32_t Lmax) {
    const uint32_t span = Lmax + 64 + kLead + 64;           // rank positions
    uint32_t b = 0;
    b += align_up(span + 64 + 16, 16);                       // bytes
    b += align_up(padded_len(span) * 2, 16);                 // ranks
    b += union_bytes(Lmax);                                  // union
    b += 64 * 4;                                             // misc
    return b;
}

__device__ inline TileSmem carve(uint8_t* base, uint32_t Lmax) {
    TileSmem s;
    const uint32_t span = Lmax + 64 + kLead + 64;
    uint8_t* p = base;
    s.bytes32 = reinterpret_cast<uint32_t*>(p); p += align_up(span + 64 + 16, 16);
    s.ranks = reinterpret_cast<uint16_t*>(p); p += align_up(padded_len(span) * 2, 16);
    uint8_t* u = p;
    s.hist = u;
    s.fres = reinterpret_cast<uint16_t*>(u); u += align_up(padded_len(Lmax + 64 + kLead) * 2, 16);
    s.score32 = reinterpret_cast<uint32_t*>(u); u += align_up(Lmax + 16, 16);
    s.list = reinterpret_cast<uint32_t*>(u); u += align_up(((Lmax + 64) / 15 + 8) * 4, 16);
    s.sig = reinterpret_cast<uint64_t*>(u); u += kSegs * 8;
    s.tau = reinterpret_cast<uint64_t*>(u); u += kSegs * 8;
    s.own = reinterpret_cast<uint32_t*>(p + own_offset(Lmax));
    p += union_bytes(Lmax);
    s.misc = reinterpret_cast<uint32_t*>(p);
    return s;
}

// Layout of a stream tile whose ranks come precomputed (k_stream_ranks):
// ranks | fres (the compaction list reuses it) | scores | sig | tau | misc.
// No bytes or histograms: 42.9 KB, so five tiles fit on an SM.
__host__ __device__ inline uint32_t fres_bytes(uint32_t Lmax) { return align_up(padded_len(Lmax + 64 + kLead) * 2, 16); }
__host__ __device__ inline uint32_t tile_smem_bytes_pre(uint32_t Lmax) {
    const uint32_t span = Lmax + 64 + kLead + 64;
    return align_up(padded_len(span) * 2, 16) + fres_bytes(Lmax) + align_up(Lmax + 16, 16) + 2 * kSegs * 8 + 64 * 4;
}
__device__ inline TileSmem carve_pre(uint8_t* base, uint32_t Lmax) {
    TileSmem s;
    const uint32_t span = Lmax + 64 + kLead + 64;
    uint8_t* p = base;
    s.bytes32 = nullptr;
    s.hist = nullptr;
    s.own = nullptr;
    s.ranks = reinterpret_cast<uint16_t*>(p); p += align_up(padded_len(span) * 2, 16);
    s.fres = reinterpret_cast<uint16_t*>(p);
    s.list = reinterpret_cast<uint32_t*>(p); p += fres_bytes(Lmax);
    s.score32 = reinterpret_cast<uint32_t*>(p); p += align_up(Lmax + 16, 16);
    s.sig = reinterpret_cast<uint64_t*>(p); p += kSegs * 8;
    s.tau = reinterpret_cast<uint64_t*>(p); p += kSegs * 8;
    s.misc = reinterpret_cast<uint32_t*>(p);
    return s;
}
static_assert(((kTileL + 64) / 15 + 8) * 4 <= (kTileL + 64 + kLead) * 2, "the list fits in the fres area");

// Ranks [Q0, RE) of a tile from the chunk's precomputed ranks (src = the
// chunk's first rank, 16-byte aligned; Q0 is a multiple of 64, and the
// chunk's ranks extend to a multiple of 8), eight per 16-byte load.
__device__ inline void load_ranks(const uint16_t* __restrict__ src, const TileGeom& g, uint16_t* dst) {
    const uint32_t n8 = (g.RE - g.Q0 + 7) / 8;
    const uint4* s4 = reinterpret_cast<const uint4*>(src + g.Q0);
#pragma unroll 4
    for (uint32_t i = threadIdx.x; i < n8; i += blockDim.x) {
        const uint4 v = __ldg(s4 + i);
        uint32_t* d = reinterpret_cast<uint32_t*>(dst + pidx(8 * i));
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
        d[3] = v.w;
    }
}

// ------------------------------------------------------- phase 1: bytes
__device__ inline void load_bytes(const uint8_t* __restrict__ chunk, const TileGeom& g, uint32_t* dst32) {
    // [Q0, BE) -> dst; Q0 is a multiple of 64 relative to the chunk start and
    // chunks start 16-byte aligned, so the bulk moves as 16-byte vectors.
    const uint32_t nbytes = g.BE - g.Q0;
    const uint8_t* src = chunk + g.Q0;
    // dd blocks of a size that is not a multiple of 16 start unaligned
    const uint32_t nvec = ((reinterpret_cast<uintptr_t>(src) & 15) == 0) ? nbytes / 16 : 0;
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst32);
    for (uint32_t i = threadIdx.x; i < nvec; i += blockDim.x) d4[i] = __ldg(s4 + i);
    uint8_t* d8 = reinterpret_cast<uint8_t*>(dst32);
    for (uint32_t i = nvec * 16 + threadIdx.x; i < nbytes + 8; i += blockDim.x)
        d8[i] = (i < nbytes) ? src[i] : 0;
}

// ------------------------------------------------------- phase 2: ranks
// dtab[c] = T[c+1] - T[c] (c = 0..63): entropy change when a byte value's
// count in the window goes from c to c+1 (entr64_inc_int, entr64.cc:47-71,
// written as differences of the table of entr64_table_init_int); dtab[64]
// = 0 pads the table for the branch-free step pair.
//
// Each of kRankThreads threads owns a run of positions starting at a
// multiple of 8 and keeps the byte counts of its window in its own
// histogram.  The counts are the only thing carried from step to step, so
// everything else is moved out of that chain: bytes are read as words a
// group ahead, two steps share one round of count loads (the second step's
// counts corrected for the first step in registers), and the eight ranks of
// a group are stored together as four words.
__device__ __forceinline__ uint32_t byte_of(uint32_t w, uint32_t k) { return __byte_perm(w, 0, 0x4440u | k); }

// Two window steps: bytes a0, a1 leave, b0, b1 enter; e0 / e1 receive the
// entropy after each step.
__device__ __forceinline__ void rank_pair(uint8_t* h, uint32_t hbase, const int32_t* dtab, int32_t& e, uint32_t a0,
                                          uint32_t b0, uint32_t a1, uint32_t b1, int32_t& e0, int32_t& e1) {
    const uint32_t ha0 = hbase + ((a0 >> 2) << 7) + (a0 & 3), hb0 = hbase + ((b0 >> 2) << 7) + (b0 & 3);
    const uint32_t ha1 = hbase + ((a1 >> 2) << 7) + (a1 & 3), hb1 = hbase + ((b1 >> 2) << 7) + (b1 & 3);
    const int32_t ca0 = h[ha0], cb0 = h[hb0];
    int32_t ca1 = h[ha1], cb1 = h[hb1];
    // no branches: when a step's leaving and entering bytes are equal, its
    // two counters are one, the stores below write that count back
    // unchanged, its entropy change is dropped, and the second step's
    // corrections are 0 (dtab has a 0 at index 64 for a count of 64 there)
    const int32_t d0 = (int32_t)(a0 != b0), d1 = (int32_t)(a1 != b1);
    const int32_t x0 = dtab[cb0] - dtab[ca0 - 1];
    ca1 += (int32_t)(a1 == b0) - (int32_t)(a1 == a0);
    cb1 += (int32_t)(b1 == b0) - (int32_t)(b1 == a0);
    e += d0 ? x0 : 0;
    e0 = e;
    const int32_t x1 = dtab[cb1] - dtab[ca1 - 1];
    e += d1 ? x1 : 0;
    e1 = e;
    h[ha0] = (uint8_t)(ca0 - d0);
    h[hb0] = (uint8_t)(cb0 + d0);
    h[ha1] = (uint8_t)(ca1 - d1);
    h[hb1] = (uint8_t)(cb1 + d1);
}

// One window step: byte a leaves, byte b enters.
__device__ __forceinline__ void rank_single(uint8_t* h, uint32_t hbase, const int32_t* dtab, int32_t& e, uint32_t a,
                                            uint32_t b) {
    if (a != b) {
        const uint32_t ha = hbase + ((a >> 2) << 7) + (a & 3);
        const uint32_t hb = hbase + ((b >> 2) << 7) + (b & 3);
        const uint32_t ca = h[ha], cb = h[hb];
        h[ha] = (uint8_t)(ca - 1);
        h[hb] = (uint8_t)(cb + 1);
        e += dtab[cb] - dtab[ca - 1];
    }
}

// Where a run of ranks goes: the tile's padded shared-memory array, or a
// chunk's ranks in global memory (a group of eight as one 16-byte store).
struct SmemRanks {
    uint16_t* r;
    __device__ __forceinline__ void one(uint32_t o, uint16_t v) const { r[pidx(o)] = v; }
    __device__ __forceinline__ void eight(uint32_t o, const uint32_t (&w)[4]) const {
        uint32_t* p = reinterpret_cast<uint32_t*>(r + pidx(o));
#pragma unroll
        for (int k = 0; k < 4; k++) p[k] = w[k];
    }
};
struct GlobalRanks {
    uint16_t* r;  // 16-byte aligned
    __device__ __forceinline__ void one(uint32_t o, uint16_t v) const { r[o] = v; }
    __device__ __forceinline__ void eight(uint32_t o, const uint32_t (&w)[4]) const {
        *reinterpret_cast<uint4*>(r + o) = make_uint4(w[0], w[1], w[2], w[3]);
    }
};

// Ranks of positions [lo, hi) of the bytes at b32 (lo a multiple of 8):
// entropy ranks for [lo, vend), 0 for [vend, hi).  Bytes up to vend+62
// must be present, plus 8 bytes of padding; h + hbase is the thread's
// cleared histogram (hist_off layout).
template <class Out>
__device__ __forceinline__ void rank_run(const uint32_t* b32, uint8_t* h, uint32_t hbase, const uint16_t* rank_tab,
                                         const int32_t* dtab, uint32_t lo, uint32_t vend, uint32_t hi,
                                         const Out& out) {
    const uint8_t* b8 = reinterpret_cast<const uint8_t*>(b32);
    int32_t e = 0;
    uint32_t r = lo;
    if (r < vend) {
        // entr64_init_int (entr64.cc:27-41) built incrementally, two bytes
        // per round of count loads; lo is a multiple of 8, so the window's 64
        // bytes are 16 aligned words, read four at a time
#pragma unroll 1
        for (int q = 0; q < 16; q += 4) {
            uint32_t w[4];
#pragma unroll
            for (int k = 0; k < 4; k++) w[k] = b32[(lo >> 2) + q + k];
#pragma unroll
            for (int k = 0; k < 16; k += 2) {
                const uint32_t v0 = byte_of(w[k >> 2], k & 3), v1 = byte_of(w[k >> 2], (k & 3) + 1);
                const uint32_t o0 = hbase + ((v0 >> 2) << 7) + (v0 & 3), o1 = hbase + ((v1 >> 2) << 7) + (v1 & 3);
                const int32_t c0 = h[o0];
                const int32_t c1 = h[o1] + (int32_t)(v0 == v1);
                e += dtab[c0] + dtab[c1];
                h[o0] = (uint8_t)(c0 + 1);
                h[o1] = (uint8_t)(c1 + 1);  // the same counter when v0 == v1: this store wins
            }
        }
        out.one(r, rank_tab[e >> 10]);
        r++;
    }
    // single steps up to the next multiple of 8
    for (; r < vend && (r & 7u); r++) {
        rank_single(h, hbase, dtab, e, b8[r - 1], b8[r + 63]);
        out.one(r, rank_tab[e >> 10]);
    }
    // groups of eight: leaving bytes r-1..r+6, entering r+63..r+70 (three
    // aligned words each, the next group's words loaded ahead)
    if (r + 8 <= vend) {
        uint32_t lw0 = b32[(r - 4) >> 2], lw1 = b32[r >> 2], lw2 = b32[(r + 4) >> 2];
        uint32_t ew0 = b32[(r + 60) >> 2], ew1 = b32[(r + 64) >> 2], ew2 = b32[(r + 68) >> 2];
        for (; r + 8 <= vend; r += 8) {
            uint32_t nl0 = 0, nl1 = 0, nl2 = 0, ne0 = 0, ne1 = 0, ne2 = 0;
            if (r + 16 <= vend) {
                nl0 = b32[(r + 4) >> 2];
                nl1 = b32[(r + 8) >> 2];
                nl2 = b32[(r + 12) >> 2];
                ne0 = b32[(r + 68) >> 2];
                ne1 = b32[(r + 72) >> 2];
                ne2 = b32[(r + 76) >> 2];
            }
            uint32_t a[8], b[8];
            a[0] = byte_of(lw0, 3);
            b[0] = byte_of(ew0, 3);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                a[1 + k] = byte_of(lw1, k);
                b[1 + k] = byte_of(ew1, k);
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                a[5 + k] = byte_of(lw2, k);
                b[5 + k] = byte_of(ew2, k);
            }
            int32_t ev[8];
#pragma unroll
            for (int k = 0; k < 8; k += 2) rank_pair(h, hbase, dtab, e, a[k], b[k], a[k + 1], b[k + 1], ev[k], ev[k + 1]);
            uint32_t rk[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
                rk[k] = (uint32_t)rank_tab[ev[2 * k] >> 10] | ((uint32_t)rank_tab[ev[2 * k + 1] >> 10] << 16);
            out.eight(r, rk);
            lw0 = nl0;
            lw1 = nl1;
            lw2 = nl2;
            ew0 = ne0;
            ew1 = ne1;
            ew2 = ne2;
        }
    }
    for (; r < vend; r++) {
        rank_single(h, hbase, dtab, e, b8[r - 1], b8[r + 63]);  // byte r-1 leaves, byte r+63 enters
        out.one(r, rank_tab[e >> 10]);
    }
    for (; r < hi; r++) out.one(r, 0);  // the last 64 positions of a chunk
}

__device__ inline void compute_ranks(const TileGeom& g, const TileSmem& s, const uint16_t* rank_tab,
                                     const int32_t* dtab) {
    const uint32_t np = g.RE - g.Q0;
    const uint32_t per = ((np + kRankThreads - 1) / kRankThreads + 7) & ~7u;
    const uint32_t tid = threadIdx.x;
    if (tid >= (uint32_t)kRankThreads) return;
    const uint32_t lo = min(np, tid * per), hi = min(np, lo + per);
    const uint32_t last = g.n - kWin;  // ranks exist for o < n-64 only
    const uint32_t vend = last > g.Q0 ? min(hi, last - g.Q0) : lo;  // [lo, vend): entropy ranks
    rank_run(s.bytes32, s.hist, hist_off(tid, 0), rank_tab, dtab, lo, vend, hi, SmemRanks{s.ranks});
}

// ------------------------------------- phase 3: full-rescan result per step
// For step k with rank[k] > 0 the full rescan of gen_chunk_scores picks the
// smallest non-zero rank m of window [k, k+63], at its leftmost position f,
// extended right over the run of equal ranks (capped at k+63).  Stored as
// (m << 6) | (p - k); 0 when rank[k] == 0 (no credit, next step rescans).
//
// One thread per aligned 64-step block A (steps base..base+63); the window
// of step base+u is A[u..63] followed by B[0..u-1], B the next block.
//  pass 1, u = 63..0: the leftmost minimum of A[u..63] and the end of its
//    run inside A, as a running state -- a rank equal to the minimum
//    becomes the new leftmost one, keeping the run end only when its right
//    neighbour continues the run.  Written to fres[base+u] (0 when
//    rank[base+u] == 0).
//  pass 2, v = 0..62: the same state for the prefix B[0..v] (a run end
//    advances only while the run is contiguous) and the end of B's leading
//    run; step u = v+1 takes A's minimum on ties (leftmost), continuing its
//    run into B when it reaches A's last position and B starts with the
//    same rank.  Both run ends stay within the window, so no cap is needed.
// Positions past the tile's last step are read but only feed steps that no
// walk uses (every array extends past them).
//
// Both passes move eight steps at a time: the next group's ranks (two per
// 32-bit word; pidx keeps a block contiguous and 4-byte aligned) are loaded
// before the current group's results are stored, so no load waits behind a
// store.
__device__ inline void compute_fres(const TileGeom& g, const TileSmem& s) {
    const uint32_t nsteps = g.SE - g.Q0;
    const uint32_t nblk = (nsteps + 63) / 64;
    for (uint32_t j = threadIdx.x; j < nblk; j += blockDim.x) {
        const uint32_t base = j * 64;
        const uint32_t* __restrict__ Ra = reinterpret_cast<const uint32_t*>(s.ranks + pidx(base));
        const uint32_t* __restrict__ Rb = reinterpret_cast<const uint32_t*>(s.ranks + pidx(base + 64));
        uint32_t* __restrict__ Fa = reinterpret_cast<uint32_t*>(s.fres + pidx(base));
        // pass 1: suffix states of A, steps 63..0
        uint32_t m = 1023, e = 63, rn = 0;
        uint32_t cur[4], nxt[4] = {0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < 4; q++) cur[q] = Ra[28 + q];
        uint32_t first = 0;  // result of step 0 (final after pass 1)
        uint32_t any = 0;    // OR of block A's ranks
#pragma unroll 1
        for (int gi = 7; gi >= 0; gi--) {
            any |= cur[0] | cur[1] | cur[2] | cur[3];
            if (gi > 0) {
#pragma unroll
                for (int q = 0; q < 4; q++) nxt[q] = Ra[4 * (gi - 1) + q];
            }
            uint32_t out[4];
#pragma unroll
            for (int q = 3; q >= 0; q--) {
                uint32_t o2 = 0;
#pragma unroll
                for (int h = 1; h >= 0; h--) {
                    const uint32_t u = 8u * gi + 2 * q + h;
                    const uint32_t r = h ? (cur[q] >> 16) : (cur[q] & 0xFFFFu);
                    // r != 0 and (r < m, or r == m after a run break), as one
                    // unsigned compare (m >= 1): r - 1 < m - (rn == m)
                    const bool take = (r - 1u) < (m - (uint32_t)(rn == m));
                    m = take ? r : m;
                    e = take ? u : e;
                    rn = r;
                    o2 |= (r == 0 ? 0u : ((m << 6) | e)) << (16 * h);
                }
                out[q] = o2;
            }
            first = out[0] & 0xFFFFu;
#pragma unroll
            for (int q = 0; q < 4; q++) Fa[4 * gi + q] = out[q];
#pragma unroll
            for (int q = 0; q < 4; q++) cur[q] = nxt[q];
        }
        // a block whose ranks are all 0 (low-entropy content) is done: every
        // step's result is 0, as pass 1 wrote
        if (any == 0) continue;
        // pass 2: prefix states of B, steps u = v + 1 = 1..63; results are
        // packed into aligned words with the previous group's last one
        uint32_t rb[4], fa[5], nrb[4] = {0, 0, 0, 0}, nfa[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < 4; q++) rb[q] = Rb[q];
#pragma unroll
        for (int q = 0; q < 5; q++) fa[q] = Fa[q];
        const uint32_t rb0 = rb[0] & 0xFFFFu;
        // A's leftmost minimum whose run reaches A's last position has A's
        // last rank, so it continues into B iff B starts with that rank
        const uint32_t r63 = Ra[31] >> 16;
        const bool contB = r63 != 0 && r63 == rb0;
        // pm / pe64: minimum of B[0..v] and 64 + the end of its leftmost run;
        // open: that run ends at v; lead64: 64 + the end of B's leading run
        uint32_t pm = 1023, pe64 = 64, lead64 = 64;
        bool open = false, lead_open = true;
        uint32_t carry = first;
#pragma unroll 1
        for (uint32_t gi = 0; gi < 8; gi++) {
            if (gi < 7) {
#pragma unroll
                for (int q = 0; q < 4; q++) nrb[q] = Rb[4 * (gi + 1) + q];
#pragma unroll
                for (int q = 0; q < 4; q++) nfa[q] = Fa[4 * (gi + 1) + q];
                nfa[4] = gi < 6 ? Fa[4 * (gi + 1) + 4] : 0u;
            }
            uint32_t res[8];
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const uint32_t v = 8 * gi + t;
                const uint32_t r = (t & 1) ? (rb[t >> 1] >> 16) : (rb[t >> 1] & 0xFFFFu);
                lead_open = lead_open && r == rb0;
                lead64 = lead_open ? 64 + v : lead64;
                const bool lower = (r - 1u) < (pm - 1u);  // r != 0 && r < pm (pm >= 1)
                const bool cont = open && r == pm;  // pm > 0, so r != 0
                pm = lower ? r : pm;
                open = lower || cont;
                pe64 = open ? 64 + v : pe64;
                const uint32_t u = v + 1;  // its suffix state is halfword t + 1 of fa
                const uint32_t sv = ((t + 1) & 1) ? (fa[(t + 1) >> 1] >> 16) : (fa[(t + 1) >> 1] & 0xFFFFu);
                const uint32_t sm = sv >> 6, se = sv & 63;
                const bool a_wins = sm <= pm;
                const uint32_t mm = a_wins ? sm : pm;
                const uint32_t p = a_wins ? ((se == 63 && contB) ? lead64 : se) : pe64;
                res[t] = sv == 0 ? 0u : ((mm << 6) | (p - u));
            }
            // steps 8gi .. 8gi+7 as words 4gi .. 4gi+3 (step 8gi from the carry)
            Fa[4 * gi] = carry | (res[0] << 16);
            Fa[4 * gi + 1] = res[1] | (res[2] << 16);
            Fa[4 * gi + 2] = res[3] | (res[4] << 16);
            Fa[4 * gi + 3] = res[5] | (res[6] << 16);
            carry = res[7];  // step 8gi + 8 (the next block's step 0 when gi == 7: dropped)
#pragma unroll
            for (int q = 0; q < 4; q++) rb[q] = nrb[q];
#pragma unroll
            for (int q = 0; q < 5; q++) fa[q] = nfa[q];
        }
    }
}

// ------------------------------------------------------ phase 4: chains
// Run-length credit accumulator: a cheap slide credits the same position
// many times in a row, so credits are added to the shared score array only
// when the credited position changes.
template <int kSign>
struct Credit {
    uint32_t* score32;
    uint32_t lo, hi;      // credited positions [lo, hi) (chunk-relative)
    uint32_t cur, start;  // position credited by the open run of steps (~0u: none) and its first step
    // closes the open run at step i (its steps [start, i) all credited cur)
    __device__ __forceinline__ void flush(uint32_t i) {
        const uint32_t o = cur - lo;
        if (o < hi - lo && i > start) {
            const uint32_t inc = (i - start) << (8 * (o & 3));
            if (kSign > 0) atomicAdd(&score32[o >> 2], inc);
            else atomicSub(&score32[o >> 2], inc);
        }
    }
    // step i credits p when act (its min rank is not 0); a step that
    // credits nothing opens a run of ~0u, which is never added
    // (the open run is closed inline: one predicate for "changed and in range")
    __device__ __forceinline__ void add(uint32_t i, uint32_t p, bool act) {
        const uint32_t key = act ? p : ~0u;
        const bool chg = key != cur;
        const uint32_t o = cur - lo;
        if (chg && o < hi - lo) {
            const uint32_t inc = (i - start) << (8 * (o & 3));
            if (kSign > 0) atomicAdd(&score32[o >> 2], inc);
            else atomicSub(&score32[o >> 2], inc);
        }
        cur = chg ? key : cur;
        start = chg ? i : start;
    }
};

// One step of gen_chunk_scores (sdbf_core.cc:59-80) from state st, given
// rank[i+64] and the full-rescan result of step i.
template <typename CR>
__device__ __forceinline__ void walk_step(ChainState& st, uint32_t i, uint32_t r64, uint32_t f, CR* cr) {
    const bool cheap = (st.M != 0) & (r64 >= st.M) & (i < st.P);
    const uint32_t cheapP = (r64 == st.M) ? i + 64 : st.P;
    st.P = cheap ? cheapP : i + (f & 63);
    st.M = cheap ? st.M : (f >> 6);
    if (cr) cr->add(i, st.P, st.M != 0);
}

// Eight consecutive 16-bit entries starting at an 8-aligned index (inside
// one 64-block of the padded layout, 4-byte aligned) as four words.
__device__ __forceinline__ void load8(const uint16_t* p, uint32_t* w) {
    const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
#pragma unroll
    for (int k = 0; k < 4; k++) w[k] = q[k];
}
__device__ __forceinline__ uint32_t half16(const uint32_t* w, int k) {
    return (k & 1) ? (w[k >> 1] >> 16) : (w[k >> 1] & 0xFFFFu);
}

// Walk steps [a, b) of gen_chunk_scores from state `st` (st.M == 0 makes step
// a a full rescan: the speculative start, or step 0).  Single steps up to an
// 8-aligned step (Q0 is a multiple of 64, so tile offsets are aligned too),
// then groups of eight whose operands (rank[i+64..], fres[i..]) are loaded
// one group ahead.  With rec set, the state entering step chk is stored
// there (the steps before chk then run one at a time).
template <typename CR>
__device__ __forceinline__ ChainState walk(const TileGeom& g, const TileSmem& s, uint32_t a, uint32_t b,
                                           ChainState st, CR* cr, uint32_t chk = 0, uint64_t* rec = nullptr) {
    const uint16_t* __restrict__ R = s.ranks;
    const uint16_t* __restrict__ Fr = s.fres;
    uint32_t i = a;
    if (rec && chk >= a && chk < b) {
        for (; i < chk; i++) walk_step(st, i, R[pidx(i + 64 - g.Q0)], Fr[pidx(i - g.Q0)], cr);
        *rec = pack_state(st);
    }
    for (; i < b && (i & 7u); i++) walk_step(st, i, R[pidx(i + 64 - g.Q0)], Fr[pidx(i - g.Q0)], cr);
    if (i + 8 <= b) {
        uint32_t rw[4], fw[4];
        load8(R + pidx(i + 64 - g.Q0), rw);
        load8(Fr + pidx(i - g.Q0), fw);
        for (; i + 8 <= b; i += 8) {
            uint32_t nrw[4] = {0, 0, 0, 0}, nfw[4] = {0, 0, 0, 0};
            if (i + 16 <= b) {
                load8(R + pidx(i + 72 - g.Q0), nrw);
                load8(Fr + pidx(i + 8 - g.Q0), nfw);
            }
#pragma unroll
            for (int k = 0; k < 8; k++) walk_step(st, i + k, half16(rw, k), half16(fw, k), cr);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                rw[k] = nrw[k];
                fw[k] = nfw[k];
            }
        }
    }
    for (; i < b; i++) walk_step(st, i, R[pidx(i + 64 - g.Q0)], Fr[pidx(i - g.Q0)], cr);
    return st;
}

// Re-walk segment [St, Et) from its true entry state `nw` next to the chain
// it was credited with (`old`, from its speculative entry).  Both walks run
// in lockstep; credits differ only until the two states coincide, after
// which the rest of the old walk (and its exit state) stands.  Returns the
// segment's exit state.
__device__ uint64_t relink_segment(const TileGeom& g, const TileSmem& s, uint32_t St, uint32_t Et, ChainState old,
                                   ChainState nw, uint32_t chk, uint64_t old_exit) {
    Credit<-1> un{s.score32, g.t0, g.t0 + g.L, ~0u, St};
    Credit<1> re{s.score32, g.t0, g.t0 + g.L, ~0u, St};
    uint32_t i = St;
    for (; i < Et; i++) {
        if (pack_state(old) == pack_state(nw)) break;
        if (i == chk) *reinterpret_cast<uint64_t*>(&s.misc[10]) = pack_state(nw);
        const uint32_t r64 = s.ranks[pidx(i + 64 - g.Q0)], f = s.fres[pidx(i - g.Q0)];
        walk_step(old, i, r64, f, &un);
        walk_step(nw, i, r64, f, &re);
    }
    un.flush(i);
    re.flush(i);
    return i < Et ? old_exit : pack_state(nw);
}

__device__ __forceinline__ void stamp(long long* tm, int k) {
    if (tm && threadIdx.x == 0) tm[k] = clock64();
}

// Walk segment [St, Et) from `st` with credits of sign kSign; records the
// state entering step chk (the next tile's first credited step) when the
// segment contains it.
template <int kSign>
__device__ __forceinline__ ChainState walk_segment(const TileGeom& g, const TileSmem& s, uint32_t St, uint32_t Et,
                                                   ChainState st, uint32_t chk) {
    Credit<kSign> cr{s.score32, g.t0, g.t0 + g.L, ~0u, St};
    st = walk(g, s, St, Et, st, &cr, chk, kSign > 0 ? reinterpret_cast<uint64_t*>(&s.misc[10]) : nullptr);
    cr.flush(Et);
    return st;
}

// Runs all phases for one tile.  entry != nullptr: the state entering step
// S0 is known (re-computation after a failed link check); otherwise thread 0
// starts speculatively `lead` steps early.  Writes sig_in / tau_out.
// kPre: the ranks come from pre_ranks (the chunk's precomputed ranks)
// instead of the chunk bytes.
template <bool kPre = false>
__device__ void tile_pipeline(const uint8_t* __restrict__ chunk, const TileGeom& g, const TileSmem& s,
                              const uint16_t* rank_tab, const int32_t* dtab, const uint64_t* entry,
                              uint64_t* sig_in, uint64_t* tau_out, uint32_t lead, long long* tm,
                              const uint16_t* pre_ranks = nullptr) {
    stamp(tm, 0);
    if constexpr (kPre) {
        load_ranks(pre_ranks, g, s.ranks);
        __syncthreads();
        stamp(tm, 1);
    } else {
        load_bytes(chunk, g, s.bytes32);
        {
            uint4* h4 = reinterpret_cast<uint4*>(s.hist);
            for (uint32_t i = threadIdx.x; i < 256 * kRankThreads / 16; i += blockDim.x)
                h4[i] = make_uint4(0, 0, 0, 0);
        }
        __syncthreads();
        stamp(tm, 1);
        compute_ranks(g, s, rank_tab, dtab);
        __syncthreads();
    }
    stamp(tm, 2);
    compute_fres(g, s);
    // clear scores (in-tile ranks: aliases the histogram area, free after phase 2)
    for (uint32_t i = threadIdx.x; i < (g.L + 3) / 4 + 1; i += blockDim.x) s.score32[i] = 0;
    if (threadIdx.x == 0) {
        s.misc[9] = 0;
        s.misc[10] = 0;
        s.misc[11] = 0;
    }
    __syncthreads();
    stamp(tm, 3);
    // segments over steps [S0, SE)
    const uint32_t total = g.SE > g.S0 ? g.SE - g.S0 : 0;
    // segment length a multiple of 8 (S0 is a multiple of 64): every walk then
    // starts and ends on a group of eight steps (trailing threads may idle)
    const uint32_t SL = ((total + kSegs - 1) / kSegs + 7) & ~7u;
    const uint32_t chk = g.t0 + g.L - 64;  // next tile's S0
    const uint32_t t = threadIdx.x;
    const uint32_t St = g.S0 + t * SL;
    const uint32_t Et = min(St + SL, g.SE);
    const bool has_seg = t < kSegs && SL > 0 && St < g.SE;
    if (t < kSegs) {
        if (has_seg) {
            ChainState st{0, 0};
            if (t == 0 && entry) {
                st = unpack_state(*entry);
            } else {
                // lead-in (never below Q0, since every lead <= kLead); a lead-in
                // from step 0 makes the walk exact.  The tile's first segment
                // has the same lead as the others (a longer one would hold up
                // its warp): its rare mis-speculation costs a tile recompute
                // in k_stream_fix.
                const uint32_t Ls = St > lead ? St - lead : 0;
                st = walk(g, s, Ls, St, st, (Credit<1>*)nullptr);
            }
            s.sig[t] = pack_state(st);
            s.tau[t] = pack_state(walk_segment<1>(g, s, St, Et, st, chk));
        } else {
            s.sig[t] = ~0ull;
            s.tau[t] = ~0ull;
        }
    }
    __syncthreads();
    stamp(tm, 4);
    // phase 5: link segments.  A segment is exact iff its entry state equals
    // its left neighbour's exit state; mismatched segments are re-walked in
    // parallel rounds until every link holds (normally zero rounds).
    while (true) {
        bool need = false;
        uint64_t from = 0;
        if (has_seg && t >= 1) {
            from = s.tau[t - 1];
            need = s.sig[t] != from;
        }
        if (!__syncthreads_or(need)) break;
        if (need) {
            const uint64_t out = relink_segment(g, s, St, Et, unpack_state(s.sig[t]), unpack_state(from), chk,
                                                s.tau[t]);
            s.sig[t] = from;
            s.tau[t] = out;
            atomicAdd(&s.misc[9], 1u);
        }
        __syncthreads();
    }
    if (t == 0) {
        if (sig_in) *sig_in = s.sig[0];
        if (tau_out) *tau_out = *reinterpret_cast<uint64_t*>(&s.misc[10]);
    }
    __syncthreads();
    stamp(tm, 5);
}

// ------------------------------------------- phase 6: ordered compaction
// Writes the positions (relative to t0) with score > thr (or >= thr when
// ge) among [t0, t0+nown) into s.list in ascending order; returns count.
// Each warp owns a contiguous run of score words; lanes read consecutive
// 32-bit words (4 positions each), so the reads are conflict-free.  A
// position's place in the list comes from four ballots (one per byte of
// the word): the selected positions of earlier lanes, plus those earlier in
// the lane's own word.
__device__ __forceinline__ uint32_t word_flags(const uint32_t* sc32, uint32_t wd, uint32_t nown, uint32_t thr,
                                               bool ge) {
    const uint32_t w = sc32[wd];
    // per byte: bit 7 set when selected (bytes are scores <= 65 and the
    // threshold byte is <= 66, so no byte borrows from its neighbour)
    const uint32_t t4 = (ge ? thr : thr + 1) * 0x01010101u;
    const uint32_t hb = ((w | 0x80808080u) - t4) & 0x80808080u;
    uint32_t f = (hb >> 7 | hb >> 14 | hb >> 21 | hb >> 28) & 0xFu;
    const uint32_t p0 = 4 * wd;
    if (p0 + 4 > nown) f &= (p0 >= nown) ? 0u : ((1u << (nown - p0)) - 1u);
    return f;
}

__device__ uint32_t compact(const TileSmem& s, uint32_t nown, uint32_t thr, bool ge, uint32_t* tmp_counts) {
    const uint32_t nwords = (nown + 3) / 4;
    const uint32_t nwarps = blockDim.x / 32, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t per = ((nwords + nwarps - 1) / nwarps + 31) / 32 * 32;
    const uint32_t w0 = min(nwords, wid * per), w1 = min(nwords, w0 + per);
    uint32_t c = 0;
    for (uint32_t wd = w0 + lane; wd < w1; wd += 32) c += __popc(word_flags(s.score32, wd, nown, thr, ge));
    c = __reduce_add_sync(0xffffffffu, c);
    if (lane == 0) tmp_counts[wid] = c;
    __syncthreads();
    uint32_t base = 0, total = 0;
    for (uint32_t w = 0; w < nwarps; w++) {
        if (w < wid) base += tmp_counts[w];
        total += tmp_counts[w];
    }
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t wd0 = w0; wd0 < w1; wd0 += 32) {
        const uint32_t wd = wd0 + lane;
        const uint32_t f = wd < w1 ? word_flags(s.score32, wd, nown, thr, ge) : 0u;
        const uint32_t m0 = __ballot_sync(0xffffffffu, f & 1u), m1 = __ballot_sync(0xffffffffu, f & 2u);
        const uint32_t m2 = __ballot_sync(0xffffffffu, f & 4u), m3 = __ballot_sync(0xffffffffu, f & 8u);
        uint32_t pos = base + __popc(m0 & lt) + __popc(m1 & lt) + __popc(m2 & lt) + __popc(m3 & lt);
#pragma unroll
        for (int b = 0; b < 4; b++)
            if ((f >> b) & 1u) s.list[pos++] = 4 * wd + b;
        base += __popc(m0) + __popc(m1) + __popc(m2) + __popc(m3);
    }
    __syncthreads();
    return total;
}

// Stream tiles (threshold 16): one pass.  Warp w writes its selected
// positions to its own list s.list[w * kWarpList ..] and their number to
// counts[w]; feature f of the tile is entry f - (the counts of earlier
// warps) of the first warp list that reaches it.  A lane reads 16 scores
// (one 16-byte load; a warp's 32 loads are one contiguous 512-byte run) and
// gets their selection bits from four byte-parallel compares; a shuffle scan
// of the lanes' counts places them.  A warp's range holds at most 2,048
// positions, so at most (2048 + 64) / 17 = 124 of them reach a score of 17
// (each step credits one position in [i, i+64]).
constexpr uint32_t kWarpList = 128;
__device__ __forceinline__ uint32_t sel4(uint32_t w, uint32_t t4) {
    const uint32_t hb = ((w | 0x80808080u) - t4) & 0x80808080u;
    return (hb >> 7 | hb >> 14 | hb >> 21 | hb >> 28) & 0xFu;
}
__device__ void compact_stream(const TileSmem& s, uint32_t nown, uint32_t* counts) {
    const uint32_t nq = (nown + 15) / 16;  // 16-position quads
    const uint32_t nwarps = blockDim.x / 32, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t per = ((nq + nwarps - 1) / nwarps + 31) / 32 * 32;
    const uint32_t q0 = min(nq, wid * per), q1 = min(nq, q0 + per);
    uint32_t* list = s.list + wid * kWarpList;
    const uint4* sc4 = reinterpret_cast<const uint4*>(s.score32);
    const uint32_t t4 = (kThreshold + 1) * 0x01010101u;
    uint32_t n = 0;
    for (uint32_t qb = q0; qb < q1; qb += 32) {
        const uint32_t q = qb + lane;
        uint32_t m = 0;
        if (q < q1) {
            const uint4 w = sc4[q];
            m = sel4(w.x, t4) | (sel4(w.y, t4) << 4) | (sel4(w.z, t4) << 8) | (sel4(w.w, t4) << 12);
            if (16 * q + 16 > nown) m &= (1u << (nown - 16 * q)) - 1u;
        }
        const uint32_t c = __popc(m);
        uint32_t incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        uint32_t pos = n + incl - c;
        while (m) {
            list[pos++] = 16 * q + (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
        }
        n += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) counts[wid] = n;
    __syncthreads();
}

// ---------------------------------------------------------- stream tiles
__device__ inline TileGeom stream_geom(uint32_t n, uint32_t t0) {
    TileGeom g;
    g.n = n;
    g.t0 = t0;
    g.L = kTileL;
    g.S0 = t0 >= 64 ? t0 - 64 : 0;
    const uint32_t last = n - kWin;
    g.SE = min(t0 + kTileL, last);
    g.Q0 = g.S0 > kLead ? g.S0 - kLead : 0;
    g.RE = min(g.SE + 64, n);
    g.BE = min(g.RE + 63, n);
    return g;
}

// kPre: ranks precomputed in P.ranks (tile_smem_bytes_pre layout); the
// SHA-1 phase then reads the feature bytes from global memory.
template <bool kPre>
__device__ void stream_tile_body(const GenParams& P, uint32_t tile, const uint64_t* entry, uint8_t* smem) {
    const GenTile T = P.tiles[tile];
    const GenChunk C = P.chunks[T.chunk];
    const TileGeom g = stream_geom(C.n, T.t0);
    TileSmem s = kPre ? carve_pre(smem, kTileL) : carve(smem, kTileL);
    const uint16_t* rank_tab = nullptr;
    const int32_t* dt = nullptr;
    if constexpr (!kPre) {
        __shared__ int32_t dtab[65];
        for (uint32_t i = threadIdx.x; i < 65; i += blockDim.x)
            dtab[i] = i < 64 ? (int32_t)P.ent_tab[i + 1] - (int32_t)P.ent_tab[i] : 0;
        // the rank table (2 KB) in shared memory: a lookup is one shared-memory read
        __shared__ uint16_t s_rank[(SDBF_RANK_BINS + 7) / 8 * 8];
        for (uint32_t i = threadIdx.x; i < SDBF_RANK_BINS; i += blockDim.x) s_rank[i] = P.rank_tab[i];
        __syncthreads();
        rank_tab = s_rank;
        dt = dtab;
    }
    TileOut* out = P.tile_out + tile;
    long long tm[9];
    const uint8_t* chunk = P.data + C.data_off;
    tile_pipeline<kPre>(chunk, g, s, rank_tab, dt, entry, &out->sig_in, &out->tau_out, P.lead,
                        P.phase ? tm : nullptr, kPre ? P.ranks + (size_t)C.rank_off8 * 8 : nullptr);
    const uint32_t nown = g.SE > g.t0 ? g.SE - g.t0 : 0;
    __shared__ uint32_t counts[kGenThreads / 32];
    static_assert(kGenThreads / 32 == 4 && 4 * kWarpList <= (kTileL + 64) / 15 + 8, "stream list layout");
    compact_stream(s, nown, counts);
    const uint32_t c1 = counts[0], c2 = c1 + counts[1], c3 = c2 + counts[2], nf = c3 + counts[3];
    stamp(P.phase ? tm : nullptr, 6);
    // SHA-1 of each selected feature (sdbf_core.cc:103-105)
    uint32_t* feat = P.features + (size_t)tile * 5 * kTileCap;
    const uint32_t off = g.t0 - g.Q0;
    for (uint32_t f = threadIdx.x; f < nf; f += blockDim.x) {
        const uint32_t wl = (f >= c1) + (f >= c2) + (f >= c3);
        const uint32_t before = wl == 0 ? 0u : wl == 1 ? c1 : wl == 2 ? c2 : c3;
        const uint32_t p = s.list[wl * kWarpList + (f - before)] + off;
        uint32_t w[16], h[5];
        if constexpr (kPre)
            load_be16_global(chunk + g.Q0 + p, w);
        else
            load_be16(s.bytes32, p, w);
        sha1_feature(w, h);
#pragma unroll
        for (int k = 0; k < 5; k++) feat[k * kTileCap + f] = h[k];
    }
    if (threadIdx.x == 0) {
        out->count = nf;
        out->fixups = s.misc[9];
    }
    if (P.phase) {
        __syncthreads();
        stamp(tm, 7);
        if (threadIdx.x == 0) {
            for (int k = 0; k < 7; k++) atomicAdd(P.phase + k, (unsigned long long)(tm[k + 1] - tm[k]));
            atomicAdd(P.phase + kPhTiles, 1ull);
            atomicAdd(P.phase + kPhFixups, (unsigned long long)s.misc[9]);
        }
    }
}

__global__ void __launch_bounds__(kGenThreads, 4) k_stream_tiles(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    for (uint32_t tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
        stream_tile_body<false>(P, tile, nullptr, smem);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kGenThreads, 5) k_stream_tiles_pre(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    for (uint32_t tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
        stream_tile_body<true>(P, tile, nullptr, smem);
        __syncthreads();
    }
}

// Link tiles of a chunk: a tile's speculative entry state must equal its
// predecessor's exit state (tiles whose lead-in reaches step 0 are exact).
// k_stream_check (one warp per chunk, no shared memory) finds the first
// tile of each chunk whose link fails; k_stream_fix (one CTA per chunk,
// normally exiting at once) recomputes that tile from the true entry state
// and moves on through the chunk: its threads check the links of the next
// kGenThreads tiles at once, and the first failing one (a later tile whose
// entry no longer matches, or an unrelated mis-speculation) is recomputed
// next.
__device__ __forceinline__ bool link_fails(const GenParams& P, const GenChunk& C, uint32_t tile) {
    const TileGeom g = stream_geom(C.n, P.tiles[tile].t0);
    return g.S0 > P.lead && P.tile_out[tile - 1].tau_out != P.tile_out[tile].sig_in;
}

__global__ void __launch_bounds__(128) k_stream_check(GenParams P) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    for (uint32_t c = warp; c < P.nchunks; c += nwarps) {
        const GenChunk C = P.chunks[c];
        uint32_t first = 0xFFFFFFFFu;
        for (uint32_t j0 = 1; j0 < C.ntiles && first == 0xFFFFFFFFu; j0 += 32) {
            const uint32_t j = j0 + lane;
            const bool bad = j < C.ntiles && link_fails(P, C, C.first_tile + j);
            const uint32_t m = __ballot_sync(0xffffffffu, bad);
            if (m) first = j0 + __ffs(m) - 1;
        }
        if (lane == 0) P.chunk_redo[c] = first;
    }
}

// Before k_stream_check / k_stream_fix: every tile whose link fails goes
// to P.fix_list (fix_list[0] = their number, zeroed by the host), and
// k_stream_fix_list recomputes them all at once, one CTA each, from their
// predecessors' exit states as they stand.  A tile whose predecessor is
// recomputed in the same launch may start from the stale state; the
// serial pass that follows finds and redoes it (normally nothing is left).
__global__ void __launch_bounds__(256) k_stream_fails(GenParams P) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < P.ntiles; t += gridDim.x * blockDim.x) {
        const GenChunk C = P.chunks[P.tiles[t].chunk];
        if (t > C.first_tile && link_fails(P, C, t)) P.fix_list[1 + atomicAdd(P.fix_list, 1u)] = t;
    }
}

template <bool kPre>
__global__ void __launch_bounds__(kGenThreads) k_stream_fix_list(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ uint64_t entry;
    const uint32_t n = P.fix_list[0];
    for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
        const uint32_t tile = P.fix_list[1 + k];
        if (threadIdx.x == 0) entry = P.tile_out[tile - 1].tau_out;
        __syncthreads();
        stream_tile_body<kPre>(P, tile, &entry, smem);
        if (threadIdx.x == 0) atomicAdd(P.counters + 0, 1u);
        __syncthreads();
    }
}

template <bool kPre>
__global__ void __launch_bounds__(kGenThreads) k_stream_fix(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ uint64_t entry;
    __shared__ uint32_t bad_first;
    for (uint32_t c = blockIdx.x; c < P.nchunks; c += gridDim.x) {
        const uint32_t first = P.chunk_redo[c];
        if (first == 0xFFFFFFFFu) continue;
        const GenChunk C = P.chunks[c];
        uint32_t j = first;
        while (j < C.ntiles) {
            // the first failing link among tiles [j, j + blockDim.x); tiles
            // recomputed before it are visible here (same CTA, after a barrier)
            if (threadIdx.x == 0) bad_first = 0xFFFFFFFFu;
            __syncthreads();
            const uint32_t jj = j + threadIdx.x;
            if (jj < C.ntiles && link_fails(P, C, C.first_tile + jj)) atomicMin(&bad_first, jj);
            __syncthreads();
            const uint32_t f = bad_first;
            if (f == 0xFFFFFFFFu) {
                j += blockDim.x;
                continue;
            }
            const uint32_t tile = C.first_tile + f;
            if (threadIdx.x == 0) entry = P.tile_out[tile - 1].tau_out;
            __syncthreads();
            stream_tile_body<kPre>(P, tile, &entry, smem);
            if (threadIdx.x == 0) atomicAdd(P.counters + 0, 1u);
            __syncthreads();
            j = f + 1;
        }
    }
}

// ------------------------------------------------------ async copies
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }
// The L2 prefetch of [gmem, gmem+bytes) (16-byte aligned, a multiple of 16 bytes).
__device__ __forceinline__ void prefetch_l2(const void* gmem, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(gmem), "r"(bytes) : "memory");
}

// ------------------------------------------------ precomputed ranks
// Entropy ranks of a stream launch group ahead of its tile kernel.  One CTA
// item is a stretch of kRkSpan positions of a chunk, its bytes staged in
// shared memory by 16-byte asynchronous copies (the CTA's next stretch
// prefetched into L2 meanwhile); each thread ranks kRkPer consecutive
// positions with its own histogram (rank_run, the tile kernel's rank loop),
// so a thread's 64-byte window set-up is spread over 312 positions instead
// of a tile thread's 88.  Ranks of positions >= n-64 are 0; the chunk's
// ranks run to a multiple of 8 (GenChunk::rank_off8).
constexpr uint32_t kRkBytes = align_up(kRkSpan + 64 + 16, 16);  // staged bytes + zero padding
constexpr uint32_t kRkSmem = 256 * kRkThreads + kRkBytes;

__global__ void __launch_bounds__(kRkThreads, 3) k_stream_ranks(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint8_t* hist = smem;
    uint32_t* b32 = reinterpret_cast<uint32_t*>(smem + 256 * kRkThreads);
    __shared__ int32_t dtab[65];
    __shared__ uint16_t s_rank[(SDBF_RANK_BINS + 7) / 8 * 8];
    for (uint32_t i = threadIdx.x; i < 65; i += blockDim.x) dtab[i] = i < 64 ? (int32_t)P.ent_tab[i + 1] - (int32_t)P.ent_tab[i] : 0;
    for (uint32_t i = threadIdx.x; i < SDBF_RANK_BINS; i += blockDim.x) s_rank[i] = P.rank_tab[i];
    const uint32_t tid = threadIdx.x;
    for (uint32_t item = blockIdx.x; item < P.nrk_items; item += gridDim.x) {
        const uint2 it = P.rk_items[item];
        const GenChunk C = P.chunks[it.x];
        const uint32_t s0 = it.y, n = C.n;
        const uint32_t np = min(kRkSpan, align_up(n, 8) - s0);  // positions [s0, s0+np)
        const uint32_t nb = min(kRkSpan + 64, n - s0);          // bytes [s0, s0+nb)
        __syncthreads();  // the previous stretch is done with the bytes and histograms
        // the stretch's bytes: 16-byte asynchronous copies, all in flight at once
        const uint8_t* src = P.data + C.data_off + s0;
        const uint32_t nvec = ((reinterpret_cast<uintptr_t>(src) & 15) == 0) ? nb / 16 : 0;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(b32);
        for (uint32_t i = tid; i < nvec; i += blockDim.x) cp_async16(d4 + i, s4 + i);
        cp_async_commit();
        uint8_t* d8 = reinterpret_cast<uint8_t*>(b32);
        for (uint32_t i = nvec * 16 + tid; i < nb + 8; i += blockDim.x) d8[i] = (i < nb) ? src[i] : 0;
        uint4* h4 = reinterpret_cast<uint4*>(hist);
        for (uint32_t i = tid; i < 256 * kRkThreads / 16; i += blockDim.x) h4[i] = make_uint4(0, 0, 0, 0);
        // the CTA's next stretch into L2 while this one is ranked
        if (tid == 0 && item + gridDim.x < P.nrk_items) {
            const uint2 nx = P.rk_items[item + gridDim.x];
            const GenChunk Cn = P.chunks[nx.x];
            const uint8_t* ns = P.data + Cn.data_off + nx.y;
            const uint32_t nnb = min(kRkSpan + 64, Cn.n - nx.y) & ~15u;
            if ((reinterpret_cast<uintptr_t>(ns) & 15) == 0 && nnb) prefetch_l2(ns, nnb);
        }
        cp_async_wait_all();
        __syncthreads();
        const uint32_t lo = min(np, tid * kRkPer), hi = min(np, lo + kRkPer);
        const uint32_t last = n > kWin ? n - kWin : 0;  // ranks exist for o < n-64 only
        const uint32_t vend = last > s0 ? min(hi, last - s0) : lo;
        rank_run(b32, hist, hist_off(tid, 0), s_rank, dtab, lo, vend, hi,
                 GlobalRanks{P.ranks + (size_t)C.rank_off8 * 8 + s0});
    }
}

// ------------------------------------------------------- ordered commit
// Per-warp shared state for the stream commit.
struct CommitSmem {
    uint32_t F[64];                  // current 256-byte filter
    uint32_t own[2048];              // lanes of the group holding each filter index
    uint32_t G[kBigBytes / 4];       // current 16 KiB big filter
    uint32_t feat[2][5][kTileCap];   // double-buffered features of a tile
};

__device__ inline uint32_t lanemask_le() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_le;" : "=r"(m));
    return m;
}
__device__ inline uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}


// Stage the first `nf` features of a tile (5 rows of kTileCap words) into buf.
__device__ __forceinline__ void stage_tile(uint32_t (*buf)[kTileCap], const uint32_t* feat, uint32_t nf,
                                           uint32_t lane) {
    const uint32_t n4 = (nf + 3) / 4;
    for (uint32_t q = lane; q < 5 * n4; q += 32) {
        const uint32_t k = q / n4, j = q - k * n4;
        cp_async16(&buf[k][4 * j], feat + (size_t)k * kTileCap + 4 * j);
    }
    cp_async_commit();
}

// The ordered filter fill for one group of up to 32 features (lane l holds
// feature l), in feature order, with the semantics of gen_chunk_hash
// (sdbf_core.cc:103-130): a feature is counted iff it sets a new bit in the
// 256-byte filter F (bf_sha1_insert) and a new bit in the big filter G
// (query_and_set); F keeps the bits of features that fail G.
//
// "New" means unset before this feature, i.e. unset in the state before the
// group and not held by an earlier lane of the group.  Earlier holders of a
// filter index come from an owner mask (bit l set for every lane holding the
// 11-bit index).  Two big-filter indices can only be equal if their low 11
// bits -- the filter index -- are, so the same mask names the only lanes
// whose 17-bit values need an exact comparison (register shuffles).  Bits
// are written only for lanes up to the first roll-over, which is found
// before anything is written; later lanes are re-run against the new state.
//
// With an index being built (sdhash --index: sdbf_core.cc:108-114), a
// feature whose filter insert set a new bit is inserted into the index and
// is skipped unless that set a new index bit -- so each file depends on
// every earlier file's features.  Two ways to get that order:
// * kCommitSeq: one warp commits all files in input order, one feature at
//   a time (lane 0), the index in global memory;
// * kCommitRound: one round of a fixed point.  Files commit in parallel; a
//   feature is taken as setting a new index bit iff no feature inserted in
//   the previous round precedes it as the first setter of one of its bits
//   (GenParams::index_pred, one bit per feature, read with the tile), and
//   the inserted features are recorded (GenParams::index_seen).  A file's
//   commit depends only on its own features and their predicate bits, so
//   later rounds re-commit only the files whose bits changed
//   (GenParams::commit_dirty), after clearing their seen bits.  A round that inserts the same features as
//   the previous one reproduces the sequential result: by induction over
//   the input order, every decision then depends only on earlier decisions
//   that already agree.
enum : int { kCommitPlain = 0, kCommitSeq = 1, kCommitRound = 2 };

template <int kMode>
__device__ __forceinline__ void commit_files(const GenParams& P, uint8_t* smem) {
    constexpr bool kIdx = kMode == kCommitSeq;
    const uint32_t wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (kIdx && (blockIdx.x != 0 || wid != 0)) return;
    CommitSmem& S = reinterpret_cast<CommitSmem*>(smem)[wid];
    for (uint32_t i = lane; i < 2048; i += 32) S.own[i] = 0;
    const uint32_t fstep = kIdx ? 1u : gridDim.x * kCommitWarps;
    constexpr uint32_t kGroup = kIdx ? 1u : 32u;
    for (uint32_t fi = kIdx ? 0u : blockIdx.x * kCommitWarps + wid; fi < P.nfiles; fi += fstep) {
        const uint32_t file = P.file_order[fi];
        if (kMode == kCommitRound && P.commit_dirty && !P.commit_dirty[file]) continue;
        const GenFile Fd = P.files[file];
        if (Fd.nchunks == 0) continue;
        uint32_t* out = P.out_filters + (size_t)Fd.filter_base * 64;
        // the file's tiles are one contiguous range
        const GenChunk c0 = P.chunks[Fd.first_chunk];
        const GenChunk cl = P.chunks[Fd.first_chunk + Fd.nchunks - 1];
        const uint32_t t_first = c0.first_tile, t_end = cl.first_tile + cl.ntiles;
        uint32_t chunk = Fd.first_chunk;
        uint32_t next_chunk_tile = (Fd.nchunks > 1) ? P.chunks[chunk + 1].first_tile : 0xFFFFFFFFu;
        uint32_t bf_count = 1, last_count = 0, bigfi = 0;
        // tiles [ts, t_end) commit now: a later index round restarts from the
        // last checkpoint at or before the first changed predicate (nothing
        // before it changed, so the state there is the one recorded)
        uint32_t ts = t_first;
        if (kMode == kCommitRound && P.commit_dirty) {
            const uint32_t from = P.commit_from[file];
            const uint32_t tc = from == 0xFFFFFFFFu ? 0u : from / kTileCap / kCkptTiles * kCkptTiles;
            if (tc > t_first && tc < t_end) ts = tc;
            if (P.phase && lane == 0 && ts > t_first) atomicAdd(P.phase + kPhCkptRestarts, 1ull);
        }
        if (ts > t_first) {
            const uint32_t* ck = P.commit_ckpt + (size_t)(ts / kCkptTiles) * kCkptWords;
            for (uint32_t i = lane; i < 64; i += 32) S.F[i] = ck[i];
            const uint4* g4 = reinterpret_cast<const uint4*>(ck + 64);
            for (uint32_t i = lane; i < kBigBytes / 16; i += 32) reinterpret_cast<uint4*>(S.G)[i] = g4[i];
            bf_count = ck[64 + 4096];
            last_count = ck[64 + 4096 + 1];
            bigfi = ck[64 + 4096 + 2];
            // the chunk holding tile ts - 1, as the loop leaves it
            while (next_chunk_tile < ts) {
                chunk++;
                next_chunk_tile = (chunk + 1 < Fd.first_chunk + Fd.nchunks) ? P.chunks[chunk + 1].first_tile
                                                                             : 0xFFFFFFFFu;
            }
        } else {
            for (uint32_t i = lane; i < 64; i += 32) S.F[i] = 0;
            for (uint32_t i = lane; i < kBigBytes / 4; i += 32) S.G[i] = 0;
        }
        if (kMode == kCommitRound && P.commit_dirty && ts < t_end) {
            // clear the file's seen bits, ordinals [ts, t_end) * kTileCap;
            // inner words are the file's alone, edge words shared with neighbours
            const uint32_t o0 = ts * kTileCap, o1 = t_end * kTileCap - 1;
            for (uint32_t w = (o0 >> 5) + lane; w <= (o1 >> 5); w += 32) {
                const uint32_t lo = w == (o0 >> 5) ? (o0 & 31u) : 0u, hi = w == (o1 >> 5) ? (o1 & 31u) : 31u;
                const uint32_t m = (0xffffffffu >> (31u - hi)) & (0xffffffffu << lo);
                if (m == 0xffffffffu) P.index_seen[w] = 0;
                else atomicAnd(P.index_seen + w, ~m);
            }
            __syncwarp();
        }
        uint32_t nf_cur = ts < t_end ? P.tile_out[ts].count : 0;
        uint32_t nf_next = ts + 1 < t_end ? P.tile_out[ts + 1].count : 0;
        if (ts < t_end) stage_tile(S.feat[0], P.features + (size_t)ts * 5 * kTileCap, nf_cur, lane);
        // kCommitRound: the tile's predicate words (its <= 472 ordinals span
        // at most 16 words), lane q holding word q; the next tile's in flight
        uint32_t pw_cur = 0, pw_next = 0;
        if (kMode == kCommitRound) {
            if (ts < t_end && lane < 16) pw_cur = __ldg(P.index_pred + ((ts * kTileCap) >> 5) + lane);
            if (ts + 1 < t_end && lane < 16) pw_next = __ldg(P.index_pred + (((ts + 1) * kTileCap) >> 5) + lane);
        }
        __syncwarp();
        long long t_file = clock64(), t_wait = 0;
        uint32_t n_groups = 0, n_loops = 0;
        for (uint32_t t = ts; t < t_end; t++) {
            const uint32_t cur = (t - ts) & 1u;
            if (kMode == kCommitRound && t > ts && t % kCkptTiles == 0) {
                // checkpoint of the state entering tile t
                uint32_t* ck = P.commit_ckpt + (size_t)(t / kCkptTiles) * kCkptWords;
                for (uint32_t i = lane; i < 64; i += 32) ck[i] = S.F[i];
                uint4* g4 = reinterpret_cast<uint4*>(ck + 64);
                for (uint32_t i = lane; i < kBigBytes / 16; i += 32) g4[i] = reinterpret_cast<const uint4*>(S.G)[i];
                if (lane == 0) {
                    ck[64 + 4096] = bf_count;
                    ck[64 + 4096 + 1] = last_count;
                    ck[64 + 4096 + 2] = bigfi;
                }
            }
            // chunk boundary: the big-filter counter is local to each chunk
            // (sdbf_core.cc:100); the big filter itself continues
            while (t >= next_chunk_tile) {
                bigfi = 0;
                chunk++;
                next_chunk_tile = (chunk + 1 < Fd.first_chunk + Fd.nchunks) ? P.chunks[chunk + 1].first_tile
                                                                             : 0xFFFFFFFFu;
            }
            const long long w0 = clock64();
            cp_async_wait_all();
            __syncwarp();
            t_wait += clock64() - w0;
            const uint32_t nf = nf_cur;
            if (t + 1 < t_end)
                stage_tile(S.feat[cur ^ 1u], P.features + (size_t)(t + 1) * 5 * kTileCap, nf_next, lane);
            const uint32_t pw = pw_cur;
            if (kMode == kCommitRound) {
                pw_cur = pw_next;
                pw_next = (t + 2 < t_end && lane < 16) ? __ldg(P.index_pred + (((t + 2) * kTileCap) >> 5) + lane) : 0u;
            }
            nf_cur = nf_next;
            nf_next = t + 2 < t_end ? P.tile_out[t + 2].count : 0;
            for (uint32_t g0 = 0; g0 < nf; g0 += kGroup) {
                const uint32_t gi = g0 + (kIdx ? 0u : lane);
                const bool have = gi < nf && (!kIdx || lane == 0);
                uint32_t a[5], b[5], hw[5];
#pragma unroll
                for (int k = 0; k < 5; k++) {
                    const uint32_t h = have ? S.feat[cur][k][gi] : 0u;
                    hw[k] = h;
                    a[k] = h & kBfMask;
                    b[k] = h & kBigMask;
                }
                bool ipred = false;
                if (kMode == kCommitRound) {
                    const uint32_t o = t * kTileCap + gi;
                    const uint32_t w = __shfl_sync(0xffffffffu, pw, ((o >> 5) - ((t * kTileCap) >> 5)) & 31u);
                    ipred = have && ((w >> (o & 31u)) & 1u);
                }
                uint32_t start = 0;
                n_groups++;
                while (true) {
                    const bool act = have && lane >= start;
                    if (!__any_sync(0xffffffffu, act)) break;
                    n_loops++;
                    // pass 1: state before the group, publish holders
                    uint32_t fpre = 0, gpre = 0;
                    if (act) {
#pragma unroll
                        for (int k = 0; k < 5; k++) {
                            fpre |= ((S.F[a[k] >> 5] >> (a[k] & 31)) & 1u) << k;
                            gpre |= ((S.G[b[k] >> 5] >> (b[k] & 31)) & 1u) << k;
                            atomicOr(&S.own[a[k]], 1u << lane);
                        }
                    }
                    __syncwarp();
                    // pass 2: holders of each index
                    uint32_t m[5];
#pragma unroll
                    for (int k = 0; k < 5; k++) m[k] = act ? S.own[a[k]] : 0u;
                    __syncwarp();
                    if (act) {
#pragma unroll
                        for (int k = 0; k < 5; k++) S.own[a[k]] = 0;
                    }
                    // 256-byte filter: new iff unset before the group and this
                    // lane is the first holder
                    bool fpass = false;
#pragma unroll
                    for (int k = 0; k < 5; k++)
                        if (act && !((fpre >> k) & 1u) && (uint32_t)(__ffs(m[k]) - 1) == lane) fpass = true;
                    const uint32_t fmask = __ballot_sync(0xffffffffu, fpass);
                    // index: insert_sha1 of the filter-passing feature; it goes
                    // on only if that set a new index bit
                    bool inew = true;
                    if (kMode == kCommitRound) inew = fpass && ipred;
                    if (kIdx) {
                        inew = false;
                        if (fpass) {
#pragma unroll
                            for (int k = 0; k < 5; k++) {
                                const uint32_t pos = hw[k] & P.index_mask, bit = 1u << (pos & 31);
                                if (!(atomicOr(P.index_bits + (pos >> 5), bit) & bit)) inew = true;
                            }
                            if (inew) atomicAdd(P.index_new, 1ull);
                        }
                    }
                    // big filter: new iff unset before the group and no earlier
                    // filter-passing lane holds the same 17-bit value
                    uint32_t gnew = 0, pend = 0;
                    uint32_t cand[5];
                    const uint32_t imask = kMode == kCommitRound ? __ballot_sync(0xffffffffu, fpass && inew) : fmask;
#pragma unroll
                    for (int k = 0; k < 5; k++) {
                        cand[k] = m[k] & imask & lanemask_lt();
                        if (fpass && inew && !((gpre >> k) & 1u)) {
                            if (cand[k]) pend |= 1u << k;
                            else gnew |= 1u << k;
                        }
                    }
                    while (__any_sync(0xffffffffu, pend != 0)) {
                        // each pending lane checks one candidate lane per pass
                        int kk = pend ? __ffs(pend) - 1 : 0;
                        uint32_t ck = 0, vk = 0;
#pragma unroll
                        for (int k = 0; k < 5; k++)
                            if (k == kk) {
                                ck = cand[k];
                                vk = b[k];
                            }
                        const uint32_t j = pend ? (uint32_t)(__ffs(ck) - 1) : lane;
                        bool same = false;
#pragma unroll
                        for (int q = 0; q < 5; q++) same |= (__shfl_sync(0xffffffffu, b[q], j) == vk);
                        if (pend) {
                            ck &= ck - 1u;
#pragma unroll
                            for (int k = 0; k < 5; k++)
                                if (k == kk) cand[k] = ck;
                            if (same) pend &= ~(1u << kk);
                            else if (ck == 0) {
                                pend &= ~(1u << kk);
                                gnew |= 1u << kk;
                            }
                        }
                    }
                    const bool counted = fpass && inew && gnew != 0;
                    const uint32_t cm = __ballot_sync(0xffffffffu, counted);
                    const uint32_t before = __popc(cm & lanemask_le());
                    const bool hit_small = counted && (last_count + before == (uint32_t)kMaxElem);
                    const bool hit_big = counted && (bigfi + before == (uint32_t)kBigElem);
                    const uint32_t hm = __ballot_sync(0xffffffffu, hit_small || hit_big);
                    const uint32_t r = hm ? (uint32_t)(__ffs(hm) - 1) : 31u;
                    if (kMode == kCommitRound) {
                        // the inserted features of this pass: filter-passing lanes up to r
                        const uint32_t sm = __ballot_sync(0xffffffffu, act && lane <= r && fpass);
                        if (lane == 0 && sm) {
                            const uint32_t base = t * kTileCap + g0, sh = base & 31u;
                            atomicOr(P.index_seen + (base >> 5), sm << sh);
                            if (sh && (sm >> (32u - sh))) atomicOr(P.index_seen + (base >> 5) + 1, sm >> (32u - sh));
                        }
                    }
                    // write the bits of lanes up to r (all of them without a roll-over)
                    if (act && lane <= r) {
#pragma unroll
                        for (int k = 0; k < 5; k++) {
                            atomicOr(&S.F[a[k] >> 5], 1u << (a[k] & 31));
                            if (fpass && inew) atomicOr(&S.G[b[k] >> 5], 1u << (b[k] & 31));
                        }
                    }
                    __syncwarp();
                    if (!hm) {
                        last_count += __popc(cm);
                        bigfi += __popc(cm);
                        break;
                    }
                    const bool roll_small = __shfl_sync(0xffffffffu, hit_small, r);
                    const bool roll_big = __shfl_sync(0xffffffffu, hit_big, r);
                    const uint32_t ncnt = __popc(cm & ((2u << r) - 1u));
                    last_count += ncnt;
                    bigfi += ncnt;
                    if (roll_small) {
                        const bool fits = bf_count <= Fd.filter_cap;
                        for (uint32_t i = lane; i < 64; i += 32) {
                            if (fits) out[(size_t)(bf_count - 1) * 64 + i] = S.F[i];
                            S.F[i] = 0;
                        }
                        if (!fits && lane == 0) atomicAdd(P.counters + 1, 1u);
                        bf_count++;
                        last_count = 0;
                    }
                    if (roll_big) {
                        for (uint32_t i = lane; i < kBigBytes / 4; i += 32) S.G[i] = 0;
                        bigfi = 0;
                    }
                    __syncwarp();
                    start = r + 1;
                }
            }
        }
        cp_async_wait_all();
        __syncwarp();
        // emit the current (last) filter, then the chop of sdbf_core.cc:235-238
        if (bf_count <= Fd.filter_cap) {
            for (uint32_t i = lane; i < 64; i += 32) out[(size_t)(bf_count - 1) * 64 + i] = S.F[i];
        } else if (lane == 0) {
            atomicAdd(P.counters + 1, 1u);
        }
        if (bf_count > 1 && last_count < (uint32_t)kMaxElem / 8) {
            bf_count--;
            last_count = kMaxElem;
        }
        if (lane == 0) {
            P.out_info[file].bf_count = bf_count;
            P.out_info[file].last_count = last_count;
            if (P.phase) {
                const long long busy = clock64() - t_file;
                atomicAdd(P.phase + kPhCommitWait, (unsigned long long)t_wait);
                atomicAdd(P.phase + kPhCommitBusy, (unsigned long long)busy);
                atomicAdd(P.phase + kPhCommitGroups, (unsigned long long)n_groups);
                atomicAdd(P.phase + kPhCommitLoops, (unsigned long long)n_loops);
                atomicMax(P.phase + kPhCommitMaxFile, (unsigned long long)busy);
            }
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kCommitWarps * 32) k_stream_commit(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    commit_files<kCommitPlain>(P, smem);
}

__global__ void __launch_bounds__(kCommitWarps * 32) k_stream_commit_index(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    commit_files<kCommitSeq>(P, smem);
}

__global__ void __launch_bounds__(kCommitWarps * 32) k_stream_commit_round(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    commit_files<kCommitRound>(P, smem);
}

// Features of a stream launch recorded in a seen bitmap (ordinal = tile *
// kTileCap + feature): the first setter of each of their index bits, then
// (once the rounds agree) the bits and the count of first setters.
// k_stream_index_pred: for every feature, whether it would own the first
// setting of one of its bits (one bit per ordinal, a warp per word).
__global__ void k_stream_index_pred(const uint32_t* __restrict__ feats, const TileOut* __restrict__ tile_out,
                                    uint32_t ntiles, const uint32_t* __restrict__ first, uint32_t mask,
                                    uint32_t* __restrict__ pred) {
    const uint64_t n = (uint64_t)ntiles * kTileCap, npad = (n + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npad; i += (uint64_t)gridDim.x * blockDim.x) {
        bool p = false;
        if (i < n) {
            const uint32_t t = (uint32_t)(i / kTileCap), g = (uint32_t)(i - (uint64_t)t * kTileCap);
            if (g < tile_out[t].count) {
                const uint32_t* w = feats + (size_t)t * 5 * kTileCap + g;
#pragma unroll
                for (int k = 0; k < 5; k++) p |= __ldg(first + (w[(size_t)k * kTileCap] & mask)) >= (uint32_t)i + 1u;
            }
        }
        const uint32_t word = __ballot_sync(0xffffffffu, p);
        if ((threadIdx.x & 31) == 0) pred[i >> 5] = word;
    }
}

__global__ void k_stream_index_first(const uint32_t* __restrict__ feats, const TileOut* __restrict__ tile_out,
                                     uint32_t ntiles, const uint32_t* __restrict__ seen, uint32_t mask,
                                     uint32_t* __restrict__ first) {
    const uint64_t n = (uint64_t)ntiles * kTileCap;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!((seen[i >> 5] >> (i & 31)) & 1u)) continue;
        const uint32_t t = (uint32_t)(i / kTileCap), g = (uint32_t)(i - (uint64_t)t * kTileCap);
        if (g >= tile_out[t].count) continue;
        const uint32_t* w = feats + (size_t)t * 5 * kTileCap + g;
#pragma unroll
        for (int k = 0; k < 5; k++) atomicMin(first + (w[(size_t)k * kTileCap] & mask), (uint32_t)i + 1u);
    }
}

__global__ void k_stream_index_mark(const uint32_t* __restrict__ feats, const TileOut* __restrict__ tile_out,
                                    uint32_t ntiles, const uint32_t* __restrict__ seen, uint32_t mask,
                                    const uint32_t* __restrict__ first, uint32_t* __restrict__ bits,
                                    unsigned long long* __restrict__ count) {
    const uint64_t n = (uint64_t)ntiles * kTileCap;
    uint32_t mine = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!((seen[i >> 5] >> (i & 31)) & 1u)) continue;
        const uint32_t t = (uint32_t)(i / kTileCap), g = (uint32_t)(i - (uint64_t)t * kTileCap);
        if (g >= tile_out[t].count) continue;
        const uint32_t* w = feats + (size_t)t * 5 * kTileCap + g;
        bool fresh = false;
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const uint32_t pos = w[(size_t)k * kTileCap] & mask;
            fresh |= first[pos] == (uint32_t)i + 1u;
            atomicOr(bits + (pos >> 5), 1u << (pos & 31));
        }
        mine += fresh;
    }
    for (int d = 16; d > 0; d >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, d);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(count, (unsigned long long)mine);
}

__global__ void k_pred_dirty(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint64_t nwords,
                             const GenTile* __restrict__ tiles, const GenChunk* __restrict__ chunks, uint32_t ntiles,
                             uint8_t* __restrict__ dirty, uint32_t* __restrict__ from,
                             unsigned int* __restrict__ ndirty) {
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nwords;
         w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = a[w] ^ b[w];
        while (x) {
            const uint64_t ord = w * 32 + (uint32_t)(__ffs(x) - 1);
            x &= x - 1u;
            const uint64_t t = ord / kTileCap;
            if (t >= ntiles) continue;
            const uint32_t f = chunks[tiles[t].chunk].file;
            atomicMin(from + f, (uint32_t)ord);
            if (!dirty[f]) {
                dirty[f] = 1;
                atomicAdd(ndirty, 1u);
            }
        }
    }
}

// ------------------------------------------------------------ block mode
__device__ inline TileGeom block_geom(uint32_t n) {
    TileGeom g;
    g.n = n;
    g.t0 = 0;
    g.S0 = 0;
    g.Q0 = 0;
    g.SE = n - kWin;
    g.L = n - kWin;
    g.RE = n;
    g.BE = n;
    return g;
}

__global__ void __launch_bounds__(kGenThreads) k_block_digest(GenParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ int32_t dtab[65];
    __shared__ uint32_t histo[66];
    __shared__ uint32_t counts[kGenThreads / 32];
    __shared__ uint32_t filt[64];
    __shared__ uint32_t hsh[kGenThreads][5];
    __shared__ int state[4];  // k, allowed, hashed, done
    for (uint32_t i = threadIdx.x; i < 65; i += blockDim.x) dtab[i] = i < 64 ? (int32_t)P.ent_tab[i + 1] - (int32_t)P.ent_tab[i] : 0;
    __syncthreads();
    __shared__ uint16_t s_rank[(SDBF_RANK_BINS + 7) / 8 * 8];
    for (uint32_t i = threadIdx.x; i < SDBF_RANK_BINS; i += blockDim.x) s_rank[i] = P.rank_tab[i];
    __syncthreads();
    const uint16_t* rank_tab = s_rank;
    TileSmem s = carve(smem, P.block_lmax);
    for (uint32_t b = blockIdx.x; b < P.nchunks; b += gridDim.x) {
        const GenChunk C = P.chunks[b];
        const TileGeom g = block_geom(C.n);
        tile_pipeline(P.data + C.data_off, g, s, rank_tab, dtab, nullptr, nullptr, nullptr, P.lead, nullptr);
        const uint8_t* sc = reinterpret_cast<const uint8_t*>(s.score32);
        const uint32_t nown = g.SE;
        if (threadIdx.x < 66) histo[threadIdx.x] = 0;
        if (threadIdx.x < 64) filt[threadIdx.x] = 0;
        __syncthreads();
        if (C.kind == 0) {
            for (uint32_t o = threadIdx.x; o < nown; o += blockDim.x) atomicAdd(&histo[sc[o]], 1u);
            __syncthreads();
            if (threadIdx.x == 0) {
                // thresholding of thread_gen_block_sdbf (sdbf_core.cc:271-276);
                // k may end at 15 when the loop does not break
                int k = 65;
                uint32_t sum = 0;
                for (; k >= kThreshold; k--) {
                    if (sum <= (uint32_t)kMaxElemDD && sum + histo[k] > (uint32_t)kMaxElemDD) break;
                    sum += histo[k];
                }
                state[0] = k;
                state[1] = kMaxElemDD - (int)sum;
            }
        } else if (threadIdx.x == 0) {
            state[0] = kThreshold;  // tail block (sdbf_core.cc:315)
            state[1] = kMaxElemDD;
        }
        if (threadIdx.x == 0) {
            state[2] = 0;
            state[3] = 0;
        }
        __syncthreads();
        const uint32_t k = (uint32_t)state[0];
        const uint32_t ncand = compact(s, nown, k, true, counts);
        // owner masks of the insert passes, over space dead once the scores
        // are known
        uint32_t* own = s.own;
        for (uint32_t i = threadIdx.x; i < 2048; i += blockDim.x) own[i] = 0;
        __syncthreads();
        for (uint32_t base = 0; base < ncand; base += blockDim.x) {
            if (state[3]) break;
            const uint32_t ci = base + threadIdx.x;
            if (ci < ncand) {
                const uint32_t p = s.list[ci];
                uint32_t w[16], h[5];
                load_be16(s.bytes32, p, w);
                sha1_feature(w, h);
#pragma unroll
                for (int q = 0; q < 5; q++) hsh[threadIdx.x][q] = h[q];
            }
            __syncthreads();
            if (threadIdx.x < 32) {
                // gen_block_hash ordered insert (sdbf_core.cc:157-183) by warp 0,
                // 32 candidates per pass: a candidate is eligible if its score
                // is above k, or equal to k while `allowed` lasts; an eligible
                // one sets its 5 filter bits and is counted if one was new.
                // A pass takes every lane as eligible, then keeps the lanes
                // before the first one that was counted past the allowance
                // (that lane is skipped and the rest re-run with the allowance
                // spent) and stops after the lane that reaches 192.
                const uint32_t lane = threadIdx.x;
                int allowed = state[1];
                int hashed = state[2];
                const uint32_t lim = min(ncand - base, (uint32_t)blockDim.x);
                for (uint32_t g0 = 0; g0 < lim && hashed < kMaxElemDD; g0 += 32) {
                    const uint32_t q = g0 + lane;
                    const bool have = q < lim;
                    const bool isK = have && sc[s.list[base + (have ? q : 0)]] == k;
                    uint32_t a[5];
#pragma unroll
                    for (int z = 0; z < 5; z++) a[z] = have ? (hsh[q][z] & kBfMask) : 0u;
                    uint32_t start = 0;
                    bool stop = false;
                    while (true) {
                        const bool act = have && lane >= start && (!isK || allowed > 0);
                        if (!__any_sync(0xffffffffu, act)) break;
                        uint32_t fpre = 0;
                        if (act) {
#pragma unroll
                            for (int z = 0; z < 5; z++) {
                                fpre |= ((filt[a[z] >> 5] >> (a[z] & 31)) & 1u) << z;
                                atomicOr(&own[a[z]], 1u << lane);
                            }
                        }
                        __syncwarp();
                        uint32_t m[5];
#pragma unroll
                        for (int z = 0; z < 5; z++) m[z] = act ? own[a[z]] : 0u;
                        __syncwarp();
                        if (act) {
#pragma unroll
                            for (int z = 0; z < 5; z++) own[a[z]] = 0;
                        }
                        bool added = false;
#pragma unroll
                        for (int z = 0; z < 5; z++)
                            if (act && !((fpre >> z) & 1u) && (uint32_t)(__ffs(m[z]) - 1) == lane) added = true;
                        const uint32_t cm = __ballot_sync(0xffffffffu, added);
                        const uint32_t ckm = __ballot_sync(0xffffffffu, added && isK);
                        const uint32_t le = lanemask_le();
                        const uint32_t om =
                            __ballot_sync(0xffffffffu, added && isK && __popc(ckm & le) > allowed);
                        const uint32_t L = om ? (uint32_t)(__ffs(om) - 1) : 32u;
                        const uint32_t fm =
                            __ballot_sync(0xffffffffu, added && hashed + __popc(cm & le) == kMaxElemDD);
                        const uint32_t H = fm ? (uint32_t)(__ffs(fm) - 1) : 32u;
                        const uint32_t rx = min(L, H + 1);  // lanes [0, rx) stand
                        const uint32_t keep = rx >= 32 ? 0xffffffffu : ((1u << rx) - 1u);
                        if (act && lane < rx) {
#pragma unroll
                            for (int z = 0; z < 5; z++) atomicOr(&filt[a[z] >> 5], 1u << (a[z] & 31));
                            if (added) {
                                const uint32_t idx = (uint32_t)hashed + __popc(cm & lanemask_lt());
                                if (P.feats) {  // index build: every counted feature (sdbf_core.cc:164-167)
                                    uint32_t* fw = P.feats + (size_t)C.filter * kFeatWords + idx * 5;
#pragma unroll
                                    for (int z = 0; z < 5; z++) fw[z] = hsh[q][z];
                                }
                                if (P.probes && (idx & 3) == 0) {  // index search sample (sdbf_core.cc:168-175)
                                    uint32_t* pr = P.probes + (size_t)C.filter * kProbeWords + (idx >> 2) * 5;
#pragma unroll
                                    for (int z = 0; z < 5; z++) pr[z] = hsh[q][z];
                                }
                            }
                        }
                        hashed += __popc(cm & keep);
                        allowed -= __popc(ckm & keep);
                        __syncwarp();
                        if (H < L) {  // the 192nd element: the block is full
                            stop = true;
                            break;
                        }
                        if (L >= 32) break;
                        start = L + 1;  // lane L is skipped (allowance spent)
                    }
                    if (stop) break;
                }
                if (lane == 0) {
                    state[1] = allowed;
                    state[2] = hashed;
                    if (hashed >= kMaxElemDD) state[3] = 1;
                }
            }
            __syncthreads();
        }
        if (threadIdx.x < 64) P.out_filters[(size_t)C.filter * 64 + threadIdx.x] = filt[threadIdx.x];
        if (threadIdx.x == 0) P.out_counts[C.filter] = (uint16_t)state[2];
        if (threadIdx.x == 0 && P.nprobes) P.nprobes[C.filter] = (uint8_t)((state[2] + 3) >> 2);
        __syncthreads();
    }
}

// ---------------------------------------------------------------- launch
size_t stream_tile_smem() { return tile_smem_bytes(kTileL); }
size_t stream_tile_smem_pre() { return tile_smem_bytes_pre(kTileL); }
size_t block_smem(uint32_t lmax) { return tile_smem_bytes(lmax); }

static void set_stream_attrs() {
    static bool done = false;
    if (done) return;
    const int sm = (int)stream_tile_smem(), smp = (int)stream_tile_smem_pre();
    cudaFuncSetAttribute(k_stream_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    cudaFuncSetAttribute(k_stream_fix<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    cudaFuncSetAttribute(k_stream_tiles_pre, cudaFuncAttributeMaxDynamicSharedMemorySize, smp);
    cudaFuncSetAttribute(k_stream_fix<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smp);
    cudaFuncSetAttribute(k_stream_fix_list<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    cudaFuncSetAttribute(k_stream_fix_list<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smp);
    cudaFuncSetAttribute(k_stream_ranks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRkSmem);
    cudaFuncSetAttribute(k_stream_commit, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(CommitSmem) * kCommitWarps));
    // one shared-memory / L1 split for every kernel of the stream pipeline
    // (the largest shared memory): CTAs of different kernels can then share
    // an SM
    for (const void* f : {(const void*)k_stream_ranks, (const void*)k_stream_tiles, (const void*)k_stream_tiles_pre,
                          (const void*)k_stream_fails, (const void*)k_stream_fix_list<false>,
                          (const void*)k_stream_fix_list<true>, (const void*)k_stream_check,
                          (const void*)k_stream_fix<false>, (const void*)k_stream_fix<true>,
                          (const void*)k_stream_commit, (const void*)k_stream_commit_round,
                          (const void*)k_stream_commit_index})
        cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    done = true;
}

cudaError_t launch_stream_ranks(const GenParams& P, uint32_t grid, cudaStream_t st) {
    set_stream_attrs();
    if (grid) k_stream_ranks<<<grid, kRkThreads, kRkSmem, st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_stream_tiles(const GenParams& P, uint32_t grid, cudaStream_t st) {
    set_stream_attrs();
    if (P.ranks)
        k_stream_tiles_pre<<<grid, kGenThreads, stream_tile_smem_pre(), st>>>(P);
    else
        k_stream_tiles<<<grid, kGenThreads, stream_tile_smem(), st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_stream_fails(const GenParams& P, uint32_t grid, cudaStream_t st) {
    if (grid) k_stream_fails<<<grid, 256, 0, st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_stream_fix_list(const GenParams& P, uint32_t grid, cudaStream_t st) {
    set_stream_attrs();
    if (P.ranks)
        k_stream_fix_list<true><<<grid, kGenThreads, stream_tile_smem_pre(), st>>>(P);
    else
        k_stream_fix_list<false><<<grid, kGenThreads, stream_tile_smem(), st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_stream_check(const GenParams& P, uint32_t grid, cudaStream_t st) {
    k_stream_check<<<grid, 128, 0, st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_stream_fix(const GenParams& P, uint32_t grid, cudaStream_t st) {
    set_stream_attrs();
    if (P.ranks)
        k_stream_fix<true><<<grid, kGenThreads, stream_tile_smem_pre(), st>>>(P);
    else
        k_stream_fix<false><<<grid, kGenThreads, stream_tile_smem(), st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_stream_commit_index(const GenParams& P, cudaStream_t st) {
    cudaFuncSetAttribute(k_stream_commit_index, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(CommitSmem) * kCommitWarps));
    k_stream_commit_index<<<1, kCommitWarps * 32, sizeof(CommitSmem) * kCommitWarps, st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_stream_commit_round(const GenParams& P, uint32_t grid, cudaStream_t st) {
    cudaFuncSetAttribute(k_stream_commit_round, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(CommitSmem) * kCommitWarps));
    k_stream_commit_round<<<grid, kCommitWarps * 32, sizeof(CommitSmem) * kCommitWarps, st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_stream_index_pred(const GenParams& P, const uint32_t* first, uint32_t* pred, uint32_t grid,
                                     cudaStream_t st) {
    k_stream_index_pred<<<grid, 256, 0, st>>>(P.features, P.tile_out, P.ntiles, first, P.index_mask, pred);
    return cudaGetLastError();
}

cudaError_t launch_stream_index_first(const GenParams& P, const uint32_t* seen, uint32_t* first, uint32_t grid,
                                      cudaStream_t st) {
    k_stream_index_first<<<grid, 256, 0, st>>>(P.features, P.tile_out, P.ntiles, seen, P.index_mask, first);
    return cudaGetLastError();
}

cudaError_t launch_stream_index_mark(const GenParams& P, const uint32_t* seen, const uint32_t* first, uint32_t grid,
                                     cudaStream_t st) {
    k_stream_index_mark<<<grid, 256, 0, st>>>(P.features, P.tile_out, P.ntiles, seen, P.index_mask, first,
                                              P.index_bits, P.index_new);
    return cudaGetLastError();
}

cudaError_t launch_pred_dirty(const GenParams& P, const uint32_t* a, const uint32_t* b, uint64_t nwords,
                              uint8_t* dirty, uint32_t* from, unsigned int* ndirty, uint32_t grid, cudaStream_t st) {
    k_pred_dirty<<<grid, 256, 0, st>>>(a, b, nwords, P.tiles, P.chunks, P.ntiles, dirty, from, ndirty);
    return cudaGetLastError();
}

cudaError_t launch_stream_commit(const GenParams& P, uint32_t grid, cudaStream_t st) {
    set_stream_attrs();
    k_stream_commit<<<grid, kCommitWarps * 32, sizeof(CommitSmem) * kCommitWarps, st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_block(const GenParams& P, uint32_t grid, cudaStream_t st) {
    const size_t sm = block_smem(P.block_lmax);
    cudaFuncSetAttribute(k_block_digest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (P.nchunks) k_block_digest<<<grid, kGenThreads, sm, st>>>(P);
    return cudaGetLastError();
}

}  // namespace sdbfg

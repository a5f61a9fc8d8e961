// matrix_tc.cu -- the filter-matrix comparison counted on the tensor cores.
//
// popcount(a & b) of two 2048-bit filters is the dot product of their bit
// vectors.  With each bit widened to an e4m3 byte (0x08 = 2^-6, or 0) and
// fp32 accumulation, tcgen05.mma computes it exactly: every product is
// 2^-12, every partial sum a multiple of 2^-12 no larger than 2048 * 2^-12,
// well inside fp32's 24-bit significand; the count is the sum times 4096.  One CTA multiplies 128 reference filters (TMEM lanes)
// by tiles of up to 256 target filters (TMEM columns) over K = 2048 in 16
// chunks of 128.  The CTA is a two-stage software pipeline: warps 4-7
// compose tile g, fetch its filter bits with cp.async, widen each chunk into
// a 128-byte-swizzled shared-memory stage (two stages, so widening overlaps
// the MMAs of the previous chunk) and issue the four K=32 MMAs per chunk into
// accumulator g & 1 (512 TMEM columns hold two); meanwhile warps 0-3 read
// tile g-1's counts from the other accumulator, one row per thread, and
// score it exactly as the CUDA-core kernel does (compare_kernels.cu
// k_matrix): a pair can score above 0 only if its full count exceeds the
// cut, and for those rare pairs the reference's staged exits
// (bf_utils.cc:114-206) are rechecked from the filters in memory.  Each
// 32-column slice is scored in two passes: a branch-free pass marks the
// row's counted columns and those above the cut, then the slice's segments
// are walked in column order, re-checking only the marked columns.  Maxima
// of completed targets collect in a ring of eight and are summed in filter
// order as it fills.  Work units, group units, running sums and split pairs
// are those of k_matrix.
//
// The widening permutes K inside each 32-bit word (output word k of a word
// w holds bits k, k+8, k+16, k+24 of w), identically for both operands, so
// the dot product is unchanged; bit k of each byte moves to bit 3 (the
// single set bit of 0x08), one shift and one mask per output word.  --fast digests count only chunks 0-3 (their first
// 64 bytes).
//
// Every mbarrier wait is bounded; a wait that gives up sets P.error, all
// threads leave together (the decision is made by __syncthreads_and), the
// MMAs still in flight are waited for and the TMEM is released.
#include <cstdint>
#include <cuda_runtime.h>

#include "compare_device.cuh"
#include "compare_kernels.h"
#include "sdbf_device.cuh"

namespace sdbfg {

namespace {

constexpr int kTcRows = 128;       // reference rows per pass = TMEM lanes
constexpr int kTcCols = 256;       // target filters per tile = MMA N (max)
constexpr int kTcThreads = 256;    // warps 0-3 score (one row each), warps 4-7 widen and issue
constexpr int kTcChunk = 128;      // K elements (bits) per stage
constexpr int kTcChunks = 2048 / kTcChunk;
constexpr int kTcRing = 8;         // completed targets held before their maxima are summed
constexpr uint32_t kTcAStage = kTcRows * kTcChunk;   // 16 KB of e4m3
constexpr uint32_t kTcBStage = kTcCols * kTcChunk;   // 32 KB
constexpr uint32_t kTcStage = kTcAStage + kTcBStage;
constexpr uint32_t kTcWaitSpins = 1u << 20;
constexpr int kTcBitSlots = 3;     // chunks of filter bits in flight (cp.async ring)

// one tile's composition (double-buffered: warps 4-7 compose and count tile
// k while warps 0-3 score tile k-1)
struct TcTile {
    uint4 tw[8][kTcCols];  // first 128 bytes of each target filter, chunk-major (staged re-check)
    uint32_t gidx[kTcCols], tmeta[kTcCols], tinfo[kTcCols], comp[kTcCols];
    uint32_t seg_first[kTcCols], seg_start[kTcCols + 1], seg_te[kTcCols];  // one segment per target
    uint32_t lastmask[kTcCols / 32];
    uint32_t ntile, ncomp, produced, nseg, last_open;
};

struct TcSmem {
    uint4 bits[kTcBitSlots][kTcRows + kTcCols];  // 16 filter bytes per row per chunk
    TcTile tile[2];
    uint32_t rowf[kTcRows];           // filter index of each reference row (~0: none)
    double mv[kTcRows][kTcRing + 1];  // row maxima of completed targets (ring)
    uint16_t cstage[32][kTcRows];     // one 32-column slice of counts, column-major per row thread
    double run[kMatMaxTargets];
    uint32_t gref[kTcRows], gstart[kTcRows + 1], gsparse[kTcRows];
    uint16_t cut_sum[1024], cut64_sum[1024], cut256[SDBF_CUTOFF_BINS], cut64[SDBF_CUTOFF_BINS];
    MatUnit unit;
    uint32_t unit_id, cur_t, cur_f, sparse, tmem;
    alignas(8) uint64_t mbar[5];      // stage 0, stage 1 emptied; accumulator 0, 1 full; drain
};

static_assert(kTcRows == 128 && kTcCols == 256 && kTcThreads == 256,
              "producer threads widen one reference row and two target columns each");
constexpr size_t kTcSmemBytes = 1024 /* alignment */ + 2 * kTcStage + sizeof(TcSmem);
static_assert(kTcSmemBytes <= 227 * 1024, "tensor-core kernel exceeds the shared memory of one CTA");

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
    for (uint32_t i = 0; i < kTcWaitSpins; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// bit k of every byte of w, as 0x08 or 0x00 in that byte
__device__ __forceinline__ uint32_t bit_to_08(uint32_t w, int k) {
    return (k <= 3 ? w << (3 - k) : w >> (k - 3)) & 0x08080808u;
}

// row r's 128 e4m3 bytes of one chunk from its 128 filter bits (4 words):
// 8 granules of 16 bytes at their swizzled places
__device__ __forceinline__ void widen_row(uint8_t* stage, uint32_t r, uint4 bits) {
    const uint32_t w[4] = {bits.x, bits.y, bits.z, bits.w};
    uint8_t* row = stage + (r >> 3) * 1024 + (r & 7) * 128;
#pragma unroll
    for (int m = 0; m < 4; m++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            uint4 g;
            g.x = bit_to_08(w[m], 4 * h + 0);
            g.y = bit_to_08(w[m], 4 * h + 1);
            g.z = bit_to_08(w[m], 4 * h + 2);
            g.w = bit_to_08(w[m], 4 * h + 3);
            const uint32_t gi = 2 * m + h;
            *reinterpret_cast<uint4*>(row + ((gi ^ (r & 7)) << 4)) = g;
        }
    }
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait2() { asm volatile("cp.async.wait_group 2;" ::: "memory"); }

// slot j of a composed tile: its segment k (seg_start[k] <= j < seg_start[k+1])
__device__ __forceinline__ uint32_t find_segment(const uint32_t* seg_start, uint32_t nseg, uint32_t j) {
    uint32_t lo = 0, hi = nseg;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (seg_start[mid] <= j) lo = mid;
        else hi = mid;
    }
    return lo;
}

// the row's first 128 bytes (the staged re-check needs words 0..31)
struct RowHead {
    uint4 w[8];
};

// A pair whose full count is above the cut (rare): the reference's staged
// exits (normal mode: after 8, 16, 32 words) or its 32-byte stage (fast
// mode), from the row's first 128 bytes and the target's (shared memory,
// 16 bytes every kTcCols uint4s).
// Returns (num << 32) | den of the pair's score (0 / 1 when it scores 0).
__device__ __forceinline__ uint64_t candidate_fraction(const RowHead& aw, const uint4* tw, uint32_t cnt,
                                                      uint32_t cut, bool fast, uint32_t max_est) {
    // all eight loads first, then the three stage counts (an exit at any
    // stage is an exit: the stages only end the count early)
    uint32_t p[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const uint4 y = tw[q * kTcCols];
        p[q] = __popc(aw.w[q].x & y.x) + __popc(aw.w[q].y & y.y) + __popc(aw.w[q].z & y.z) + __popc(aw.w[q].w & y.w);
    }
    const uint32_t c1 = p[0] + p[1], c2 = c1 + p[2] + p[3], c3 = c2 + p[4] + p[5] + p[6] + p[7];
    const bool exit = fast ? 2 * c1 + 48 < cut : (8 * c1 + 48 < cut || 4 * c2 + 48 < cut || 2 * c3 + 48 < cut);
    if (exit || cnt <= cut) return 1;
    return ((uint64_t)(cnt - cut) << 32) | (uint32_t)(max_est - cut);
}

// A row's maximum over a completed target (max_value), with the division
// of the rare positive score out of line.
__device__ __noinline__ double score_ratio(uint32_t bnum, uint32_t bden) { return __ddiv_rn((double)bnum, (double)bden); }

__device__ __forceinline__ double row_maximum(bool active, uint32_t bnum, uint32_t bden, bool counted) {
    if (!active) return 0.0;
    if (!counted) return -1.0;
    return bnum == 0 ? 0.0 : score_ratio(bnum, bden);
}

// Sums the maxima of `done` completed targets (completion indices from
// ring_base) in filter order: group units finish their (reference, target)
// scores, multi-pass units extend the running sums.  All 128 consumer threads.
__device__ __noinline__ void fold_ring(const MatParams& P, TcSmem& S, const TcTile& T, uint32_t ring_base,
                                       uint32_t done, bool group, uint32_t nref, uint32_t nrows, uint32_t t0,
                                       uint32_t rs, uint32_t tid) {
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (group) {
        for (uint32_t t = tid; t < done * nref; t += 128) {
            const uint32_t kk = t % nref, ci = ring_base + t / nref;
            double sum = -1.0;
            for (uint32_t r = S.gstart[kk]; r < S.gstart[kk + 1]; r++) {
                const double m = S.mv[r][ci % kTcRing];
                if (sum < 0) sum = m;
                else if (m != 0.0) sum = __dadd_rn(sum, m);
            }
            const uint32_t tgt = P.targets[t0 + T.comp[ci]];
            P.scores[out_index(P, rs != 0, S.gref[kk], tgt)] =
                final_score(sum, S.gstart[kk + 1] - S.gstart[kk], S.gsparse[kk]);
        }
    } else {
        for (uint32_t t = tid; t < done; t += 128) {
            const uint32_t ci = ring_base + t;
            double sum = S.run[T.comp[ci]];
            for (uint32_t r = 0; r < nrows; r++) {
                const double m = S.mv[r][ci % kTcRing];
                if (sum < 0) sum = m;
                else if (m != 0.0) sum = __dadd_rn(sum, m);
            }
            S.run[T.comp[ci]] = sum;
        }
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
}

}  // namespace

// AND-reduction of a predicate over one 128-thread group (named barrier id)
template <int ID>
__device__ __forceinline__ bool group_and(bool v) {
    uint32_t r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, 128, p;\n"
                 " selp.u32 %0, 1, 0, q;\n}\n"
                 : "=r"(r)
                 : "r"((uint32_t)v), "n"(ID)
                 : "memory");
    return r != 0;
}

template <int ID>
__device__ __forceinline__ void group_sync() {
    asm volatile("bar.sync %0, 128;" ::"n"(ID) : "memory");
}

#define TC_STAMP(var) const long long var = P.phase ? clock64() : 0
#define TC_ADD(ph, t0) \
    do { if (P.phase) atomicAdd(P.phase + (ph), (unsigned long long)(clock64() - (t0))); } while (0)

__global__ void __launch_bounds__(kTcThreads, 1) k_matrix_tc(MatParams P) {
    extern __shared__ uint8_t tc_smem_raw[];
    const uint32_t raw = smem_addr(tc_smem_raw);
    uint8_t* stages = tc_smem_raw + (((raw + 1023) & ~1023u) - raw);
    TcSmem& S = *reinterpret_cast<TcSmem*>(stages + 2 * kTcStage);
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool producer = warp >= 4;
    const uint32_t ptid = tid - 128;  // producers: 0..127

    for (uint32_t i = tid; i < 1024; i += kTcThreads) {
        S.cut_sum[i] = P.cutoffs[i >= 32 ? 4096u / i : (uint32_t)SDBF_CUTOFF_BINS - 1];
        S.cut64_sum[i] = P.cutoffs64[i >= 8 ? 1024u / i : (uint32_t)SDBF_CUTOFF_BINS - 1];
    }
    for (uint32_t i = tid; i < SDBF_CUTOFF_BINS; i += kTcThreads) {
        S.cut256[i] = P.cutoffs[i];
        S.cut64[i] = P.cutoffs64[i];
    }
    if (tid == 0) {
        for (int i = 0; i < 5; i++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&S.mbar[i])));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {  // two accumulators of 256 columns
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&S.tmem)),
                     "r"(2 * kTcCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = S.tmem;

    uint32_t suses[2] = {0, 0};  // producers: commits to each stage barrier
    uint32_t gtile = 0;          // tiles counted so far (all threads keep the same count)
    bool ok = true;

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            const uint32_t u = atomicAdd(P.next_unit, 1u);
            S.unit_id = u;
            if (u < P.nunits) S.unit = P.units[u];
        }
        __syncthreads();
        if (S.unit_id >= P.nunits) break;
        const MatUnit U = S.unit;
        const uint32_t rs = U.flags & kUnitRefSide1 ? 1 : 0, ts = U.flags & kUnitTgtSide1 ? 1 : 0;
        const bool split = (U.flags & kUnitSplit) != 0;
        const bool group = (U.flags & kUnitGroup) != 0;
        const uint32_t nref = group ? U.nref : 1;
        const uint32_t nT = U.t1 - U.t0;
        if (group) {
            if (tid < 32) {
                uint32_t base_row = 0;
                for (uint32_t b = 0; b < nref; b += 32) {
                    const uint32_t k = b + lane;
                    uint32_t n = 0, id = 0;
                    if (k < nref) {
                        id = P.refs[U.ref + k];
                        n = P.digests[rs][id].nfilters;
                    }
                    uint32_t incl = n;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
                        if (lane >= (uint32_t)d) incl += v;
                    }
                    if (k < nref) {
                        S.gref[k] = id;
                        S.gstart[k] = base_row + incl - n;
                        S.gsparse[k] = 0;
                    }
                    base_row += __shfl_sync(0xffffffffu, incl, 31);
                }
                if (lane == 0) S.gstart[nref] = base_row;
            }
        } else {
            for (uint32_t k = tid; k < nT && !split; k += kTcThreads) S.run[k] = -1.0;
        }
        if (tid == 0) S.sparse = 0;
        __syncthreads();
        const CmpDigest A = P.digests[rs][group ? S.gref[0] : U.ref];
        const bool fastA = (A.flags & kDigestFast) != 0;
        const uint32_t nch = fastA ? 4 : kTcChunks;  // fast mode: the first 64 bytes

        for (uint32_t rc = U.r0; rc < U.r1 && ok; rc += kTcRows) {
            // ---- reference rows of this pass (threads 0..127)
            const uint32_t row = rc + tid;
            const bool have = tid < kTcRows && row < U.r1;
            uint32_t s1 = 0, e1 = 0, gk = 0;
            uint32_t fidx = A.first + row;
            if (group && have) {
                uint32_t lo = 0, hi = nref;
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (S.gstart[mid] <= row) lo = mid;
                    else hi = mid;
                }
                gk = lo;
                fidx = P.digests[rs][S.gref[gk]].first + (row - S.gstart[gk]);
            }
            if (have) {
                const uint32_t m = P.meta[rs][fidx];
                s1 = m & 0xFFFFu;
                e1 = m >> 16;
            }
            if (tid < kTcRows) S.rowf[tid] = have ? fidx : 0xFFFFFFFFu;
            const bool active = have && s1 >= (uint32_t)kMinElem;
            if (group && have && !active) atomicAdd(&S.gsparse[gk], 1u);
            const uint32_t nsparse = __syncthreads_count(have && !active);
            if (tid == 0) {
                S.sparse += nsparse;
                S.cur_t = 0;
                S.cur_f = 0;
                S.tile[0].produced = 0;
                S.tile[1].produced = 0;
            }
            uint32_t bnum = 0, bden = 1;
            bool counted = false;
            const uint32_t nrows = min((uint32_t)kTcRows, U.r1 - rc);
            RowHead aw;  // the row's first 128 bytes, for the staged re-check of candidates
#pragma unroll
            for (int q = 0; q < 8; q++)
                aw.w[q] = have ? __ldg(reinterpret_cast<const uint4*>(P.filters[rs] + (size_t)fidx * 64) + q)
                               : make_uint4(0, 0, 0, 0);
            __syncthreads();
            // ---- software pipeline: each step counts tile g (producers) and
            // scores tile g-1 (consumers); one CTA barrier per step.  Tile g
            // uses accumulator and tile slot g & 1, so accumulator b's n-th use
            // is tile 2n + b and its barrier parity is (g >> 1) & 1.
            bool pending = false;  // a counted tile waits to be scored
            for (;;) {
                const uint32_t b = gtile & 1;  // tile gtile is counted into accumulator / tile slot b
                TC_STAMP(t_step);
                if (producer) {
                    TcTile& T = S.tile[b];
                    TC_STAMP(t_comp);
                    if (warp == 4) {  // compose tile g: up to 256 filters of up to 256 targets
                        uint32_t filled = 0, ncomp = 0, nseg = 0, ct = S.cur_t, cf = S.cur_f;
                        bool open = false;
                        while (filled < (uint32_t)kTcCols && ct < nT) {
                            const uint32_t te = ct + lane;
                            const uint32_t f0 = lane == 0 ? cf : 0;
                            uint32_t rem = 0, first = 0;
                            if (te < nT) {
                                const CmpDigest B = P.digests[ts][P.targets[U.t0 + te]];
                                rem = B.nfilters - f0;
                                first = B.first + f0;
                            }
                            uint32_t incl = rem;
#pragma unroll
                            for (int d = 1; d < 32; d <<= 1) {
                                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
                                if (lane >= (uint32_t)d) incl += v;
                            }
                            const uint32_t excl = incl - rem, room = (uint32_t)kTcCols - filled;
                            const bool done_here = rem > 0 && incl <= room;
                            const bool has = rem > 0 && excl < room;
                            if (has) {  // every earlier segment of this tile completed, so index nseg + lane
                                T.seg_first[nseg + lane] = first;
                                T.seg_start[nseg + lane] = filled + excl;
                                T.seg_te[nseg + lane] = te;
                            }
                            if (done_here) T.comp[ncomp + lane] = te;
                            const uint32_t done_mask = __ballot_sync(0xffffffffu, done_here);
                            const uint32_t has_mask = __ballot_sync(0xffffffffu, has);
                            const uint32_t over_mask = __ballot_sync(0xffffffffu, rem > 0 && incl > room);
                            const uint32_t open_mask = __ballot_sync(0xffffffffu, has && incl > room);
                            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                            ncomp += __popc(done_mask);
                            nseg += __popc(has_mask);
                            if (over_mask) {
                                const uint32_t l = __ffs(over_mask) - 1;
                                const uint32_t ex_l = __shfl_sync(0xffffffffu, excl, l);
                                const uint32_t f0_l = __shfl_sync(0xffffffffu, f0, l);
                                ct += l;
                                cf = f0_l + (room - ex_l);
                                filled = kTcCols;
                                open = open_mask != 0;
                            } else {
                                ct = min(ct + 32u, nT);
                                cf = 0;
                                filled += total;
                            }
                        }
                        if (lane < kTcCols / 32) T.lastmask[lane] = 0;
                        if (lane == 0) {
                            S.cur_t = ct;
                            S.cur_f = cf;
                            T.ntile = filled;
                            T.ncomp = ncomp;
                            T.nseg = nseg;
                            T.seg_start[nseg] = filled;
                            T.last_open = open;
                            T.produced = filled > 0;
                        }
                    }
                    group_sync<2>();
                    if (ptid == 0) TC_ADD(kTcPhCompose, t_comp);
                    TC_STAMP(t_fill);
                    // slots of the tile, filled by all producers (loads in parallel)
                    {
                        const uint32_t nseg = T.nseg;
                        for (uint32_t j = ptid; j < T.ntile; j += 128) {
                            const uint32_t k = find_segment(T.seg_start, nseg, j);
                            const uint32_t f = T.seg_first[k] + (j - T.seg_start[k]);
                            const bool last = j + 1 == T.seg_start[k + 1] && !(k + 1 == nseg && T.last_open);
                            T.gidx[j] = f;
                            T.tmeta[j] = P.meta[ts][f];
                            T.tinfo[j] = T.seg_te[k] | (k << 16) | (last ? 0x80000000u : 0u);
                            if (last) atomicOr(&T.lastmask[j >> 5], 1u << (j & 31));
                        }
                    }
                    group_sync<2>();
                    if (ptid == 0) TC_ADD(kTcPhFill, t_fill);
                    if (T.produced) {
                        if (ptid == 0 && P.phase) atomicAdd(P.phase + kTcPhTiles, 1ull);
                        const uint32_t nt = T.ntile;
                        const uint32_t ncols = (nt + 15) & ~15u;  // MMA N: multiple of 16
                        const uint32_t idesc = (1u << 4) | ((ncols >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
                        const uint32_t dacc = tmem + b * kTcCols;
                        auto fetch = [&](uint32_t c) {
                            uint4* slot = S.bits[c % kTcBitSlots];
                            for (uint32_t i = ptid; i < kTcRows + ncols; i += 128) {
                                if (i < kTcRows) {
                                    const uint32_t f = S.rowf[i];
                                    if (f != 0xFFFFFFFFu) cp_async16(slot + i, P.filters[rs] + (size_t)f * 64 + c * 4);
                                } else if (i - kTcRows < nt) {
                                    cp_async16(slot + i, P.filters[ts] + (size_t)T.gidx[i - kTcRows] * 64 + c * 4);
                                }
                            }
                            cp_async_commit();
                        };
                        fetch(0);
                        if (nch > 1) fetch(1);
                        for (uint32_t c = 0; c < nch; c++) {
                            TC_STAMP(t_fw);
                            if (c + 2 < nch) fetch(c + 2);
                            else cp_async_commit();
                            cp_async_wait2();
                            if (ptid == 0) TC_ADD(kTcPhFetchWait, t_fw);
                            TC_STAMP(t_sw);
                            const uint32_t s = (suses[0] + suses[1]) & 1;
                            bool w = true;
                            if (suses[s] > 0) w = mbar_wait(smem_addr(&S.mbar[s]), (suses[s] - 1) & 1);
                            ok = group_and<2>(ok && w);
                            if (ptid == 0) TC_ADD(kTcPhStageWait, t_sw);
                            if (!ok) break;
                            TC_STAMP(t_wd);
                            uint8_t* sa = stages + s * kTcStage;
                            uint8_t* sb = sa + kTcAStage;
                            const uint4* slot = S.bits[c % kTcBitSlots];
                            {
                                // each producer thread: reference row ptid and target
                                // columns ptid, ptid + 128 (zero bits past the tile);
                                // the three loads first, then the three widenings
                                const uint32_t c1 = ptid, c2 = ptid + 128;
                                const uint4 z = make_uint4(0, 0, 0, 0);
                                const uint4 ba = S.rowf[ptid] != 0xFFFFFFFFu ? slot[ptid] : z;
                                const uint4 b1 = c1 < nt ? slot[kTcRows + c1] : z;
                                const uint4 b2 = c2 < nt ? slot[kTcRows + c2] : z;
                                if (c < 8) {
                                    if (c1 < nt) T.tw[c][c1] = b1;
                                    if (c2 < nt) T.tw[c][c2] = b2;
                                }
                                widen_row(sa, ptid, ba);
                                if (c1 < ncols) widen_row(sb, c1, b1);
                                if (c2 < ncols) widen_row(sb, c2, b2);
                            }
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            group_sync<2>();
                            if (ptid == 0) TC_ADD(kTcPhWiden, t_wd);
                            TC_STAMP(t_is);
                            if (ptid == 0) {
                                asm volatile("tcgen05.fence::after_thread_sync;");
                                const uint32_t a0 = smem_addr(sa), b0 = smem_addr(sb);
#pragma unroll
                                for (uint32_t kk = 0; kk < kTcChunk / 32; kk++) {
                                    const uint64_t ad = sw128_desc(a0 + kk * 32), bd = sw128_desc(b0 + kk * 32);
                                    const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
                                    asm volatile(
                                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                        " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(dacc),
                                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                                }
                                mma_commit(smem_addr(&S.mbar[s]));
                                TC_ADD(kTcPhIssue, t_is);
                            }
                            suses[s]++;
                        }
                        if (ok && ptid == 0) mma_commit(smem_addr(&S.mbar[2 + b]));
                    }
                    if (ptid == 0) TC_ADD(kTcPhProdStep, t_step);
                } else if (pending) {
                    // ---- consumers: score tile gtile-1 from accumulator 1-b
                    const uint32_t pb = b ^ 1;
                    const TcTile& T = S.tile[pb];
                    const uint32_t g = gtile - 1;  // its tile number: the (g >> 1)-th use of accumulator pb
                    TC_STAMP(t_aw);
                    bool w = mbar_wait(smem_addr(&S.mbar[2 + pb]), (g >> 1) & 1);
                    ok = group_and<1>(ok && w);
                    if (tid == 0) TC_ADD(kTcPhAccWait, t_aw);
                    TC_STAMP(t_sc);
                    if (ok) {
                        asm volatile("tcgen05.fence::after_thread_sync;");
                        uint32_t ring_base = 0;                 // completion index of ring slot 0
                        const uint32_t nt = T.ntile;
                        uint32_t pend = 0;  // completed targets in the ring, not yet summed
                        for (uint32_t c0 = 0; c0 < nt; c0 += 32) {
                            TC_STAMP(t_ld);
                            uint32_t v[32];
                            const uint32_t taddr = tmem + ((warp * 32) << 16) + pb * kTcCols + c0;
                            asm volatile(
                                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
                                "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                                  "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
                                  "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
                                  "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
                                  "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
                                  "=r"(v[31])
                                : "r"(taddr));
                            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                            for (int q = 0; q < 32; q++) S.cstage[q][tid] = (uint16_t)(__uint_as_float(v[q]) * 4096.0f);
                            if (tid == 0) TC_ADD(kTcPhLd, t_ld);
                            const uint32_t lim = min(32u, nt - c0);
                            const uint32_t valid = lim == 32 ? 0xFFFFFFFFu : (1u << lim) - 1u;
                            // pass 1, no branches: which columns count for this row
                            // (kmask) and which are above the cut (cmask)
                            uint32_t kmask = 0, cmask = 0;
                            TC_STAMP(t_mk);
                            // a table lookup only: element sums of 1024 and more (beyond
                            // the reference's limits, never produced by its generator) are
                            // marked and get their exact cut in pass 2
                            const uint16_t* ctab = fastA ? S.cut64_sum : S.cut_sum;
                            // (all 32 columns from the registers; c0 + 31 < 256, so the
                            // columns past the tile read stale entries and are masked off)
#pragma unroll
                            for (uint32_t q = 0; q < 32; q++) {
                                const uint32_t s2 = T.tmeta[c0 + q] & 0xFFFFu;
                                const uint32_t sum = s1 + s2;
                                const uint32_t cut = sum < 1024 ? ctab[sum] : 0u;
                                const bool ct = s2 >= (uint32_t)kMinElem;
                                kmask |= (uint32_t)ct << q;
                                cmask |= (uint32_t)(ct && (uint32_t)(__uint_as_float(v[q]) * 4096.0f) > cut) << q;
                            }
                            kmask = active ? kmask & valid : 0u;
                            cmask = active ? cmask & valid : 0u;
                            // pass 2: the slice's segments in column order (the same for
                            // every thread, so the ring fold's barrier stays uniform); in
                            // each, this row's columns above the cut, then the segment end
                            if (tid == 0) TC_ADD(kTcPhMark, t_mk);
                            TC_STAMP(t_wk);
                            uint32_t lmq = T.lastmask[c0 >> 5] & valid;
                            uint32_t q0 = 0;
                            for (;;) {
                                const uint32_t qe = lmq ? (uint32_t)(__ffs(lmq) - 1) : lim;  // end column (incl.) or slice end
                                const uint32_t upto = lmq ? qe + 1 : lim;
                                const uint32_t range = (upto == 32 ? 0xFFFFFFFFu : (1u << upto) - 1u) & ~(q0 >= 32 ? 0xFFFFFFFFu : (1u << q0) - 1u);
                                if (kmask & range) counted = true;  // a counted target filter scores at least 0
                                for (uint32_t cm = cmask & range; cm; cm &= cm - 1u) {
                                    const uint32_t q = __ffs(cm) - 1;
                                    const uint32_t j = c0 + q;
                                    const uint32_t tm = T.tmeta[j];
                                    const uint32_t sum = s1 + (tm & 0xFFFFu);
                                    const uint32_t cut = !fastA
                                        ? (sum < 1024 ? S.cut_sum[sum] : S.cut256[4096u / sum])
                                        : (sum < 1024 ? S.cut64_sum[sum] : S.cut64[1024u / sum]);
                                    const uint64_t fr = candidate_fraction(aw, &T.tw[0][j], S.cstage[q][tid], cut, fastA,
                                                                           min(e1, tm >> 16));
                                    const uint32_t num = (uint32_t)(fr >> 32), den = (uint32_t)fr;
                                    if ((uint64_t)num * bden > (uint64_t)bnum * den) {
                                        bnum = num;
                                        bden = den;
                                    }
                                }
                                if (!lmq) break;  // the open segment goes on in the next slice
                                lmq &= lmq - 1u;
                                q0 = qe + 1;
                                const uint32_t j = c0 + qe;
                                {
                                    const double m = row_maximum(active, bnum, bden, counted);
                                    if (split) {
                                        if (have) P.slots[P.split[U.split].slot_base + row] = m;
                                    } else {
                                        S.mv[tid][((T.tinfo[j] >> 16) & 0xFFu) % kTcRing] = m;
                                    }
                                    bnum = 0;
                                    bden = 1;
                                    counted = false;
                                    if (!split && ++pend == (uint32_t)kTcRing) {  // ring full: sum it
                                        TC_STAMP(t_fo);
                                        fold_ring(P, S, T, ring_base, pend, group, nref, nrows, U.t0, rs, tid);
                                        if (tid == 0) TC_ADD(kTcPhFold, t_fo);
                                        ring_base += pend;
                                        pend = 0;
                                    }
                                }
                            }
                            if (tid == 0) TC_ADD(kTcPhWalk, t_wk);
                        }
                        if (pend) {  // the tile's last completed targets
                            TC_STAMP(t_fo);
                            fold_ring(P, S, T, ring_base, pend, group, nref, nrows, U.t0, rs, tid);
                            if (tid == 0) TC_ADD(kTcPhFold, t_fo);
                        }
                        asm volatile("tcgen05.fence::before_thread_sync;");
                    }
                    if (tid == 0) TC_ADD(kTcPhScore, t_sc);
                    if (tid == 0) TC_ADD(kTcPhConsStep, t_step);
                }
                TC_STAMP(t_bar);
                ok = __syncthreads_and(ok);
                if (tid == 0) TC_ADD(kTcPhStepBarrier, t_bar);
                if (!ok) break;
                const bool produced = S.tile[b].produced != 0;
                if (produced) gtile++;
                pending = produced;
                if (!produced) break;  // no tile counted in this step: the pass is done
            }
        }
        if (!ok) break;
        if (!split && !group) {
            for (uint32_t k = tid; k < nT; k += kTcThreads) {
                const uint32_t tgt = P.targets[U.t0 + k];
                P.scores[out_index(P, rs != 0, U.ref, tgt)] = final_score(S.run[k], A.nfilters, S.sparse);
            }
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    if (!ok && tid == 0) {
        atomicAdd(P.error, 1u);
        // wait (bounded) for any MMA still reading shared memory or writing TMEM
        mma_commit(smem_addr(&S.mbar[4]));
        mbar_wait(smem_addr(&S.mbar[4]), 0);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kTcCols));
}

cudaError_t launch_matrix_tc(const MatParams& P, uint32_t grid, cudaStream_t st) {
    if (P.nunits == 0) return cudaSuccess;
    k_matrix_tc<<<grid, kTcThreads, kTcSmemBytes, st>>>(P);
    return cudaGetLastError();
}

int matrix_tc_ctas_per_sm() {
    cudaFuncSetAttribute(k_matrix_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmemBytes);
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_matrix_tc, kTcThreads, kTcSmemBytes);
    return n > 0 ? n : 1;
}

}  // namespace sdbfg

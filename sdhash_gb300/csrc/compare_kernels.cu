// compare_kernels.cu -- SDBF digest comparison on sm_103a.
//
// Restates sdbf_score / sdbf_max_score (sdbf/sdbf_core.cc:330-455) for a
// list of digest pairs whose orientation (the swap rule, :351-359) was fixed
// on the host:
//   for each filter i of the reference digest:
//       s1 = elements(i); s1 < 16 -> 0, else
//       max over target filters j with s2 >= 16 of
//         cut   = CUTOFFS256[4096 / (s1 + s2)]
//         match = staged AND-popcount (bf_utils.cc:114-206): 0 when after
//                 8/16/32 of the 64 words 8c+48 / 4c+48 / 2c+48 < cut
//         score = match <= cut ? 0 : (match-cut) / (min(ham_i, ham_j)-cut)
//   sum the per-filter maxima in filter order in double precision with the
//   reference's -1 sentinel, divide by the non-sparse filter count and round
//   half away from zero as boost::math::round does: floor(x + 0.5).
//
// The maximum over j is tracked exactly as the fraction (num, den) and
// turned into one IEEE division at the end: division is correctly rounded
// and monotone, so max_j fl(a_j/b_j) == fl(max_j a_j/b_j).
#include <cstdint>
#include <cuda_runtime.h>

#include "compare_device.cuh"
#include "compare_kernels.h"
#include "sdbf_device.cuh"

// Two kernels: k_compare_pairs (one CTA per listed pair: the per-call path)
// and k_matrix (the batched engine: persistent CTAs over work units of one
// reference digest against a run of targets).
//
// Per filter pair the reference computes a staged AND-popcount whose
// early exits only ever turn a count into 0, followed by
// "match <= cut -> 0".  A pair can therefore contribute a non-zero score
// only if its full 2048-bit AND-popcount exceeds the cut.  The engine
// computes the full count of every pair with a carry-save (Harley-Seal)
// adder tree -- 3-input LOP3 majority / parity over the 64 ANDed words, 8
// POPC instead of 64 -- and runs the reference's staged tests only for the
// pairs above the cut, which gives exactly the reference's value for every
// pair.

namespace sdbfg {

constexpr int kTgtTile = 32;  // target filters staged per shared-memory tile

namespace {

__device__ __forceinline__ uint32_t xor3(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

__device__ __forceinline__ uint32_t maj3(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("lop3.b32 %0, %1, %2, %3, 0xE8;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// carry-save adder: (h, l) = a + b + c bitwise
#define MAT_CSA(h, l, a, b, c)            \
    do {                                  \
        const uint32_t a_ = (a), b_ = (b), c_ = (c); \
        (h) = maj3(a_, b_, c_);           \
        (l) = xor3(a_, b_, c_);           \
    } while (0)

// popcount(a & t) over 64 words: a in registers, t in shared memory.
__device__ __forceinline__ uint32_t and_popc_hs(const uint32_t (&a)[64], const uint32_t* t) {
    const uint4* t4 = reinterpret_cast<const uint4*>(t);
    uint32_t ones = 0, twos = 0, fours = 0, eights = 0, total16 = 0;
#pragma unroll
    for (int blk = 0; blk < 4; blk++) {
        uint32_t x[16];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint4 v = t4[blk * 4 + q];
            x[4 * q + 0] = a[blk * 16 + 4 * q + 0] & v.x;
            x[4 * q + 1] = a[blk * 16 + 4 * q + 1] & v.y;
            x[4 * q + 2] = a[blk * 16 + 4 * q + 2] & v.z;
            x[4 * q + 3] = a[blk * 16 + 4 * q + 3] & v.w;
        }
        uint32_t twosA, twosB, foursA, foursB, eightsA, eightsB, sixteens;
        MAT_CSA(twosA, ones, ones, x[0], x[1]);
        MAT_CSA(twosB, ones, ones, x[2], x[3]);
        MAT_CSA(foursA, twos, twos, twosA, twosB);
        MAT_CSA(twosA, ones, ones, x[4], x[5]);
        MAT_CSA(twosB, ones, ones, x[6], x[7]);
        MAT_CSA(foursB, twos, twos, twosA, twosB);
        MAT_CSA(eightsA, fours, fours, foursA, foursB);
        MAT_CSA(twosA, ones, ones, x[8], x[9]);
        MAT_CSA(twosB, ones, ones, x[10], x[11]);
        MAT_CSA(foursA, twos, twos, twosA, twosB);
        MAT_CSA(twosA, ones, ones, x[12], x[13]);
        MAT_CSA(twosB, ones, ones, x[14], x[15]);
        MAT_CSA(foursB, twos, twos, twosA, twosB);
        MAT_CSA(eightsB, fours, fours, foursA, foursB);
        MAT_CSA(sixteens, eights, eights, eightsA, eightsB);
        total16 += __popc(sixteens);
    }
    return 16 * total16 + 8 * __popc(eights) + 4 * __popc(fours) + 2 * __popc(twos) + __popc(ones);
}

// Two independent carry-save trees: popcount(a & t0) and popcount(a & t1).
// The two dependency chains interleave, which doubles the instruction-level
// parallelism of the inner loop; a[] is read once for both.
struct HsAcc {
    uint32_t ones = 0, twos = 0, fours = 0, eights = 0, total16 = 0;
    uint32_t foursA = 0, eightsA = 0;
};

__device__ __forceinline__ void hs_quad(HsAcc& h, uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3, int q) {
    uint32_t twosA, twosB, fours_new;
    MAT_CSA(twosA, h.ones, h.ones, x0, x1);
    MAT_CSA(twosB, h.ones, h.ones, x2, x3);
    MAT_CSA(fours_new, h.twos, h.twos, twosA, twosB);
    if ((q & 1) == 0) {
        h.foursA = fours_new;
    } else {
        uint32_t eights_new;
        MAT_CSA(eights_new, h.fours, h.fours, h.foursA, fours_new);
        if ((q & 3) == 1) {
            h.eightsA = eights_new;
        } else {
            uint32_t sixteens;
            MAT_CSA(sixteens, h.eights, h.eights, h.eightsA, eights_new);
            h.total16 += __popc(sixteens);
        }
    }
}

__device__ __forceinline__ uint32_t hs_total(const HsAcc& h) {
    return 16 * h.total16 + 8 * __popc(h.eights) + 4 * __popc(h.fours) + 2 * __popc(h.twos) + __popc(h.ones);
}

__device__ __forceinline__ void and_popc_hs2(const uint32_t (&a)[64], const uint32_t* t0, const uint32_t* t1,
                                             uint32_t& c0, uint32_t& c1) {
    const uint4* u0 = reinterpret_cast<const uint4*>(t0);
    const uint4* u1 = reinterpret_cast<const uint4*>(t1);
    HsAcc h0, h1;
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const uint4 v0 = u0[q], v1 = u1[q];
        hs_quad(h0, a[4 * q] & v0.x, a[4 * q + 1] & v0.y, a[4 * q + 2] & v0.z, a[4 * q + 3] & v0.w, q);
        hs_quad(h1, a[4 * q] & v1.x, a[4 * q + 1] & v1.y, a[4 * q + 2] & v1.z, a[4 * q + 3] & v1.w, q);
    }
    c0 = hs_total(h0);
    c1 = hs_total(h1);
}

// The reference's staged exits (bf_utils.cc:114-206) for a pair whose full
// count is above the cut: true when an early stage would have returned 0.
__device__ __forceinline__ bool staged_exit(const uint32_t (&a)[64], const uint32_t* t, uint32_t cut) {
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < 8; w++) c += __popc(a[w] & t[w]);
    if (8 * c + 48 < cut) return true;
#pragma unroll
    for (int w = 8; w < 16; w++) c += __popc(a[w] & t[w]);
    if (4 * c + 48 < cut) return true;
#pragma unroll
    for (int w = 16; w < 32; w++) c += __popc(a[w] & t[w]);
    return 2 * c + 48 < cut;
}

// popcount(a & t) over the first 16 words (64 bytes) for two targets, and
// the 8-word partial counts for the fast-mode stage test.
__device__ __forceinline__ void and_popc_16x2(const uint32_t (&a)[64], const uint32_t* t0, const uint32_t* t1,
                                              uint32_t& h0, uint32_t& f0, uint32_t& h1, uint32_t& f1) {
    const uint4* u0 = reinterpret_cast<const uint4*>(t0);
    const uint4* u1 = reinterpret_cast<const uint4*>(t1);
    uint32_t c0 = 0, c1 = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const uint4 v0 = u0[q], v1 = u1[q];
        c0 += __popc(a[4 * q] & v0.x) + __popc(a[4 * q + 1] & v0.y) + __popc(a[4 * q + 2] & v0.z) +
              __popc(a[4 * q + 3] & v0.w);
        c1 += __popc(a[4 * q] & v1.x) + __popc(a[4 * q + 1] & v1.y) + __popc(a[4 * q + 2] & v1.z) +
              __popc(a[4 * q + 3] & v1.w);
        if (q == 1) {
            h0 = c0;
            h1 = c1;
        }
    }
    f0 = c0;
    f1 = c1;
}

}  // namespace

__global__ void __launch_bounds__(kCmpThreads) k_compare_pairs(CmpParams P) {
    __shared__ __align__(16) uint32_t tf[kTgtTile][64];
    __shared__ uint32_t tmeta[kTgtTile];
    __shared__ uint16_t cut_tab[SDBF_CUTOFF_BINS], cut64_tab[SDBF_CUTOFF_BINS];
    __shared__ double msc[kCmpThreads];
    __shared__ uint32_t sparse_flag[kCmpThreads];
    for (uint32_t i = threadIdx.x; i < SDBF_CUTOFF_BINS; i += blockDim.x) {
        cut_tab[i] = P.cutoffs[i];
        cut64_tab[i] = P.cutoffs64[i];
    }
    __syncthreads();
    for (uint64_t pr = blockIdx.x; pr < P.npairs; pr += gridDim.x) {
        const CmpPair pair = P.pairs[pr];
        const uint32_t sa = pair.sides & 1u, sb = (pair.sides >> 1) & 1u;
        const CmpDigest A = P.digests[sa][pair.ref];
        const CmpDigest B = P.digests[sb][pair.tgt];
        const uint32_t* __restrict__ fa = P.filters[sa];
        const uint32_t* __restrict__ fb = P.filters[sb];
        const uint32_t* __restrict__ ma = P.meta[sa];
        const uint32_t* __restrict__ mb = P.meta[sb];
        const uint32_t n1 = pair.n1;  // filters of A used (== A.nfilters, sampling not applied here)
        const bool fastA = (A.flags & kDigestFast) != 0;  // the reference digest's fastmode decides
        double sum = -1.0;
        uint32_t sparse = 0;
        for (uint32_t c0 = 0; c0 < n1; c0 += blockDim.x) {
            const uint32_t i = c0 + threadIdx.x;
            const bool have = i < n1;
            uint32_t a[64];
            uint32_t s1 = 0, e1 = 0;
            if (have) {
                const uint32_t meta = ma[A.first + i];
                s1 = meta & 0xFFFFu;
                e1 = meta >> 16;
                const uint4* src = reinterpret_cast<const uint4*>(fa + (size_t)(A.first + i) * 64);
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const uint4 v = __ldg(src + q);
                    a[4 * q] = v.x; a[4 * q + 1] = v.y; a[4 * q + 2] = v.z; a[4 * q + 3] = v.w;
                }
            }
            const bool active = have && s1 >= (uint32_t)kMinElem;
            // best = num/den; counted: a target filter with >= 16 elements was seen
            uint32_t bnum = 0, bden = 1;
            bool counted = false;
            for (uint32_t j0 = 0; j0 < B.nfilters; j0 += kTgtTile) {
                const uint32_t nt = min((uint32_t)kTgtTile, B.nfilters - j0);
                __syncthreads();
                {
                    const uint4* src = reinterpret_cast<const uint4*>(fb + (size_t)(B.first + j0) * 64);
                    uint4* dst = reinterpret_cast<uint4*>(&tf[0][0]);
                    for (uint32_t q = threadIdx.x; q < nt * 16; q += blockDim.x) dst[q] = __ldg(src + q);
                    for (uint32_t q = threadIdx.x; q < nt; q += blockDim.x) tmeta[q] = mb[B.first + j0 + q];
                }
                __syncthreads();
                if (active) {
                    for (uint32_t j = 0; j < nt; j++) {
                        const uint32_t meta = tmeta[j];
                        const uint32_t s2 = meta & 0xFFFFu;
                        if (s2 < (uint32_t)kMinElem) continue;
                        const uint32_t e2 = meta >> 16;
                        const uint32_t max_est = min(e1, e2);
                        uint32_t cut, match;
                        if (!fastA) {
                            cut = cut_tab[4096u / (s1 + s2)];
                            match = and_popc_hs(a, &tf[j][0]);
                            if (match > cut && staged_exit(a, &tf[j][0], cut)) match = 0;
                        } else {  // bf_bitcount_cut_64 (bf_utils.cc:78-110) on the folded 64 bytes
                            cut = cut64_tab[1024u / (s1 + s2)];
                            uint32_t h8, h16, u8, u16;
                            and_popc_16x2(a, &tf[j][0], &tf[j][0], h8, h16, u8, u16);
                            match = (2 * h8 + 48 < cut) ? 0u : h16;
                        }
                        uint32_t num = 0, den = 1;
                        if (match > cut) {
                            num = match - cut;
                            den = max_est - cut;  // uint32 as in the reference
                        }
                        if (!counted || (uint64_t)num * bden > (uint64_t)bnum * den) {
                            bnum = num;
                            bden = den;
                            counted = true;
                        }
                    }
                }
            }
            if (have) {
                msc[threadIdx.x] = max_value(active, bnum, bden, counted);
                sparse_flag[threadIdx.x] = s1 < (uint32_t)kMinElem;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                const uint32_t lim = min((uint32_t)blockDim.x, n1 - c0);
                for (uint32_t q = 0; q < lim; q++) {
                    const double m = msc[q];
                    sum = (sum < 0) ? m : __dadd_rn(sum, m);
                    sparse += sparse_flag[q];
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            uint64_t denom = n1;
            if (n1 > 1) denom -= sparse;
            int32_t score;
            if (denom == 0 || sum < 0) score = -1;
            else score = (int32_t)floor(__dadd_rn(__ddiv_rn(__dmul_rn(100.0, sum), (double)denom), 0.5));
            P.scores[pr] = score;
        }
    }
}

// One warp per filter: 16 lanes fold words k, k+16, k+32, k+48 into word k
// (bloom_filter::fold(2), bloom_filter.cc:262-288: two halvings by OR),
// write the folded 64 bytes over the first 64, and the hamming weight of
// the folded filter goes into the meta word (sdbf::fast, sdbf_class.cc:425-439).
__global__ void k_fold(uint32_t* __restrict__ filters, uint32_t* __restrict__ meta, CmpDigest* digests,
                       uint32_t first, uint32_t count) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t f0 = digests[first].first;
    const uint32_t f1 = digests[first + count - 1].first + digests[first + count - 1].nfilters;
    for (uint32_t f = f0 + warp; f < f1; f += nwarps) {
        uint32_t* w = filters + (size_t)f * 64;
        uint32_t v = 0;
        if (lane < 16) v = w[lane] | w[lane + 16] | w[lane + 32] | w[lane + 48];
        __syncwarp();
        if (lane < 16) w[lane] = v;
        uint32_t h = __popc(v);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) h += __shfl_xor_sync(0xffffffffu, h, d);
        if (lane == 0) meta[f] = (h << 16) | (meta[f] & 0xFFFFu);
    }
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t d = gt; d < count; d += gridDim.x * blockDim.x) digests[first + d].flags |= kDigestFast;
}

cudaError_t launch_fold(uint32_t* filters, uint32_t* meta, CmpDigest* digests, uint32_t first, uint32_t count,
                        cudaStream_t st) {
    if (count) k_fold<<<512, 256, 0, st>>>(filters, meta, digests, first, count);
    return cudaGetLastError();
}

cudaError_t launch_compare_pairs(const CmpParams& P, uint32_t grid, cudaStream_t st) {
    if (P.npairs) k_compare_pairs<<<grid, kCmpThreads, 0, st>>>(P);
    return cudaGetLastError();
}

}  // namespace sdbfg

// ---------------------------------------------------------- matrix engine
namespace sdbfg {

const MatVariant kMatVariantTable[kMatVariants] = {{128, 32}, {128, 16}, {128, 64}, {64, 32}, {256, 32}, {128, 256}};

template <int R, int TJ>
struct MatSmem {
    uint32_t tf[TJ][64];          // target filters of the current tile
    uint32_t tmeta[TJ];
    uint32_t tinfo[TJ];           // local target index | completion index << 16 | last << 31
    uint32_t gidx[TJ];            // global filter index per slot
    uint32_t comp[TJ];            // local target index of the k-th completed target
    double mv[R][TJ + 1];         // per row and completed target: the filter's maximum
    double run[kMatMaxTargets];   // running sums per target of the unit (multi-pass units)
    uint32_t gref[R];             // group units: reference digest ids,
    uint32_t gstart[R + 1];       //   first row of each,
    uint32_t gsparse[R];          //   and its count of sparse filters
    uint16_t cut_sum[1024];       // CUTOFFS256[4096 / (s1 + s2)] by s1 + s2
    uint16_t cut64_sum[1024];     // CUTOFFS64[1024 / (s1 + s2)] by s1 + s2
    uint16_t cut256[SDBF_CUTOFF_BINS];
    uint16_t cut64[SDBF_CUTOFF_BINS];
    uint32_t seg_first[32], seg_start[33], seg_te[32];  // tile composition: one segment per target
    MatUnit unit;
    uint32_t unit_id, ntile, ncomp, cur_t, cur_f, sparse, nseg, last_open;
};

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

template <int R, int TJ>
__global__ void __launch_bounds__(R, 512 / R) k_matrix(MatParams P) {
    extern __shared__ __align__(16) uint8_t mat_smem[];
    MatSmem<R, TJ>& S = *reinterpret_cast<MatSmem<R, TJ>*>(mat_smem);
    const uint32_t tid = threadIdx.x, lane = tid & 31;
    for (uint32_t i = tid; i < 1024; i += R) {
        S.cut_sum[i] = P.cutoffs[i >= 32 ? 4096u / i : (uint32_t)SDBF_CUTOFF_BINS - 1];
        S.cut64_sum[i] = P.cutoffs64[i >= 8 ? 1024u / i : (uint32_t)SDBF_CUTOFF_BINS - 1];
    }
    for (uint32_t i = tid; i < SDBF_CUTOFF_BINS; i += R) {
        S.cut256[i] = P.cutoffs[i];
        S.cut64[i] = P.cutoffs64[i];
    }
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
            // reference digests of the group and their first rows (warp 0)
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
            for (uint32_t k = tid; k < nT && !split; k += R) S.run[k] = -1.0;
        }
        if (tid == 0) S.sparse = 0;
        __syncthreads();
        const CmpDigest A = P.digests[rs][group ? S.gref[0] : U.ref];
        const bool fastA = (A.flags & kDigestFast) != 0;  // the reference digest's fastmode decides
        for (uint32_t rc = U.r0; rc < U.r1; rc += R) {
            const uint32_t row = rc + tid;
            const bool have = row < U.r1;
            uint32_t a[64];
            uint32_t s1 = 0, e1 = 0;
            uint32_t gk = 0;  // group units: this row's digest in the group
            uint32_t fidx = A.first + row;
            if (group && have) {
                uint32_t lo = 0, hi = nref;  // largest k with gstart[k] <= row
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
                const uint4* src = reinterpret_cast<const uint4*>(P.filters[rs] + (size_t)fidx * 64);
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const uint4 v = __ldg(src + q);
                    a[4 * q] = v.x; a[4 * q + 1] = v.y; a[4 * q + 2] = v.z; a[4 * q + 3] = v.w;
                }
            } else {
#pragma unroll
                for (int q = 0; q < 64; q++) a[q] = 0;
            }
            const bool active = have && s1 >= (uint32_t)kMinElem;
            if (group && have && !active) atomicAdd(&S.gsparse[gk], 1u);
            const uint32_t nsparse = __syncthreads_count(have && !active);
            if (tid == 0) {
                S.sparse += nsparse;
                S.cur_t = 0;
                S.cur_f = 0;
            }
            uint32_t bnum = 0, bden = 1;  // best fraction so far
            bool counted = false;          // a target filter with >= 16 elements was seen
            const uint32_t nrows = min((uint32_t)R, U.r1 - rc);
            __syncthreads();
            for (;;) {
                const bool more = S.cur_t < nT;
                __syncthreads();  // every thread has read the cursor before warp 0 moves it
                if (!more) break;
                // ---- tile composition (warp 0): targets cur_t.. fill TJ slots in order
                if (tid < 32) {
                    const uint32_t te = S.cur_t + lane;
                    const uint32_t f0 = lane == 0 ? S.cur_f : 0;
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
                    const uint32_t excl = incl - rem;
                    const bool done_here = rem > 0 && incl <= (uint32_t)TJ;
                    // segment of this lane's target (slots are filled by all threads below)
                    const bool has = rem > 0 && excl < (uint32_t)TJ;
                    if (has) {
                        S.seg_first[lane] = first;
                        S.seg_start[lane] = excl;
                        S.seg_te[lane] = te;
                    }
                    if (done_here) S.comp[lane] = te;
                    const uint32_t done_mask = __ballot_sync(0xffffffffu, done_here);
                    const uint32_t has_mask = __ballot_sync(0xffffffffu, has);
                    const uint32_t over_mask = __ballot_sync(0xffffffffu, rem > 0 && incl > (uint32_t)TJ);
                    const uint32_t open_mask = __ballot_sync(0xffffffffu, has && incl > (uint32_t)TJ);
                    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                    if (lane == 0) {
                        S.ncomp = __popc(done_mask);
                        S.ntile = min(total, (uint32_t)TJ);
                        S.nseg = __popc(has_mask);
                        S.seg_start[__popc(has_mask)] = min(total, (uint32_t)TJ);
                        S.last_open = open_mask != 0;  // the last segment continues in the next tile
                    }
                    // cursor update: first lane whose target does not fit
                    const uint32_t l = over_mask ? (uint32_t)(__ffs(over_mask) - 1) : 32u;
                    const uint32_t ex_l = __shfl_sync(0xffffffffu, excl, l & 31);
                    const uint32_t f0_l = __shfl_sync(0xffffffffu, f0, l & 31);
                    if (lane == 0) {
                        if (l < 32) {
                            S.cur_t += l;
                            S.cur_f = f0_l + ((uint32_t)TJ - ex_l);
                        } else {
                            S.cur_t = min(S.cur_t + 32u, nT);
                            S.cur_f = 0;
                        }
                    }
                }
                __syncthreads();
                // ---- slots of the tile, filled in parallel
                {
                    const uint32_t nseg = S.nseg;
                    for (uint32_t j = tid; j < S.ntile; j += R) {
                        const uint32_t k = find_segment(S.seg_start, nseg, j);
                        const uint32_t f = S.seg_first[k] + (j - S.seg_start[k]);
                        const bool last = j + 1 == S.seg_start[k + 1] && !(k + 1 == nseg && S.last_open);
                        S.gidx[j] = f;
                        S.tmeta[j] = P.meta[ts][f];
                        S.tinfo[j] = S.seg_te[k] | (k << 16) | (last ? 0x80000000u : 0u);
                    }
                }
                __syncthreads();
                // ---- target filters -> shared memory
                const uint32_t nt = S.ntile;
                for (uint32_t q = tid; q < nt * 16; q += R) {
                    const uint4* src = reinterpret_cast<const uint4*>(P.filters[ts] + (size_t)S.gidx[q >> 4] * 64);
                    reinterpret_cast<uint4*>(&S.tf[q >> 4][0])[q & 15] = __ldg(src + (q & 15));
                }
                __syncthreads();
                // ---- every row against the tile, two target filters at a time
                // consume(j, count, h8): count = full 2048-bit count (normal mode) or
                // the 64-byte count (fast mode, h8 = its first 32 bytes)
                auto consume = [&](uint32_t j, uint32_t cnt, uint32_t h8) {
                    const uint32_t tm = S.tmeta[j];
                    const uint32_t s2 = tm & 0xFFFFu;
                    if (active && s2 >= (uint32_t)kMinElem) {
                        uint32_t cut, match = cnt;
                        if (!fastA) {
                            cut = cut_for(S.cut_sum, S.cut256, s1, s2);
                            if (match > cut && staged_exit(a, &S.tf[j][0], cut)) match = 0;
                        } else {
                            const uint32_t sum = s1 + s2;
                            cut = sum < 1024 ? S.cut64_sum[sum] : S.cut64[1024u / sum];
                            if (2 * h8 + 48 < cut) match = 0;
                        }
                        uint32_t num = 0, den = 1;
                        if (match > cut) {
                            num = match - cut;
                            den = min(e1, tm >> 16) - cut;  // uint32 as in the reference
                        }
                        if (!counted || (uint64_t)num * bden > (uint64_t)bnum * den) {
                            bnum = num;
                            bden = den;
                            counted = true;
                        }
                    }
                    const uint32_t info = S.tinfo[j];
                    if (info & 0x80000000u) {
                        const double m = max_value(active, bnum, bden, counted);
                        if (split) {
                            if (have) P.slots[P.split[U.split].slot_base + row] = m;
                        } else {
                            S.mv[tid][(info >> 16) & 0x7FFFu] = m;
                        }
                        bnum = 0;
                        bden = 1;
                        counted = false;
                    }
                };
                uint32_t j = 0;
                if (!fastA) {
                    for (; j + 1 < nt; j += 2) {
                        uint32_t m0 = 0, m1 = 0;
                        if (active) and_popc_hs2(a, &S.tf[j][0], &S.tf[j + 1][0], m0, m1);
                        consume(j, m0, 0);
                        consume(j + 1, m1, 0);
                    }
                    if (j < nt) consume(j, active ? and_popc_hs(a, &S.tf[j][0]) : 0u, 0);
                } else {
                    for (; j < nt; j += 2) {
                        const uint32_t j1 = j + 1 < nt ? j + 1 : j;
                        uint32_t h0 = 0, f0 = 0, h1 = 0, f1 = 0;
                        if (active) and_popc_16x2(a, &S.tf[j][0], &S.tf[j1][0], h0, f0, h1, f1);
                        consume(j, f0, h0);
                        if (j + 1 < nt) consume(j + 1, f1, h1);
                    }
                }
                __syncthreads();
                // ---- fold the completed targets' maxima in filter order
                if (group) {  // every (reference, completed target) pair is finished here
                    const uint32_t ncomp = S.ncomp;
                    for (uint32_t t = tid; t < ncomp * nref; t += R) {
                        const uint32_t k = t % nref, col = t / nref;
                        double sum = -1.0;
                        for (uint32_t r = S.gstart[k]; r < S.gstart[k + 1]; r++) {
                            const double m = S.mv[r][col];
                            if (sum < 0) sum = m;
                            else if (m != 0.0) sum = __dadd_rn(sum, m);
                        }
                        const uint32_t tgt = P.targets[U.t0 + S.comp[col]];
                        P.scores[out_index(P, rs != 0, S.gref[k], tgt)] =
                            final_score(sum, S.gstart[k + 1] - S.gstart[k], S.gsparse[k]);
                    }
                } else if (!split) {
                    for (uint32_t k = tid; k < S.ncomp; k += R) {
                        double sum = S.run[S.comp[k]];
                        for (uint32_t r = 0; r < nrows; r++) {
                            const double m = S.mv[r][k];
                            if (sum < 0) sum = m;
                            else if (m != 0.0) sum = __dadd_rn(sum, m);
                        }
                        S.run[S.comp[k]] = sum;
                    }
                }
                __syncthreads();
            }
        }
        if (!split && !group) {
            for (uint32_t k = tid; k < nT; k += R) {
                const uint32_t tgt = P.targets[U.t0 + k];
                P.scores[out_index(P, rs != 0, U.ref, tgt)] = final_score(S.run[k], A.nfilters, S.sparse);
            }
        }
    }
}

// One thread per split pair: the ordered sum over the reference's filters.
__global__ void k_matrix_finalize(MatParams P) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nsplit) return;
    const MatSplit sp = P.split[i];
    const uint32_t rs = sp.flags & kUnitRefSide1 ? 1 : 0;
    const CmpDigest A = P.digests[rs][sp.ref];
    double sum = -1.0;
    uint32_t sparse = 0;
    for (uint32_t r = 0; r < A.nfilters; r++) {
        const double m = P.slots[sp.slot_base + r];
        sum = sum < 0 ? m : __dadd_rn(sum, m);
        sparse += (P.meta[rs][A.first + r] & 0xFFFFu) < (uint32_t)kMinElem;
    }
    P.scores[out_index(P, rs != 0, sp.ref, sp.tgt)] = final_score(sum, A.nfilters, sparse);
}

// The dynamic shared-memory attribute is set by matrix_ctas_per_sm, which
// callers run before the first launch (and before any stream capture).
template <int R, int TJ>
static cudaError_t launch_variant(const MatParams& P, uint32_t grid, cudaStream_t st) {
    k_matrix<R, TJ><<<grid, R, sizeof(MatSmem<R, TJ>), st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_matrix(const MatParams& P, int variant, uint32_t grid, cudaStream_t st) {
    if (P.nunits == 0) return cudaSuccess;
    switch (variant) {
        case 0: return launch_variant<128, 32>(P, grid, st);
        case 1: return launch_variant<128, 16>(P, grid, st);
        case 2: return launch_variant<128, 64>(P, grid, st);
        case 3: return launch_variant<64, 32>(P, grid, st);
        case 4: return launch_variant<256, 32>(P, grid, st);
        case kMatVariantTc: return launch_matrix_tc(P, grid, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_matrix_finalize(const MatParams& P, cudaStream_t st) {
    if (P.nsplit) k_matrix_finalize<<<(P.nsplit + 127) / 128, 128, 0, st>>>(P);
    return cudaGetLastError();
}

template <int R, int TJ>
static int occupancy() {
    int n = 0;
    cudaFuncSetAttribute(k_matrix<R, TJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MatSmem<R, TJ>));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_matrix<R, TJ>, R, sizeof(MatSmem<R, TJ>));
    return n > 0 ? n : 1;
}

int matrix_ctas_per_sm(int variant) {
    static int cached[kMatVariants] = {0, 0, 0, 0, 0, 0};
    if (variant >= 0 && variant < kMatVariants && cached[variant]) return cached[variant];
    int n = 1;
    switch (variant) {
        case 0: n = occupancy<128, 32>(); break;
        case 1: n = occupancy<128, 16>(); break;
        case 2: n = occupancy<128, 64>(); break;
        case 3: n = occupancy<64, 32>(); break;
        case 4: n = occupancy<256, 32>(); break;
        case kMatVariantTc: n = matrix_tc_ctas_per_sm(); break;
        default: return 1;
    }
    cached[variant] = n;
    return n;
}

}  // namespace sdbfg

// ------------------------------------------------------ threshold matches
// Scores >= threshold compacted in pair order into (i, j, score) triples:
// per 1024-score block a count, one exclusive scan over the block counts,
// then each block writes its matches at its offset (order preserving).
namespace sdbfg {

constexpr uint32_t kMatchBlock = 1024;  // scores per block, 256 threads x 4

__global__ void __launch_bounds__(256) k_match_count(const int32_t* __restrict__ scores, uint64_t n, int32_t thr,
                                                     uint32_t* __restrict__ counts) {
    const uint64_t b = blockIdx.x;
    const uint64_t base = b * kMatchBlock + threadIdx.x * 4;
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) c += (base + k < n) && scores[base + k] >= thr;
    __shared__ uint32_t part[8];
    uint32_t w = c;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) w += __shfl_xor_sync(0xffffffffu, w, d);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int k = 0; k < 8; k++) s += part[k];
        counts[b] = s;
    }
}

// single CTA: counts[] -> exclusive offsets (u64), total in offs[nb]
__global__ void __launch_bounds__(1024) k_match_scan(const uint32_t* __restrict__ counts, uint64_t nb,
                                                     uint64_t* __restrict__ offs) {
    __shared__ uint64_t part[1024];
    const uint64_t per = (nb + 1023) / 1024;
    const uint64_t b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
    uint64_t s = 0;
    for (uint64_t b = b0; b < b1; b++) s += counts[b];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        const uint64_t v = threadIdx.x >= (uint32_t)d ? part[threadIdx.x - d] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint64_t run = part[threadIdx.x] - s;
    for (uint64_t b = b0; b < b1; b++) {
        offs[b] = run;
        run += counts[b];
    }
    if (threadIdx.x == 1023) offs[nb] = part[1023];
}

__device__ __forceinline__ void pair_of(uint64_t k, uint32_t mode, uint64_t n, uint32_t& i, uint32_t& j) {
    if (mode == kMatModeCross) {
        i = (uint32_t)(k / n);
        j = (uint32_t)(k % n);
        return;
    }
    // row i of the upper triangle: start(i) = i*(2n-i-1)/2 <= k < start(i+1)
    const double nn = (double)n;
    double r = floor(((2.0 * nn - 1.0) - sqrt((2.0 * nn - 1.0) * (2.0 * nn - 1.0) - 8.0 * (double)k)) / 2.0);
    uint64_t ii = r < 0 ? 0 : (uint64_t)r;
    auto start = [&](uint64_t x) { return x * (2 * n - x - 1) / 2; };
    while (ii > 0 && start(ii) > k) ii--;
    while (ii + 1 < n && start(ii + 1) <= k) ii++;
    i = (uint32_t)ii;
    j = (uint32_t)(k - start(ii) + ii + 1);
}

__global__ void __launch_bounds__(256) k_match_write(const int32_t* __restrict__ scores, uint64_t n, int32_t thr,
                                                     const uint64_t* __restrict__ offs, uint32_t mode,
                                                     uint64_t dim, uint32_t* __restrict__ out, uint64_t cap) {
    __shared__ uint32_t warp_base[8];
    const uint64_t b = blockIdx.x;
    const uint64_t base = b * kMatchBlock + threadIdx.x * 4;
    bool hit[4];
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        hit[k] = (base + k < n) && scores[base + k] >= thr;
        c += hit[k];
    }
    // exclusive prefix of c over the block (thread order == score order)
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (uint32_t)d) incl += v;
    }
    if (lane == 31) warp_base[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int k = 0; k < 8; k++) {
            const uint32_t v = warp_base[k];
            warp_base[k] = s;
            s += v;
        }
    }
    __syncthreads();
    uint64_t pos = offs[b] + warp_base[warp] + incl - c;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!hit[k]) continue;
        if (pos < cap) {
            uint32_t i, j;
            pair_of(base + k, mode, dim, i, j);
            out[3 * pos] = i;
            out[3 * pos + 1] = j;
            out[3 * pos + 2] = (uint32_t)scores[base + k];
        }
        pos++;
    }
}

cudaError_t launch_match_count(const int32_t* scores, uint64_t n, int32_t thr, uint32_t* counts, cudaStream_t st) {
    const uint64_t nb = (n + kMatchBlock - 1) / kMatchBlock;
    if (nb) k_match_count<<<(uint32_t)nb, 256, 0, st>>>(scores, n, thr, counts);
    return cudaGetLastError();
}

cudaError_t launch_match_scan(const uint32_t* counts, uint64_t nb, uint64_t* offs, cudaStream_t st) {
    k_match_scan<<<1, 1024, 0, st>>>(counts, nb, offs);
    return cudaGetLastError();
}

cudaError_t launch_match_write(const int32_t* scores, uint64_t n, int32_t thr, const uint64_t* offs, uint32_t mode,
                               uint64_t dim, uint32_t* out, uint64_t cap, cudaStream_t st) {
    const uint64_t nb = (n + kMatchBlock - 1) / kMatchBlock;
    if (nb) k_match_write<<<(uint32_t)nb, 256, 0, st>>>(scores, n, thr, offs, mode, dim, out, cap);
    return cudaGetLastError();
}

}  // namespace sdbfg

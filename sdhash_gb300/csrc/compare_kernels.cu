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

#include "compare_kernels.h"
#include "sdbf_device.cuh"

namespace sdbfg {

constexpr int kTgtTile = 32;  // target filters staged per shared-memory tile

__device__ __forceinline__ uint32_t popc_and(const uint32_t (&a)[64], const uint4* t, int w0, int w1) {
    uint32_t c = 0;
#pragma unroll
    for (int q = w0 / 4; q < w1 / 4; q++) {
        const uint4 v = t[q];
        c += __popc(a[4 * q] & v.x) + __popc(a[4 * q + 1] & v.y);
        c += __popc(a[4 * q + 2] & v.z) + __popc(a[4 * q + 3] & v.w);
    }
    return c;
}

__global__ void __launch_bounds__(kCmpThreads) k_compare_pairs(CmpParams P) {
    __shared__ __align__(16) uint32_t tf[kTgtTile][64];
    __shared__ uint32_t tmeta[kTgtTile];
    __shared__ uint16_t cut_tab[SDBF_CUTOFF_BINS];
    __shared__ double msc[kCmpThreads];
    __shared__ uint32_t sparse_flag[kCmpThreads];
    for (uint32_t i = threadIdx.x; i < SDBF_CUTOFF_BINS; i += blockDim.x) cut_tab[i] = P.cutoffs[i];
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
            // best = num/den; den == 0 means "no target counted yet" (-1)
            uint32_t bnum = 0, bden = 0;
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
                        const uint32_t cut = cut_tab[4096u / (s1 + s2)];
                        const uint4* t = reinterpret_cast<const uint4*>(&tf[j][0]);
                        uint32_t c = popc_and(a, t, 0, 8);
                        uint32_t match = 0;
                        if (!(8 * c + 48 < cut)) {
                            c += popc_and(a, t, 8, 16);
                            if (!(4 * c + 48 < cut)) {
                                c += popc_and(a, t, 16, 32);
                                if (!(2 * c + 48 < cut)) {
                                    c += popc_and(a, t, 32, 64);
                                    match = c;
                                }
                            }
                        }
                        uint32_t num, den;
                        if (match <= cut) {
                            num = 0;
                            den = 1;
                        } else {
                            num = match - cut;
                            den = max_est - cut;
                        }
                        if (bden == 0 || (uint64_t)num * bden > (uint64_t)bnum * den) {
                            bnum = num;
                            bden = den;
                        }
                    }
                }
            }
            if (have) {
                double m;
                if (!active) m = 0.0;
                else if (bden == 0) m = -1.0;
                else m = __ddiv_rn((double)bnum, (double)bden);
                msc[threadIdx.x] = m;
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

cudaError_t launch_compare_pairs(const CmpParams& P, uint32_t grid, cudaStream_t st) {
    if (P.npairs) k_compare_pairs<<<grid, kCmpThreads, 0, st>>>(P);
    return cudaGetLastError();
}

}  // namespace sdbfg

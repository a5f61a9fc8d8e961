// compare_device.cuh -- device helpers shared by the comparison kernels
// (compare_kernels.cu: CUDA-core paths, matrix_tc.cu: tensor-core path).
#pragma once
#include <cstdint>

#include "compare_kernels.h"

namespace sdbfg {

__device__ __forceinline__ uint32_t cut_for(const uint16_t* cut_sum, const uint16_t* cut256, uint32_t s1,
                                            uint32_t s2) {
    const uint32_t sum = s1 + s2;
    return sum < 1024 ? cut_sum[sum] : cut256[4096u / sum];
}

// A filter's maximum against one target as the reference's double:
// -1 when no target filter has >= 16 elements, else num / den (den is the
// reference's uint32 max_est - cut, which wraps when the hamming weights do
// not describe the compared bits -- mixed --fast comparisons).
__device__ __forceinline__ double max_value(bool active, uint32_t bnum, uint32_t bden, bool counted) {
    if (!active) return 0.0;
    if (!counted) return -1.0;
    return bnum == 0 ? 0.0 : __ddiv_rn((double)bnum, (double)bden);
}

__device__ __forceinline__ uint64_t out_index(const MatParams& P, bool ref_side1, uint32_t ref, uint32_t tgt) {
    if (P.mode == kMatModeAll) {
        const uint64_t i = min(ref, tgt), j = max(ref, tgt);
        return i * (2ull * P.n - i - 1) / 2 + (j - i - 1);
    }
    const uint64_t q = ref_side1 ? tgt : ref, t = ref_side1 ? ref : tgt;
    return q * P.n + t;
}

__device__ __forceinline__ int32_t final_score(double sum, uint32_t n1, uint32_t sparse) {
    uint64_t denom = n1;
    if (n1 > 1) denom -= sparse;
    if (denom == 0 || sum < 0) return -1;
    return (int32_t)floor(__dadd_rn(__ddiv_rn(__dmul_rn(100.0, sum), (double)denom), 0.5));
}


}  // namespace sdbfg

// compare_kernels.h -- descriptors for the digest comparison kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sdbfg {

constexpr int kCmpThreads = 128;

// A digest resident on the device: filters [first, first+nfilters) of the
// set's filter array; meta[f] = (hamming << 16) | element count.
struct CmpDigest {
    uint32_t first;
    uint32_t nfilters;
};

// One scored pair after the swap rule: `ref` is the side whose filters are
// summed (sdbf_1 after the swap in sdbf_core.cc:351-359).
struct CmpPair {
    uint32_t ref;
    uint32_t tgt;
    uint32_t n1;     // filters of ref that are scored
    uint32_t sides;  // bit0: ref lives in set 1, bit1: tgt lives in set 1
};

// Two device-resident digest sets (they may be the same set).
struct CmpParams {
    const uint32_t* filters[2];   // 64 words per filter
    const uint32_t* meta[2];      // per filter
    const CmpDigest* digests[2];
    const CmpPair* pairs;
    uint64_t npairs;
    int32_t* scores;           // per pair
    const uint16_t* cutoffs;   // CUTOFFS256
};

cudaError_t launch_compare_pairs(const CmpParams& P, uint32_t grid, cudaStream_t st);

}  // namespace sdbfg

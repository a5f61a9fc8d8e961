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
    uint32_t flags;  // kDigestFast: filters folded to 64 bytes (sdbf::fast)
};
constexpr uint32_t kDigestFast = 1u;

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
    const uint16_t* cutoffs64; // CUTOFFS64 (fast mode)
};

cudaError_t launch_compare_pairs(const CmpParams& P, uint32_t grid, cudaStream_t st);
// sdbf::fast on digests [first, first+count) of a set: fold every filter's
// 256 bytes into its first 64 (the other bytes unchanged), hamming of the
// folded bytes, fast flag on.
cudaError_t launch_fold(uint32_t* filters, uint32_t* meta, CmpDigest* digests, uint32_t first, uint32_t count,
                        cudaStream_t st);

}  // namespace sdbfg

// ------------------------------------------------------------------------
// Batched comparison ("filter matrix" engine): one persistent launch scores
// many digest pairs.  Work is cut into units: one reference digest (the side
// whose filters are summed after the swap rule) against a run of target
// digests from a target list, or -- for a single pair too large for one unit --
// a row range of the reference digest against one target ("split" unit, its
// per-filter maxima go to a slot array and k_matrix_finalize sums them).
namespace sdbfg {

constexpr uint32_t kMatMaxTargets = 512;  // targets per unit (running sums in shared memory)

enum : uint32_t { kMatModeAll = 0, kMatModeCross = 1 };
enum : uint32_t { kUnitRefSide1 = 1u, kUnitTgtSide1 = 2u, kUnitSplit = 4u, kUnitGroup = 8u };

// Three kinds of unit:
//  * group (kUnitGroup): nref reference digests listed at refs[ref ..
//    ref+nref), all their filters together fit one pass of the CTA's rows;
//    every (reference, target) score is finished inside the unit;
//  * multi-pass: one reference digest with more filters than the CTA has
//    rows (ref = digest id, rows [r0, r1) = all its filters), running sums
//    per target in shared memory;
//  * split (kUnitSplit): rows [r0, r1) of one reference digest against one
//    target; maxima to the slot array, summed by k_matrix_finalize.
struct MatUnit {
    uint32_t ref;     // digest id, or (group) position in MatParams::refs
    uint32_t r0, r1;  // rows [r0, r1) (group: 0 .. total filters of its digests)
    uint32_t t0, t1;  // target list entries [t0, t1); one entry for split units
    uint32_t flags;
    uint32_t split;   // split units: index into MatParams::split
    uint32_t nref;    // group units: digests in the group
};

struct MatSplit {
    uint32_t ref, tgt;
    uint32_t flags;       // kUnitRefSide1 / kUnitTgtSide1
    uint32_t pad;
    uint64_t slot_base;   // maxima of ref filter r at slots[slot_base + r]
};

struct MatParams {
    const uint32_t* filters[2];
    const uint32_t* meta[2];
    const CmpDigest* digests[2];
    const MatUnit* units;
    uint32_t nunits;
    uint32_t* next_unit;       // work counter (zero before the launch)
    const uint32_t* targets;   // target list (digest ids)
    const uint32_t* refs;      // reference digest ids of group units
    const MatSplit* split;
    uint32_t nsplit;
    double* slots;
    int32_t* scores;
    uint32_t mode;             // kMatModeAll: n*(n-1)/2 pair order; kMatModeCross: q*nt+t
    uint32_t n;                // set size (all) / number of targets (cross)
    const uint16_t* cutoffs;   // CUTOFFS256
    const uint16_t* cutoffs64; // CUTOFFS64 (fast mode)
    uint32_t* error;           // tensor-core kernel: set when a bounded wait gave up
    unsigned long long* phase; // tensor-core kernel: optional SM-cycle counters (kTcPh*), null = off
};
// phase counters of the tensor-core kernel (one producer and one consumer thread per CTA)
enum : int {
    kTcPhCompose = 0, kTcPhFill, kTcPhFetchWait, kTcPhStageWait, kTcPhWiden, kTcPhIssue, kTcPhProdStep,
    kTcPhAccWait, kTcPhScore, kTcPhFold, kTcPhConsStep, kTcPhStepBarrier, kTcPhTiles, kTcPhLd, kTcPhMark,
    kTcPhWalk, kTcPhCount
};

// Kernel variants (rows per CTA x target filters per tile), chosen by the
// autotuner.  Variants 0-4 count on the CUDA cores (carry-save AND-popcount);
// variant 5 counts on the tensor cores (tcgen05, fp8 0/1 operands, fp32
// accumulators in TMEM: the count is an exact dot product) and needs sm_100+.
struct MatVariant {
    int rows, tile;
};
constexpr int kMatVariants = 6;
constexpr int kMatVariantTc = 5;
extern const MatVariant kMatVariantTable[kMatVariants];

cudaError_t launch_matrix(const MatParams& P, int variant, uint32_t grid, cudaStream_t st);
cudaError_t launch_matrix_tc(const MatParams& P, uint32_t grid, cudaStream_t st);
int matrix_tc_ctas_per_sm();
cudaError_t launch_matrix_finalize(const MatParams& P, cudaStream_t st);
int matrix_ctas_per_sm(int variant);

// scores >= threshold -> (i, j, score) u32 triples in pair order
constexpr uint32_t kMatchBlockScores = 1024;
cudaError_t launch_match_count(const int32_t* scores, uint64_t n, int32_t thr, uint32_t* counts, cudaStream_t st);
cudaError_t launch_match_scan(const uint32_t* counts, uint64_t nblocks, uint64_t* offs, cudaStream_t st);
cudaError_t launch_match_write(const int32_t* scores, uint64_t n, int32_t thr, const uint64_t* offs, uint32_t mode,
                               uint64_t dim, uint32_t* out, uint64_t cap, cudaStream_t st);

}  // namespace sdbfg

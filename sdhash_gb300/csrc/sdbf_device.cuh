// sdbf_device.cuh -- device-side building blocks shared by the generation
// and comparison kernels (sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sdbf_tables.h"

namespace sdbfg {

// ---------------------------------------------------------------- constants
constexpr int kWin = 64;               // entropy / popularity window (sdbf_conf.cc:22,25)
constexpr int kThreshold = 16;         // selection threshold (sdbf_conf.cc:29)
constexpr int kMaxElem = 160;          // stream filter cap (sdbf_defines.h:34)
constexpr int kMaxElemDD = 192;        // block filter cap (sdbf_defines.h:35)
constexpr int kMinElem = 16;           // MIN_ELEM_COUNT (sdbf_defines.h:58)
constexpr int kBigBytes = 16384;       // big filter (sdbf_defines.h:64)
constexpr int kBigElem = 8738;         // big filter roll-over (sdbf_defines.h:65)
constexpr uint32_t kBigMask = 0x1FFFFu;
constexpr uint32_t kBfMask = 0x7FFu;   // BF_CLASS_MASKS[0]
constexpr uint64_t kChunk = 32ull << 20;  // stream chunk (sdbf_class.cc:43)
constexpr int kBf = 256;               // filter bytes

// ------------------------------------------------------------------ SHA-1
// FIPS 180-4 SHA-1 specialised for a 64-byte message: one data block plus
// the fixed padding block (0x80, zeros, bit length 512), whose message
// schedule is constant and folds into immediates once the loop is unrolled.
__device__ __forceinline__ uint32_t rotl32(uint32_t x, int n) { return __funnelshift_l(x, x, n); }

template <bool kConstSchedule>
__device__ __forceinline__ void sha1_rounds(uint32_t (&h)[5], uint32_t (&w)[16]) {
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4];
#pragma unroll
    for (int t = 0; t < 80; t++) {
        uint32_t wt;
        if (t < 16) {
            wt = w[t];
        } else {
            wt = rotl32(w[(t - 3) & 15] ^ w[(t - 8) & 15] ^ w[(t - 14) & 15] ^ w[t & 15], 1);
            w[t & 15] = wt;
        }
        uint32_t f, k;
        if (t < 20) { f = d ^ (b & (c ^ d)); k = 0x5A827999u; }
        else if (t < 40) { f = b ^ c ^ d; k = 0x6ED9EBA1u; }
        else if (t < 60) { f = (b & c) | (d & (b | c)); k = 0x8F1BBCDCu; }
        else { f = b ^ c ^ d; k = 0xCA62C1D6u; }
        uint32_t tmp = rotl32(a, 5) + f + e + k + wt;
        e = d; d = c; c = rotl32(b, 30); b = a; a = tmp;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e;
}

// msg: the 16 big-endian message words.  out: the five digest words as the
// reference reads them -- the 20 digest bytes taken as little-endian uint32
// (bf_utils.cc:32-43 casts the byte digest to uint32_t*), i.e. byte-swapped H.
__device__ __forceinline__ void sha1_feature(uint32_t (&msg)[16], uint32_t (&out)[5]) {
    uint32_t h[5] = {0x67452301u, 0xEFCDAB89u, 0x98BADCFEu, 0x10325476u, 0xC3D2E1F0u};
    sha1_rounds<false>(h, msg);
    uint32_t pad[16];
#pragma unroll
    for (int i = 0; i < 16; i++) pad[i] = 0;
    pad[0] = 0x80000000u;
    pad[15] = 512u;
    sha1_rounds<true>(h, pad);
#pragma unroll
    for (int i = 0; i < 5; i++) out[i] = __byte_perm(h[i], 0, 0x0123);
}

// Load the 64 bytes at byte offset p of a 4-byte-aligned shared buffer as 16
// big-endian words (buffer must extend 4 bytes past p+64).
__device__ __forceinline__ void load_be16(const uint32_t* sm32, uint32_t p, uint32_t (&w)[16]) {
    const uint32_t q = p >> 2, a = p & 3;
    const uint32_t sel = (a << 12) | ((a + 1) << 8) | ((a + 2) << 4) | (a + 3);
    uint32_t lo = sm32[q];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        uint32_t hi = sm32[q + k + 1];
        w[k] = __byte_perm(lo, hi, sel);
        lo = hi;
    }
}

// The same 16 words for 64 bytes at any global address: aligned word loads
// (none past the word holding the last byte) joined by byte permutes.
__device__ __forceinline__ void load_be16_global(const uint8_t* src, uint32_t (&w)[16]) {
    const uintptr_t ad = reinterpret_cast<uintptr_t>(src);
    const uint32_t* q = reinterpret_cast<const uint32_t*>(ad & ~(uintptr_t)3);
    const uint32_t a = (uint32_t)(ad & 3);
    const uint32_t sel = (a << 12) | ((a + 1) << 8) | ((a + 2) << 4) | (a + 3);
    uint32_t v[17];
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = __ldg(q + k);
    v[16] = a ? __ldg(q + 16) : 0u;
#pragma unroll
    for (int k = 0; k < 16; k++) w[k] = __byte_perm(v[k], v[k + 1], sel);
}

// ------------------------------------------------- popularity-chain state
// State entering a window step i of gen_chunk_scores (sdbf_core.cc:58-82):
// (P, M) = current (min_pos, min_rank).  M == 0 means the next step is a
// full rescan regardless of P, so P is normalised to 0 in that case.
struct ChainState {
    uint32_t P;
    uint32_t M;
};
__device__ __forceinline__ uint64_t pack_state(ChainState s) {
    return s.M == 0 ? 0ull : ((uint64_t)s.M << 32) | s.P;
}
__device__ __forceinline__ ChainState unpack_state(uint64_t v) {
    ChainState s;
    s.P = (uint32_t)v;
    s.M = (uint32_t)(v >> 32);
    return s;
}

}  // namespace sdbfg

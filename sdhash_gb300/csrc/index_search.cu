// index_search.cu -- index files and the index search of block-mode hashing.
//
// An index is one large Bloom filter (bloom_filter, sdbf/bloom_filter.cc;
// 64 MiB with 5 hash words as sdhash --index writes them,
// sdhash-src/sdhash_threads.cc:376-470).  With --index-search, block-mode
// hashing queries every fourth counted feature of each block against every
// index (sdbf::gen_block_hash, sdbf/sdbf_core.cc:141-191;
// sdbf::check_indexes :482-493) and reports, per block and index, how many
// of those features all hash bits of the index hold when that count
// exceeds 4 (print_indexes :458-472).
//
// Here the indexes are resident on the device; the block kernel records
// the sampled features' SHA-1 words of each block (GenParams::probes), and
// k_index_query counts their hits per (block, index): one warp per block,
// lanes over the indexes, each probe's words read once per warp.
//
// Index files: "sdbf-idx:<bf_size>:<elem_count>:<hash_count>:<bit_mask>:
// <compressed size>:<set name>\n" followed by the filter as one LZ4 block
// (bloom_filter::write_out / bloom_filter(string), bloom_filter.cc:87-118,
// 190-216).  The LZ4 block decoder below follows the published LZ4 block
// format (sequences of token, literals, 16-bit offset, match length).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "ctx_internal.h"

namespace {

// LZ4 block decode into exactly `out_len` bytes; returns the number of
// input bytes used, or -1 when the block is malformed or does not fill the
// output exactly.
long lz4_decode_block(const uint8_t* in, size_t in_len, uint8_t* out, size_t out_len) {
    const uint8_t* ip = in;
    const uint8_t* const iend = in + in_len;
    uint8_t* op = out;
    uint8_t* const oend = out + out_len;
    if (out_len == 0 && in_len == 0) return 0;
    while (ip < iend) {
        const uint32_t token = *ip++;
        size_t lit = token >> 4;
        if (lit == 15) {
            uint32_t b;
            do {
                if (ip >= iend) return -1;
                b = *ip++;
                lit += b;
            } while (b == 255);
        }
        if ((size_t)(iend - ip) < lit || (size_t)(oend - op) < lit) return -1;
        memcpy(op, ip, lit);
        ip += lit;
        op += lit;
        if (op == oend) return (long)(ip - in);  // the last sequence ends with its literals
        if (iend - ip < 2) return -1;
        const size_t off = (size_t)ip[0] | ((size_t)ip[1] << 8);
        ip += 2;
        if (off == 0 || off > (size_t)(op - out)) return -1;
        size_t mlen = token & 15u;
        if (mlen == 15) {
            uint32_t b;
            do {
                if (ip >= iend) return -1;
                b = *ip++;
                mlen += b;
            } while (b == 255);
        }
        mlen += 4;
        if ((size_t)(oend - op) < mlen) return -1;
        const uint8_t* src = op - off;
        for (size_t k = 0; k < mlen; k++) op[k] = src[k];  // byte order: overlapping copies repeat
        op += mlen;
    }
    return -1;
}

// LZ4 block encode (the published block format): greedy matches of at
// least 4 bytes found through a hash table of 4-byte sequences, offsets up
// to 65,535; the format's end rules are kept (the last 5 bytes are
// literals, no match starts in the last 12).  Any LZ4 decoder reads it.
void lz4_put_len(std::vector<uint8_t>& out, size_t v) {
    while (v >= 255) {
        out.push_back(255);
        v -= 255;
    }
    out.push_back((uint8_t)v);
}

void lz4_encode_block(const uint8_t* in, size_t n, std::vector<uint8_t>& out) {
    out.clear();
    auto read32 = [&](size_t i) {
        uint32_t v;
        memcpy(&v, in + i, 4);
        return v;
    };
    auto emit = [&](size_t anchor, size_t lit_end, size_t off, size_t mlen) {
        const size_t lit = lit_end - anchor;
        const size_t ml = mlen ? mlen - 4 : 0;
        uint8_t token = (uint8_t)((lit >= 15 ? 15 : lit) << 4);
        if (mlen) token |= (uint8_t)(ml >= 15 ? 15 : ml);
        out.push_back(token);
        if (lit >= 15) lz4_put_len(out, lit - 15);
        out.insert(out.end(), in + anchor, in + lit_end);
        if (!mlen) return;
        out.push_back((uint8_t)(off & 0xFF));
        out.push_back((uint8_t)(off >> 8));
        if (ml >= 15) lz4_put_len(out, ml - 15);
    };
    size_t anchor = 0;
    if (n >= 13) {
        std::vector<uint32_t> table(1u << 16, 0xFFFFFFFFu);
        const size_t mflimit = n - 12, matchlimit = n - 5;
        size_t ip = 0;
        while (ip < mflimit) {
            const uint32_t seq = read32(ip);
            const uint32_t h = (seq * 2654435761u) >> 16;
            const uint32_t ref = table[h];
            table[h] = (uint32_t)ip;
            if (ref != 0xFFFFFFFFu && ip - ref <= 65535 && read32(ref) == seq) {
                size_t len = 4;
                while (ip + len < matchlimit && in[ref + len] == in[ip + len]) len++;
                emit(anchor, ip, ip - ref, len);
                ip += len;
                anchor = ip;
            } else {
                ip++;
            }
        }
    }
    emit(anchor, n, 0, 0);  // the last literals
}

bool parse_u64(const std::string& s, uint64_t* v) {
    if (s.empty() || s.size() > 20) return false;
    uint64_t x = 0;
    for (char ch : s) {
        if (ch < '0' || ch > '9') return false;
        x = x * 10 + (uint64_t)(ch - '0');
    }
    *v = x;
    return true;
}

// BIT_MASKS_32[log2(size) + 2] of the bloom_filter constructor
// (bloom_filter.cc:52-71): the mask of a filter of `size` bytes.
uint64_t mask_for_size(uint64_t size) {
    uint32_t log_size = 0;
    for (uint64_t t = size; t; t >>= 1) log_size++;
    const uint32_t bits = log_size + 2;  // BIT_MASKS_32[i] has i+1 low bits set
    return bits >= 32 ? 0xFFFFFFFFull : ((1ull << bits) - 1);
}

int make_index(sdbfg_ctx* c, const uint8_t* bits, uint64_t bf_size, uint64_t elem_count, uint32_t hash_count,
               uint64_t bit_mask, const std::string& name, sdbfg_index** out) {
    auto* x = new sdbfg_index();
    x->ctx = c;
    x->bf_size = bf_size;
    x->elem_count = elem_count;
    x->hash_count = hash_count;
    x->bit_mask = bit_mask;
    x->name = name;
    if (x->d_bits.ensure(bf_size) != cudaSuccess) {
        delete x;
        cudaGetLastError();
        return fail(c, SDBFG_ERR_NOMEM, "index: out of device memory");
    }
    const cudaError_t e = cudaMemcpy(x->d_bits.p, bits, bf_size, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        x->d_bits.release();
        delete x;
        return fail(c, SDBFG_ERR_CUDA, "index upload: %s", cudaGetErrorString(e));
    }
    *out = x;
    return SDBFG_OK;
}

}  // namespace

// -------------------------------------------------------------- device part

struct IndexDev {
    const uint8_t* bits;
    uint32_t mask;
    uint32_t hash_count;
};

__global__ void __launch_bounds__(256) k_index_query(const uint32_t* __restrict__ probes,
                                                     const uint8_t* __restrict__ nprobes, uint64_t nslots,
                                                     const IndexDev* __restrict__ idx, uint32_t nidx,
                                                     uint8_t* __restrict__ hits) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t s = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); s < nslots; s += warps) {
        const uint32_t np = nprobes[s];
        const uint32_t* pr = probes + s * kProbeWords;
        for (uint32_t i = lane; i < nidx; i += 32) {
            const IndexDev X = idx[i];
            uint32_t cnt = 0;
            for (uint32_t p = 0; p < np; p++) {
                bool all = true;
                for (uint32_t z = 0; z < X.hash_count && all; z++) {
                    const uint32_t pos = pr[p * 5 + z] & X.mask;  // query_and_set, bloom_filter.cc:333-359
                    all = (__ldg(X.bits + (pos >> 3)) >> (pos & 7)) & 1u;
                }
                cnt += all;
            }
            hits[s * nidx + i] = (uint8_t)cnt;
        }
    }
}

int index_query(sdbfg_ctx* c, const uint32_t* d_probes, const uint8_t* d_nprobes, uint64_t nslots,
                const sdbfg_index* const* indexes, uint32_t nidx, uint8_t* d_hits, cudaStream_t st) {
    if (!nslots || !nidx) return SDBFG_OK;
    std::vector<IndexDev> h(nidx);
    for (uint32_t i = 0; i < nidx; i++)
        h[i] = IndexDev{indexes[i]->d_bits.as<uint8_t>(), (uint32_t)indexes[i]->bit_mask, indexes[i]->hash_count};
    CUDA_TRY(c, c->d_index_tab.ensure(nidx * sizeof(IndexDev)));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_index_tab.p, h.data(), nidx * sizeof(IndexDev), cudaMemcpyHostToDevice, st));
    const uint32_t grid = (uint32_t)std::min<uint64_t>((nslots + 7) / 8, (uint64_t)c->sms * 16);
    TIMED_LAUNCH_ON(c, "k_index_query", st,
                    (k_index_query<<<grid, 256, 0, st>>>(d_probes, d_nprobes, nslots, c->d_index_tab.as<IndexDev>(),
                                                         nidx, d_hits),
                     cudaGetLastError()));
    // the index table must outlive the async copy
    CUDA_TRY(c, cudaStreamSynchronize(st));
    return SDBFG_OK;
}

// ------------------------------------------------------ block-mode build
// Exact in input order without a sequential pass: a feature set a new bit
// iff it is the first setter (smallest ordinal) of one of its bits.
// Ordinal = (global slot + 1) << 8 | feature index (bits set before the
// batch have first setter 0).

// Four entries (one 16-byte store) per thread; nbits is a power of two >= 512.
__global__ void k_index_first_init(const uint32_t* __restrict__ bits, uint32_t* __restrict__ first, uint64_t nbits) {
    uint4* out = reinterpret_cast<uint4*>(first);
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nbits / 4;
         q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (__ldg(bits + (q >> 3)) >> ((q & 7) * 4)) & 15u;
        out[q] = make_uint4((b & 1u) ? 0u : ~0u, (b & 2u) ? 0u : ~0u, (b & 4u) ? 0u : ~0u, (b & 8u) ? 0u : ~0u);
    }
}

__global__ void k_index_first(const uint32_t* __restrict__ feats, const uint16_t* __restrict__ counts, uint64_t nslots,
                              uint64_t slot0, uint32_t mask, uint32_t* __restrict__ first) {
    const uint64_t n = nslots * 192;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s = i / 192;
        const uint32_t k = (uint32_t)(i % 192);
        if (k >= counts[s]) continue;
        const uint32_t ord = (uint32_t)((slot0 + s + 1) << 8) | k;
        const uint32_t* w = feats + s * kFeatWords + k * 5;
#pragma unroll
        for (int z = 0; z < 5; z++) atomicMin(first + (w[z] & mask), ord);
    }
}

__global__ void k_index_mark(const uint32_t* __restrict__ feats, const uint16_t* __restrict__ counts, uint64_t nslots,
                             uint64_t slot0, uint32_t mask, const uint32_t* __restrict__ first,
                             uint32_t* __restrict__ bits, unsigned long long* __restrict__ count) {
    const uint64_t n = nslots * 192;
    uint32_t mine = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s = i / 192;
        const uint32_t k = (uint32_t)(i % 192);
        if (k >= counts[s]) continue;
        const uint32_t ord = (uint32_t)((slot0 + s + 1) << 8) | k;
        const uint32_t* w = feats + s * kFeatWords + k * 5;
        bool fresh = false;
#pragma unroll
        for (int z = 0; z < 5; z++) {
            const uint32_t pos = w[z] & mask;
            fresh |= first[pos] == ord;
            atomicOr(bits + (pos >> 5), 1u << (pos & 31));
        }
        mine += fresh;
    }
    for (int d = 16; d > 0; d >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, d);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(count, (unsigned long long)mine);
}

int index_first_init(sdbfg_ctx* c, const uint32_t* d_bits, uint32_t* d_first, uint64_t nbits, cudaStream_t st) {
    const uint32_t grid = (uint32_t)std::min<uint64_t>((nbits / 4 + 255) / 256, (uint64_t)c->sms * 32);
    TIMED_LAUNCH_ON(c, "k_index_first_init", st,
                    (k_index_first_init<<<grid, 256, 0, st>>>(d_bits, d_first, nbits), cudaGetLastError()));
    return SDBFG_OK;
}

int index_build_group(sdbfg_ctx* c, const uint32_t* d_feats, const uint16_t* d_counts, uint64_t nslots,
                      uint64_t slot0, uint32_t mask, uint32_t* d_first, uint32_t* d_bits,
                      unsigned long long* d_count, cudaStream_t st) {
    if (!nslots) return SDBFG_OK;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((nslots * 192 + 255) / 256, (uint64_t)c->sms * 32);
    TIMED_LAUNCH_ON(c, "k_index_first", st,
                    (k_index_first<<<grid, 256, 0, st>>>(d_feats, d_counts, nslots, slot0, mask, d_first),
                     cudaGetLastError()));
    TIMED_LAUNCH_ON(c, "k_index_mark", st,
                    (k_index_mark<<<grid, 256, 0, st>>>(d_feats, d_counts, nslots, slot0, mask, d_first, d_bits,
                                                        d_count),
                     cudaGetLastError()));
    return SDBFG_OK;
}

// ------------------------------------------------------------------ C ABI

extern "C" int sdbfg_index_create(sdbfg_ctx* c, const uint8_t* bits, uint64_t bf_size, uint32_t hash_count,
                                  const char* name, sdbfg_index** out) {
    if (!c || !out || !bits) return SDBFG_ERR_ARG;
    *out = nullptr;
    // bloom_filter(size, ...) accepts powers of two >= 64 (bloom_filter.cc:58-68)
    if (bf_size < 64 || (bf_size & (bf_size - 1)) || hash_count == 0 || hash_count > 5)
        return fail(c, SDBFG_ERR_ARG, "index: size must be a power of two >= 64, 1..5 hash words");
    uint64_t mask = mask_for_size(bf_size);
    if (mask >= bf_size * 8) mask = bf_size * 8 - 1;  // the positions the filter holds
    CUDA_TRY(c, cudaSetDevice(c->device));
    return make_index(c, bits, bf_size, 0, hash_count, mask, name ? name : "", out);
}

extern "C" int sdbfg_index_load_file(sdbfg_ctx* c, const char* path, sdbfg_index** out) {
    if (!c || !out || !path) return SDBFG_ERR_ARG;
    *out = nullptr;
    FILE* f = fopen(path, "rb");
    if (!f) return fail(c, SDBFG_ERR_ARG, "index: cannot open %s", path);  // bloom_filter(string) throws -1
    std::vector<char> buf;
    char tmp[1 << 16];
    size_t k;
    while ((k = fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + k);
    fclose(f);
    // header: six ':'-terminated fields, then the set name up to '\n'
    std::string fields[6];
    size_t pos = 0;
    for (int i = 0; i < 6; i++) {
        size_t e = pos;
        while (e < buf.size() && buf[e] != ':') e++;
        if (e >= buf.size()) return fail(c, SDBFG_ERR_FORMAT, "index %s: short header", path);
        fields[i].assign(buf.data() + pos, e - pos);
        pos = e + 1;
    }
    size_t e = pos;
    while (e < buf.size() && buf[e] != '\n') e++;
    if (e >= buf.size()) return fail(c, SDBFG_ERR_FORMAT, "index %s: short header", path);
    const std::string name(buf.data() + pos, e - pos);
    pos = e + 1;
    uint64_t bf_size, elem, hc, mask, comp;
    if (!parse_u64(fields[1], &bf_size) || !parse_u64(fields[2], &elem) || !parse_u64(fields[3], &hc) ||
        !parse_u64(fields[4], &mask) || !parse_u64(fields[5], &comp))
        return fail(c, SDBFG_ERR_FORMAT, "index %s: bad header field", path);
    // the reference reads hash_count hash words of a 5-word SHA-1 and
    // positions up to bit_mask in a bf_size-byte filter; anything else
    // would read past them
    if (bf_size == 0 || bf_size > (1ull << 36) || hc == 0 || hc > 5 || mask > 0xFFFFFFFFull || mask >= bf_size * 8)
        return fail(c, SDBFG_ERR_FORMAT, "index %s: unsupported geometry", path);
    if (comp > buf.size() - pos) return fail(c, SDBFG_ERR_FORMAT, "index %s: truncated data", path);
    std::vector<uint8_t> bits(bf_size);
    if (lz4_decode_block(reinterpret_cast<const uint8_t*>(buf.data()) + pos, comp, bits.data(), bf_size) < 0)
        return fail(c, SDBFG_ERR_FORMAT, "index %s: bad compressed data", path);  // throws -2
    CUDA_TRY(c, cudaSetDevice(c->device));
    return make_index(c, bits.data(), bf_size, elem, (uint32_t)hc, mask, name, out);
}

extern "C" void sdbfg_index_free(sdbfg_index* x) {
    if (!x) return;
    cudaSetDevice(x->ctx->device);
    x->d_bits.release();
    delete x;
}

extern "C" int sdbfg_index_info(const sdbfg_index* x, uint64_t* bf_size, uint64_t* elem_count, uint32_t* hash_count,
                                uint64_t* bit_mask, const char** name) {
    if (!x) return SDBFG_ERR_ARG;
    if (bf_size) *bf_size = x->bf_size;
    if (elem_count) *elem_count = x->elem_count;
    if (hash_count) *hash_count = x->hash_count;
    if (bit_mask) *bit_mask = x->bit_mask;
    if (name) *name = x->name.c_str();
    return SDBFG_OK;
}

extern "C" int64_t sdbfg_lz4_decode(const uint8_t* in, uint64_t in_len, uint8_t* out, uint64_t out_len) {
    if ((!in && in_len) || (!out && out_len)) return SDBFG_ERR_ARG;
    const long r = lz4_decode_block(in, in_len, out, out_len);
    return r < 0 ? SDBFG_ERR_FORMAT : r;
}

extern "C" int64_t sdbfg_lz4_encode(const uint8_t* in, uint64_t in_len, uint8_t* out, uint64_t out_cap) {
    if (!in && in_len) return SDBFG_ERR_ARG;
    std::vector<uint8_t> enc;
    lz4_encode_block(in, in_len, enc);
    if (out && enc.size() <= out_cap) memcpy(out, enc.data(), enc.size());
    return (int64_t)enc.size();
}

extern "C" int sdbfg_index_write_file(const char* path, const uint8_t* bits, uint64_t bf_size, uint64_t elem_count,
                                      uint32_t hash_count, const char* set_name) {
    if (!path || !bits || bf_size < 64 || (bf_size & (bf_size - 1))) return SDBFG_ERR_ARG;
    std::vector<uint8_t> enc;
    lz4_encode_block(bits, bf_size, enc);
    FILE* f = fopen(path, "wb");
    if (!f) return SDBFG_ERR_ARG;  // bloom_filter::write_out returns -2
    const int ok = fprintf(f, "sdbf-idx:%llu:%llu:%u:%llu:%llu:%s\n", (unsigned long long)bf_size,
                           (unsigned long long)elem_count, hash_count, (unsigned long long)mask_for_size(bf_size),
                           (unsigned long long)enc.size(), set_name ? set_name : "") > 0 &&
                   fwrite(enc.data(), 1, enc.size(), f) == enc.size();
    return (fclose(f) == 0 && ok) ? SDBFG_OK : SDBFG_ERR_ARG;
}

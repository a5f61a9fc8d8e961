// sdbf_api.cu -- host orchestration behind the C ABI (include/sdbf_gb300.h).
//
// Owns the context and the generation path: builds the chunk / tile / file
// work lists for a batch, launches the generation kernels and moves digests
// back.  Comparison lives in compare_api.cu.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sdbf_gb300.h"
#include "ctx_internal.h"
#include "sdbf_tables.h"

// ------------------------------------------------------------------ context
extern "C" int sdbfg_ctx_create(int device, sdbfg_ctx** out) {
    if (!out) return SDBFG_ERR_ARG;
    *out = nullptr;
    auto* c = new sdbfg_ctx();
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete c;
        return SDBFG_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return SDBFG_ERR_CUDA;
    }
    c->stream = c->own;
    uint32_t ent[65];
    for (int i = 0; i < 65; i++) ent[i] = SDBF_ENTROPY64[i];
    if (c->d_rank.ensure(sizeof(SDBF_ENTR64_RANKS)) || c->d_ent.ensure(sizeof(ent)) ||
        c->d_cut.ensure(sizeof(SDBF_CUTOFFS256)) || c->d_cut64.ensure(sizeof(SDBF_CUTOFFS64)) ||
        c->d_counters.ensure(64)) {
        sdbfg_ctx_destroy(c);
        return SDBFG_ERR_NOMEM;
    }
    cudaMemcpy(c->d_rank.p, SDBF_ENTR64_RANKS, sizeof(SDBF_ENTR64_RANKS), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_ent.p, ent, sizeof(ent), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_cut.p, SDBF_CUTOFFS256, sizeof(SDBF_CUTOFFS256), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_cut64.p, SDBF_CUTOFFS64, sizeof(SDBF_CUTOFFS64), cudaMemcpyHostToDevice);
    cudaMemset(c->d_counters.p, 0, 64);
    *out = c;
    return SDBFG_OK;
}

extern "C" void sdbfg_ctx_destroy(sdbfg_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    for (MatPlan* p : c->plans) delete p;
    c->plans.clear();
    for (DevBuf* b : {&c->d_rank, &c->d_ent, &c->d_cut, &c->d_cut64, &c->d_data, &c->d_chunks, &c->d_tiles, &c->d_files,
                      &c->d_order, &c->d_tile_out, &c->d_features, &c->d_work_filters, &c->d_info,
                      &c->d_counters, &c->d_pack_src, &c->d_pack_dst_off, &c->d_out_filters, &c->d_out_counts,
                      &c->d_pairs, &c->d_scores, &c->d_binfo, &c->d_boff, &c->d_total, &c->d_phase,
                      &c->d_match_counts, &c->d_match_offs, &c->d_matches, &c->d_mphase, &c->d_probes,
                      &c->d_nprobes, &c->d_hits, &c->d_index_tab, &c->d_feats, &c->d_idx_bits, &c->d_idx_first,
                      &c->d_idx_count, &c->d_seen[0], &c->d_seen[1], &c->d_pred, &c->d_diff, &c->d_ckpt,
                      &c->d_from, &c->d_ranks})
        b->release();
    for (auto& S : c->slot) {
        for (DevBuf* b : {&S.data, &S.chunks, &S.tiles, &S.files, &S.order, &S.tile_out, &S.features, &S.work,
                          &S.redo, &S.rk_items, &S.fix_list})
            b->release();
        S.h_tables.release();
        if (S.stream) cudaStreamDestroy(S.stream);
        if (S.done) cudaEventDestroy(S.done);
    }
    for (cudaEvent_t e : c->ev_scan)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : c->ev_tiles)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : c->ev_copy)
        if (e) cudaEventDestroy(e);
    c->d_stage_in.release();
    c->d_stage_items.release();
    c->h_stage_items.release();
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->ev_start) cudaEventDestroy(c->ev_start);
    c->h_stage.release();
    timer_collect(c);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
}

extern "C" const char* sdbfg_last_error(const sdbfg_ctx* c) { return c ? c->err.c_str() : "no context"; }

extern "C" int sdbfg_ctx_set_stream(sdbfg_ctx* c, void* s) {
    if (!c) return SDBFG_ERR_ARG;
    c->stream = s ? static_cast<cudaStream_t>(s) : c->own;
    return SDBFG_OK;
}

extern "C" int sdbfg_ctx_synchronize(sdbfg_ctx* c) {
    if (!c) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return SDBFG_OK;
}

extern "C" uint64_t sdbfg_ctx_launch_count(const sdbfg_ctx* c) { return c ? c->launches : 0; }

extern "C" int sdbfg_ctx_profile(sdbfg_ctx* c, int enable) {
    if (!c) return SDBFG_ERR_ARG;
    timer_collect(c);
    c->profile = enable != 0;
    if (enable) {
        c->stats.clear();
        CUDA_TRY(c, c->d_phase.ensure(kPhCount * sizeof(unsigned long long)));
        CUDA_TRY(c, cudaMemset(c->d_phase.p, 0, kPhCount * sizeof(unsigned long long)));
        CUDA_TRY(c, c->d_mphase.ensure(kTcPhCount * sizeof(unsigned long long)));
        CUDA_TRY(c, cudaMemset(c->d_mphase.p, 0, kTcPhCount * sizeof(unsigned long long)));
    }
    return SDBFG_OK;
}

static const char* kPhaseNames[kPhCount] = {
    "k_stream_tiles.load", "k_stream_tiles.ranks", "k_stream_tiles.fres", "k_stream_tiles.walk",
    "k_stream_tiles.link", "k_stream_tiles.compact", "k_stream_tiles.sha1", "k_stream_tiles.count",
    "k_stream_commit.wait", "k_stream_commit.busy", "k_stream_commit.groups", "k_stream_commit.loops",
    "k_stream_commit.max_file", "k_stream_tiles.fixups", "k_stream_commit_round.restarts"};

extern "C" int sdbfg_ctx_kernel_time(sdbfg_ctx* c, const char* name, double* total_ms, uint64_t* launches) {
    if (!c || !name) return SDBFG_ERR_ARG;
    timer_collect(c);
    if (total_ms) *total_ms = 0;
    if (launches) *launches = 0;
    for (int k = 0; k < kPhCount; k++)
        if (!strcmp(name, kPhaseNames[k]) && c->d_phase.p) {
            unsigned long long v[kPhCount];
            CUDA_TRY(c, cudaMemcpy(v, c->d_phase.p, sizeof v, cudaMemcpyDeviceToHost));
            if (total_ms) *total_ms = (double)v[k];
            if (launches) *launches = v[kPhTiles];
            return SDBFG_OK;
        }
    static const char* kTcNames[kTcPhCount] = {
        "k_matrix_tc.compose", "k_matrix_tc.fill", "k_matrix_tc.fetch_wait", "k_matrix_tc.stage_wait",
        "k_matrix_tc.widen", "k_matrix_tc.issue", "k_matrix_tc.producer_step", "k_matrix_tc.acc_wait",
        "k_matrix_tc.score", "k_matrix_tc.fold", "k_matrix_tc.consumer_step", "k_matrix_tc.step_barrier",
        "k_matrix_tc.tiles", "k_matrix_tc.tmem_ld", "k_matrix_tc.mark", "k_matrix_tc.walk"};
    for (int k = 0; k < kTcPhCount; k++)
        if (!strcmp(name, kTcNames[k]) && c->d_mphase.p) {
            unsigned long long v[kTcPhCount];
            CUDA_TRY(c, cudaMemcpy(v, c->d_mphase.p, sizeof v, cudaMemcpyDeviceToHost));
            if (total_ms) *total_ms = (double)v[k];
            if (launches) *launches = v[kTcPhTiles];
            return SDBFG_OK;
        }
    for (const KernelStat& k : c->stats)
        if (k.name == name) {
            if (total_ms) *total_ms = k.ms;
            if (launches) *launches = k.launches;
        }
    return SDBFG_OK;
}

extern "C" int sdbfg_ctx_pipeline_depth(const sdbfg_ctx* c) { return c ? c->depth : 0; }

extern "C" int sdbfg_ctx_set_pipeline_depth(sdbfg_ctx* c, int depth) {
    if (!c || depth < 1 || depth > kSlots) return SDBFG_ERR_ARG;
    c->depth = depth;
    return SDBFG_OK;
}

extern "C" int sdbfg_ctx_set_lead(sdbfg_ctx* c, uint32_t steps) {
    if (!c || steps > kLead) return SDBFG_ERR_ARG;
    c->lead = steps;
    return SDBFG_OK;
}

extern "C" int sdbfg_ctx_set_index_rounds(sdbfg_ctx* c, uint32_t max_rounds) {
    if (!c || max_rounds > 1024) return SDBFG_ERR_ARG;
    c->index_max_rounds = max_rounds;
    return SDBFG_OK;
}

extern "C" uint32_t sdbfg_ctx_index_rounds(sdbfg_ctx* c) { return c ? c->index_rounds_used : 0; }

extern "C" uint64_t sdbfg_ctx_relinked_tiles(sdbfg_ctx* c) {
    if (!c) return 0;
    uint32_t v = 0;
    cudaMemcpy(&v, c->d_counters.p, 4, cudaMemcpyDeviceToHost);
    return v;
}

// ------------------------------------------------------------- generation
static uint64_t stream_cap(uint64_t len) { return (len >> 11) + 1; }
static uint64_t block_count(uint64_t len, uint32_t B) { return len / B + ((len % B) >= kMinFile ? 1 : 0); }

extern "C" uint64_t sdbfg_digest_capacity(const uint64_t* lens, uint32_t n, uint32_t dd) {
    uint64_t s = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (lens[i] < kMinFile) continue;
        s += dd ? block_count(lens[i], dd) : stream_cap(lens[i]);
    }
    return s;
}

// Packs each file's filters from the generation workspace to its final slot.
__global__ void k_pack_filters(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                               const uint64_t* __restrict__ src_off, const uint64_t* __restrict__ dst_off,
                               const FileInfoDev* __restrict__ info, const uint32_t* __restrict__ ids, uint32_t n) {
    for (uint32_t f = blockIdx.x; f < n; f += gridDim.x) {
        const uint32_t id = ids[f];
        const uint64_t words = (uint64_t)info[id].bf_count * 64;
        const uint4* s = reinterpret_cast<const uint4*>(src + src_off[f] * 64);
        uint4* d = reinterpret_cast<uint4*>(dst + dst_off[f] * 64);
        for (uint64_t q = threadIdx.x; q < words / 4; q += blockDim.x) d[q] = s[q];
    }
}

namespace {

struct Group {  // consecutive inputs processed by one launch sequence
    uint32_t first, count;
};

// Splits inputs into launch groups bounded by tiles (stream) or bytes.
// Launch groups of consecutive inputs, each at most kMaxTilesPerLaunch tiles
// and kMaxBytesPerLaunch bytes; the first group at most first_cap bytes and
// each later one at most twice its predecessor's cap (host inputs: a short
// first copy lets the kernels start early, and the ramp keeps each later
// group's copy shorter than the kernels of the groups before it).
std::vector<Group> make_groups(const uint64_t* lens, uint32_t n, uint32_t dd,
                               uint64_t first_cap = kMaxBytesPerLaunch) {
    std::vector<Group> gs;
    uint32_t start = 0;
    uint64_t tiles = 0, bytes = 0;
    uint64_t cap_bytes = std::min(first_cap, kMaxBytesPerLaunch);
    for (uint32_t i = 0; i < n; i++) {
        uint64_t t = 0;
        if (!dd && lens[i] >= kMinFile) {
            for (uint64_t pos = 0; pos < lens[i]; pos += kChunkBytes) {
                const uint64_t m = std::min<uint64_t>(kChunkBytes, lens[i] - pos);
                if (m > 64) t += (m - 64 + kTileL - 1) / kTileL;
            }
        }
        const uint64_t b = (lens[i] + 15) & ~15ull;
        if (i > start && (tiles + t > kMaxTilesPerLaunch || bytes + b > cap_bytes)) {
            gs.push_back({start, i - start});
            start = i;
            tiles = 0;
            bytes = 0;
            cap_bytes = std::min(2 * cap_bytes, kMaxBytesPerLaunch);
        }
        tiles += t;
        bytes += b;
    }
    if (n > start) gs.push_back({start, n - start});
    return gs;
}

}  // namespace

// Core: inputs for files [g.first, g.first+g.count) are in device memory at
// dev_base + dev_off[i].  Writes packed filters to dev_out (+ counts) at the
// offsets in results[] (already assigned for block mode, assigned here for
// stream mode starting at *next_slot).
static int digest_group_device(sdbfg_ctx* c, const uint8_t* dev_base, const std::vector<uint64_t>& dev_off,
                               const uint64_t* lens, const Group& g, uint32_t dd, uint32_t* dev_out,
                               uint16_t* dev_counts, sdbfg_digest_result* res, uint64_t* next_slot,
                               uint64_t out_cap) {
    cudaStream_t st = c->stream;
    GenParams P{};
    P.data = dev_base;
    P.rank_tab = c->d_rank.as<uint16_t>();
    P.ent_tab = c->d_ent.as<uint32_t>();
    P.counters = c->d_counters.as<uint32_t>();
    P.lead = c->lead;
    if (dd) {
        std::vector<GenChunk> chunks;
        uint32_t lmax = 0;
        for (uint32_t k = 0; k < g.count; k++) {
            const uint32_t i = g.first + k;
            if (lens[i] < kMinFile) continue;
            const uint64_t qt = lens[i] / dd, rem = lens[i] % dd;
            uint64_t slot = res[i].filter_offset;
            for (uint64_t b = 0; b < qt; b++) {
                chunks.push_back({dev_off[k] + b * dd, dd, i, 0, 0, (uint32_t)(slot + b), 0});
                lmax = std::max<uint32_t>(lmax, dd - 64);
            }
            if (rem >= kMinFile) {
                chunks.push_back({dev_off[k] + qt * dd, (uint32_t)rem, i, 0, 0, (uint32_t)(slot + qt), 1});
                lmax = std::max<uint32_t>(lmax, (uint32_t)rem - 64);
            }
        }
        if (chunks.empty()) return SDBFG_OK;
        CUDA_TRY(c, c->d_chunks.ensure(chunks.size() * sizeof(GenChunk)));
        CUDA_TRY(c, cudaMemcpyAsync(c->d_chunks.p, chunks.data(), chunks.size() * sizeof(GenChunk),
                                    cudaMemcpyHostToDevice, st));
        P.chunks = c->d_chunks.as<GenChunk>();
        P.nchunks = (uint32_t)chunks.size();
        P.out_filters = dev_out;
        P.out_counts = dev_counts;
        P.probes = c->probe_words;
        P.nprobes = c->probe_counts;
        P.feats = c->feat_words;
        P.block_lmax = (lmax + 63) / 64 * 64;
        const uint32_t grid = (uint32_t)std::min<size_t>(chunks.size(), (size_t)c->sms * 2 * 8);
        TIMED_LAUNCH(c, "k_block_digest", launch_block(P, grid, st));
        // the chunk table must outlive the async copy
        CUDA_TRY(c, cudaStreamSynchronize(st));
        return SDBFG_OK;
    }
    return fail(c, SDBFG_ERR_ARG, "internal: stream mode goes through the pipeline");
}

// ---------------------------------------------------- stream pipeline
// Output slots of one launch group: exclusive scan of the files' filter
// counts, continuing from the running total of the earlier groups
// (*total), so the packed layout follows input order.
__global__ void k_scan_offsets(const FileInfoDev* __restrict__ info, uint64_t* __restrict__ dst_off, uint32_t n,
                               uint64_t* __restrict__ total) {
    __shared__ uint64_t warp_sums[32];
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = *total;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint64_t v = i < n ? info[i].bf_count : 0;
        uint64_t incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        uint64_t woff = 0, tot = 0;
        for (uint32_t w = 0; w < blockDim.x / 32; w++) {
            if (w < wid) woff += warp_sums[w];
            tot += warp_sums[w];
        }
        if (i < n) dst_off[i] = carry + woff + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_pack_group(const uint32_t* __restrict__ work, const GenFile* __restrict__ files,
                             const FileInfoDev* __restrict__ info, const uint64_t* __restrict__ dst_off,
                             uint32_t* __restrict__ dst, uint32_t n) {
    for (uint32_t f = blockIdx.x; f < n; f += gridDim.x) {
        if (files[f].nchunks == 0) continue;
        const uint64_t words = (uint64_t)info[f].bf_count * 64;
        const uint4* s = reinterpret_cast<const uint4*>(work + files[f].filter_base * 64);
        uint4* d = reinterpret_cast<uint4*>(dst + dst_off[f] * 64);
        for (uint64_t q = threadIdx.x; q < words / 4; q += blockDim.x) d[q] = s[q];
    }
}

// Staging of pinned host inputs: each piece (at most kStagePiece bytes of
// one input) is read straight from host memory through the device's mapping
// of the pinned buffer and written to its 16-byte aligned staging offset;
// 16-byte loads where the source allows them, else 4-byte or single bytes.
// kGatherThreads threads and few registers, so a CTA fits on an SM beside
// the tile kernel's four.
constexpr int kGatherThreads = 128;
__global__ void __launch_bounds__(kGatherThreads) k_stage_gather(const StagePiece* __restrict__ items, uint32_t n,
                                                                  uint8_t* __restrict__ dst) {
    for (uint32_t f = blockIdx.x; f < n; f += gridDim.x) {
        const StagePiece it = items[f];
        const uint8_t* s = reinterpret_cast<const uint8_t*>(it.src);
        uint8_t* d = dst + it.dst;
        uint64_t done = 0;
        if ((it.src & 15) == 0) {
            const uint4* s4 = reinterpret_cast<const uint4*>(s);
            uint4* d4 = reinterpret_cast<uint4*>(d);
            const uint64_t n4 = it.len / 16;
            uint64_t q = threadIdx.x;
            for (; q + 3 * kGatherThreads < n4; q += 4 * kGatherThreads) {
                const uint4 a = s4[q], b = s4[q + kGatherThreads], c = s4[q + 2 * kGatherThreads],
                            e = s4[q + 3 * kGatherThreads];
                d4[q] = a;
                d4[q + kGatherThreads] = b;
                d4[q + 2 * kGatherThreads] = c;
                d4[q + 3 * kGatherThreads] = e;
            }
            for (; q < n4; q += kGatherThreads) d4[q] = s4[q];
            done = n4 * 16;
        } else if ((it.src & 3) == 0) {
            const uint32_t* s1 = reinterpret_cast<const uint32_t*>(s);
            uint32_t* d1 = reinterpret_cast<uint32_t*>(d);
            const uint64_t n1 = it.len / 4;
            for (uint64_t q = threadIdx.x; q < n1; q += kGatherThreads) d1[q] = s1[q];
            done = n1 * 4;
        }
        for (uint64_t q = done + threadIdx.x; q < it.len; q += kGatherThreads) d[q] = s[q];
    }
}

static int ensure_pipeline(sdbfg_ctx* c) {
    for (int k = 0; k < kSlots; k++) {
        if (!c->slot[k].stream) {
            CUDA_TRY(c, cudaStreamCreateWithFlags(&c->slot[k].stream, cudaStreamNonBlocking));
            CUDA_TRY(c, cudaEventCreateWithFlags(&c->slot[k].done, cudaEventDisableTiming));
            CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_scan[k], cudaEventDisableTiming));
            CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_tiles[k], cudaEventDisableTiming));
        }
    }
    if (!c->ev_start) CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming));
    // the pipeline's small kernels take the tile kernels' shared-memory / L1
    // split, so their CTAs can share an SM with them
    for (const void* f : {(const void*)k_stage_gather, (const void*)k_scan_offsets, (const void*)k_pack_group})
        cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    cudaGetLastError();
    return SDBFG_OK;
}

// Stream-mode digests of n inputs.  Inputs are either already on the device
// (dev_data + offsets[i], 16-byte aligned) or in host memory (host_data +
// offsets[i]) and copied per launch group.  Filters are packed in input
// order into dev_out (device); results[] gets counts and slots.  Launch
// groups alternate between two streams with their own workspaces, so the
// commit of one group overlaps the tiles (and the input copy) of the next;
// the host synchronises once, at the end.
// An index being built alongside (sdhash --index): device bits, bit mask,
// counter of inserts that set a new bit.
struct IndexBuild {
    uint32_t* bits;
    uint32_t mask;
    unsigned long long* count;
};

// The commit of one stream launch group with an index being built, as a
// fixed point: round 1 commits every file with the predicate bits of a first
// guess (every selected feature inserted); then, from the first setters of the features the last
// round inserted, new predicate bits; files whose bits changed commit again,
// until none changes (the digests are then the sequential ones, and the index
// takes the inserted features' bits).  After index_max_rounds commit rounds
// without that, the one-warp sequential commit runs instead.
static int commit_with_index(sdbfg_ctx* c, GenParams P, uint32_t cap_grid, cudaStream_t st) {
    c->index_rounds_used = 0;
    const uint64_t nfeat = (uint64_t)P.ntiles * kTileCap;
    if (c->index_max_rounds && P.ntiles) {
        const uint64_t nwords = nfeat / 32 + 2, nbits = (uint64_t)P.index_mask + 1;
        for (DevBuf* b : {&c->d_seen[0], &c->d_seen[1], &c->d_pred}) CUDA_TRY(c, b->ensure(nwords * 4));
        CUDA_TRY(c, c->d_diff.ensure(8 + std::max<uint64_t>(1, P.nfiles)));
        CUDA_TRY(c, c->d_from.ensure(std::max<uint64_t>(1, P.nfiles) * 4));
        CUDA_TRY(c, c->d_ckpt.ensure(((uint64_t)P.ntiles / kCkptTiles + 1) * kCkptWords * 4));
        P.commit_ckpt = c->d_ckpt.as<uint32_t>();
        P.commit_from = c->d_from.as<uint32_t>();
        CUDA_TRY(c, c->d_idx_first.ensure(nbits * 4));
        uint32_t* first = c->d_idx_first.as<uint32_t>();
        uint32_t* seen = c->d_seen[0].as<uint32_t>();
        uint32_t* pred[2] = {c->d_pred.as<uint32_t>(), c->d_seen[1].as<uint32_t>()};
        unsigned int* ndirty = c->d_diff.as<unsigned int>();
        uint8_t* dirty = c->d_diff.as<uint8_t>() + 8;
        const uint32_t commit_grid = std::min<uint32_t>((P.nfiles + kCommitWarps - 1) / kCommitWarps, cap_grid);
        const uint32_t fgrid = (uint32_t)std::min<uint64_t>((nfeat + 255) / 256, (uint64_t)c->sms * 32);
        const uint64_t pwords = (nfeat + 31) / 32;
        const uint32_t wgrid = (uint32_t)std::min<uint64_t>((pwords + 255) / 256, (uint64_t)c->sms * 8);
        // first guess: every selected feature inserted (chance collisions of
        // all five index bits are then predicted in round 1)
        int rc = index_first_init(c, P.index_bits, first, nbits, st);
        if (rc) return rc;
        CUDA_TRY(c, cudaMemsetAsync(seen, 0xFF, nwords * 4, st));
        TIMED_LAUNCH_ON(c, "k_stream_index_first", st, launch_stream_index_first(P, seen, first, fgrid, st));
        TIMED_LAUNCH_ON(c, "k_stream_index_pred", st, launch_stream_index_pred(P, first, pred[0], fgrid, st));
        CUDA_TRY(c, cudaMemsetAsync(seen, 0, nwords * 4, st));
        P.index_seen = seen;
        P.index_pred = pred[0];
        P.commit_dirty = nullptr;
        TIMED_LAUNCH_ON(c, "k_stream_commit_round", st, launch_stream_commit_round(P, commit_grid, st));
        uint32_t commits = 1;
        int cur = 0;
        while (true) {
            rc = index_first_init(c, P.index_bits, first, nbits, st);
            if (rc) return rc;
            TIMED_LAUNCH_ON(c, "k_stream_index_first", st, launch_stream_index_first(P, seen, first, fgrid, st));
            TIMED_LAUNCH_ON(c, "k_stream_index_pred", st,
                            launch_stream_index_pred(P, first, pred[cur ^ 1], fgrid, st));
            CUDA_TRY(c, cudaMemsetAsync(c->d_diff.p, 0, 8 + P.nfiles, st));
            CUDA_TRY(c, cudaMemsetAsync(c->d_from.p, 0xFF, (size_t)P.nfiles * 4, st));
            TIMED_LAUNCH_ON(c, "k_pred_dirty", st,
                            launch_pred_dirty(P, pred[cur], pred[cur ^ 1], pwords, dirty, c->d_from.as<uint32_t>(),
                                              ndirty, wgrid, st));
            unsigned int nd = 0;
            CUDA_TRY(c, cudaMemcpyAsync(&nd, ndirty, 4, cudaMemcpyDeviceToHost, st));
            CUDA_TRY(c, cudaStreamSynchronize(st));
            if (nd == 0) {
                TIMED_LAUNCH_ON(c, "k_stream_index_mark", st, launch_stream_index_mark(P, seen, first, fgrid, st));
                c->index_rounds_used = commits;
                return SDBFG_OK;
            }
            if (commits >= c->index_max_rounds) break;
            cur ^= 1;
            P.index_pred = pred[cur];
            P.commit_dirty = dirty;
            TIMED_LAUNCH_ON(c, "k_stream_commit_round", st, launch_stream_commit_round(P, commit_grid, st));
            commits++;
        }
    }
    TIMED_LAUNCH_ON(c, "k_stream_commit_index", st, launch_stream_commit_index(P, st));
    return SDBFG_OK;
}

static int digest_stream_pipelined(sdbfg_ctx* c, const uint8_t* host_data, const uint8_t* dev_data,
                                   const uint64_t* offsets_in, const uint64_t* lens_in, uint32_t n, uint32_t* dev_out,
                                   uint64_t out_cap, sdbfg_digest_result* res, uint64_t* total_out,
                                   const IndexBuild* ib = nullptr) {
    int rc = ensure_pipeline(c);
    if (rc) return rc;
    // Launch groups are formed over the inputs sorted by size (largest first),
    // so the long ordered commits of the largest inputs start early and
    // overlap the rest of the batch; the packed output follows this order and
    // results[] records where each input's filters are.
    // (an index build keeps input order: every file's digest depends on the
    // index inserts of the files before it)
    // Pinned host inputs are staged whole on the device when they fit.  A
    // gather kernel per launch group reads the group's inputs straight from
    // host memory (the device's mapping of the pinned buffer) on a
    // high-priority stream of its own, one event per group: the copies cost
    // one launch per group instead of one API call per input (tens of
    // microseconds each), and no copy waits behind an earlier group's commit
    // or a slot's reuse.  Its small CTAs fit beside the tile kernel's.
    bool staged = false;
    const uint8_t* host_dev = nullptr;  // the device's view of the pinned input
    if (host_data && !ib && n) {
        cudaPointerAttributes attr{};
        const bool pinned = cudaPointerGetAttributes(&attr, host_data) == cudaSuccess &&
                            attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr;
        cudaGetLastError();
        if (pinned)
            host_dev = static_cast<const uint8_t*>(attr.devicePointer) +
                       (host_data - static_cast<const uint8_t*>(attr.hostPointer));
        uint64_t tot = 0;
        for (uint32_t i = 0; i < n; i++) tot += (lens_in[i] + 15) & ~15ull;
        size_t freeb = 0, totb = 0;
        if (pinned && tot <= kStageMaxBytes && cudaMemGetInfo(&freeb, &totb) == cudaSuccess &&
            (c->d_stage_in.cap >= tot || tot <= freeb / 2)) {
            CUDA_TRY(c, c->d_stage_in.ensure(std::max<uint64_t>(16, tot)));
            if (!c->copy_stream) {
                int lo = 0, hi = 0;
                CUDA_TRY(c, cudaDeviceGetStreamPriorityRange(&lo, &hi));
                CUDA_TRY(c, cudaStreamCreateWithPriority(&c->copy_stream, cudaStreamNonBlocking, hi));
            }
            staged = true;
        }
        cudaGetLastError();
    }
    std::vector<uint32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0u);
    if (!ib)
        std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return lens_in[a] > lens_in[b]; });
    std::vector<uint64_t> lens_v(n), offs_v(n);
    for (uint32_t i = 0; i < n; i++) {
        lens_v[i] = lens_in[perm[i]];
        offs_v[i] = offsets_in[perm[i]];
    }
    const uint64_t* lens = lens_v.data();
    const uint64_t* offsets = offs_v.data();
    CUDA_TRY(c, c->d_binfo.ensure(std::max<size_t>(1, n) * sizeof(FileInfoDev)));
    CUDA_TRY(c, c->d_boff.ensure(std::max<size_t>(1, n) * sizeof(uint64_t)));
    CUDA_TRY(c, c->d_total.ensure(64));
    CUDA_TRY(c, cudaMemsetAsync(c->d_binfo.p, 0, std::max<size_t>(1, n) * sizeof(FileInfoDev), c->stream));
    CUDA_TRY(c, cudaMemsetAsync(c->d_total.p, 0, 64, c->stream));
    CUDA_TRY(c, cudaEventRecord(c->ev_start, c->stream));
    const std::vector<Group> groups = make_groups(lens, n, 0, host_data ? kFirstHostGroupBytes : kMaxBytesPerLaunch);
    std::vector<uint64_t> stage_off;
    if (staged) {
        stage_off.resize(n);
        uint64_t tot = 0;
        for (uint32_t i = 0; i < n; i++) {
            stage_off[i] = tot;
            tot += (lens[i] + 15) & ~15ull;
        }
        while (c->ev_copy.size() < groups.size()) {
            cudaEvent_t e;
            CUDA_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            c->ev_copy.push_back(e);
        }
        // after the previous batch's work on the caller's stream
        CUDA_TRY(c, cudaStreamWaitEvent(c->copy_stream, c->ev_start, 0));
    }
    if (staged) {
        // pieces of at most kStagePiece bytes; the item tables of all groups
        // go over in one copy, then one gather launch per group
        std::vector<uint32_t> first_item(groups.size() + 1, 0);
        uint64_t nitems = 0;
        for (size_t gi = 0; gi < groups.size(); gi++) {
            first_item[gi] = (uint32_t)nitems;
            for (uint32_t k = 0; k < groups[gi].count; k++) {
                const uint64_t len = lens[groups[gi].first + k];
                if (len >= kMinFile) nitems += (len + kStagePiece - 1) / kStagePiece;
            }
        }
        first_item[groups.size()] = (uint32_t)nitems;
        CUDA_TRY(c, c->h_stage_items.ensure(std::max<uint64_t>(1, nitems) * sizeof(StagePiece)));
        CUDA_TRY(c, c->d_stage_items.ensure(std::max<uint64_t>(1, nitems) * sizeof(StagePiece)));
        // the previous batch's table copy has finished (its call synchronised
        // at its end); the host table may be rewritten
        StagePiece* it = reinterpret_cast<StagePiece*>(c->h_stage_items.p);
        uint64_t q = 0;
        for (uint32_t i = 0; i < n; i++) {
            if (lens[i] < kMinFile) continue;
            for (uint64_t pos = 0; pos < lens[i]; pos += kStagePiece)
                it[q++] = StagePiece{stage_off[i] + pos, reinterpret_cast<uint64_t>(host_dev + offsets[i] + pos),
                                     std::min<uint64_t>(kStagePiece, lens[i] - pos)};
        }
        if (nitems)
            CUDA_TRY(c, cudaMemcpyAsync(c->d_stage_items.p, it, nitems * sizeof(StagePiece), cudaMemcpyHostToDevice,
                                        c->copy_stream));
        for (size_t gi = 0; gi < groups.size(); gi++) {
            const uint32_t ni = first_item[gi + 1] - first_item[gi];
            if (ni)
                TIMED_LAUNCH_ON(c, "k_stage_gather", c->copy_stream,
                                (k_stage_gather<<<std::min<uint32_t>(ni, (uint32_t)c->sms), kGatherThreads, 0,
                                                  c->copy_stream>>>(c->d_stage_items.as<StagePiece>() + first_item[gi],
                                                                    ni, c->d_stage_in.as<uint8_t>()),
                                 cudaGetLastError()));
            CUDA_TRY(c, cudaEventRecord(c->ev_copy[gi], c->copy_stream));
        }
    }
    // Precomputed ranks (2 bytes per input byte) in two halves, by group
    // parity: a group's rank kernel waits for the tile and fix kernels of the
    // group two back (the last readers of its half) and runs beside the
    // previous group's tile kernel.  Sized once for the largest group;
    // without the room the tile kernels compute the ranks themselves.
    bool pre_ranks = c->pre_ranks;
    if (pre_ranks) {
        uint64_t most = 0;
        for (const Group& g : groups) {
            uint64_t r8 = 0;
            for (uint32_t k = 0; k < g.count; k++) {
                const uint64_t len = lens[g.first + k];
                if (len >= kMinFile) r8 += (len + 7) / 8 + len / kChunkBytes + 1;  // per chunk, to a multiple of 8
            }
            most = std::max(most, r8);
        }
        if (c->d_ranks.ensure(2 * (most * 16 + 16)) != cudaSuccess) {
            cudaGetLastError();
            c->d_ranks.release();
            pre_ranks = false;
        }
    }
    cudaEvent_t prev_scan = c->ev_start, prev_tiles = c->ev_start, prev2_tiles = c->ev_start;
    const uint64_t rank_half = c->d_ranks.cap / 2 / 16 * 16;  // bytes per half, 16-byte aligned
    for (size_t gi = 0; gi < groups.size(); gi++) {
        const Group& g = groups[gi];
        const int depth = ib ? 1 : std::max(1, std::min(c->depth, kSlots));
        sdbfg_ctx::Slot& S = c->slot[gi % depth];
        cudaStream_t st = S.stream;
        if (S.used) CUDA_TRY(c, cudaEventSynchronize(S.done));  // its pinned tables may be reused now
        S.used = true;
        CUDA_TRY(c, cudaStreamWaitEvent(st, c->ev_start, 0));
        // ---- work lists (pinned host staging, copied asynchronously)
        // rank stretches: every chunk position (to a multiple of 8), kRkSpan at a time
        uint64_t nchunks = 0, ntiles = 0, bytes = 0, nrk = 0;
        for (uint32_t k = 0; k < g.count; k++) {
            const uint64_t len = lens[g.first + k];
            bytes += (len + 15) & ~15ull;
            if (len < kMinFile) continue;
            for (uint64_t pos = 0; pos < len; pos += kChunkBytes) {
                const uint64_t m = std::min<uint64_t>(kChunkBytes, len - pos);
                nchunks++;
                if (m > 64) ntiles += (m - 64 + kTileL - 1) / kTileL;
                nrk += ((m + 7) / 8 * 8 + kRkSpan - 1) / kRkSpan;
            }
        }
        bool pre = pre_ranks && ntiles;
        if (pre && S.rk_items.ensure(nrk * sizeof(uint2)) != cudaSuccess) {
            cudaGetLastError();
            S.rk_items.release();
            pre = false;
        }
        const size_t tb_chunks = nchunks * sizeof(GenChunk), tb_tiles = ntiles * sizeof(GenTile);
        const size_t tb_files = g.count * sizeof(GenFile), tb_order = g.count * sizeof(uint32_t);
        const size_t tb_rk = pre ? nrk * sizeof(uint2) : 0;
        CUDA_TRY(c, S.h_tables.ensure(tb_chunks + tb_tiles + tb_files + tb_order + tb_rk + 64));
        GenChunk* hc = reinterpret_cast<GenChunk*>(S.h_tables.p);
        GenTile* ht = reinterpret_cast<GenTile*>(reinterpret_cast<uint8_t*>(S.h_tables.p) + tb_chunks);
        GenFile* hf = reinterpret_cast<GenFile*>(reinterpret_cast<uint8_t*>(ht) + tb_tiles);
        uint32_t* ho = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(hf) + tb_files);
        uint2* hr = reinterpret_cast<uint2*>(reinterpret_cast<uint8_t*>(ho) + tb_order);
        const uint8_t* gdata;
        std::vector<uint64_t> doff(g.count);
        if (dev_data) {
            gdata = dev_data;
            for (uint32_t k = 0; k < g.count; k++) doff[k] = offsets[g.first + k];
        } else if (staged) {
            gdata = c->d_stage_in.as<uint8_t>();
            for (uint32_t k = 0; k < g.count; k++) doff[k] = stage_off[g.first + k];
            CUDA_TRY(c, cudaStreamWaitEvent(st, c->ev_copy[gi], 0));
        } else {
            CUDA_TRY(c, S.data.ensure(std::max<uint64_t>(16, bytes)));
            gdata = S.data.as<uint8_t>();
            uint64_t b = 0;
            for (uint32_t k = 0; k < g.count; k++) {
                doff[k] = b;
                b += (lens[g.first + k] + 15) & ~15ull;
            }
            bool contiguous = true;
            for (uint32_t k = 0; k < g.count && contiguous; k++)
                contiguous = offsets[g.first + k] - offsets[g.first] == doff[k];
            if (contiguous) {
                CUDA_TRY(c, cudaMemcpyAsync(S.data.p, host_data + offsets[g.first], bytes, cudaMemcpyHostToDevice, st));
            } else {
                for (uint32_t k = 0; k < g.count; k++) {
                    const uint32_t i = g.first + k;
                    if (lens[i] < kMinFile) continue;
                    CUDA_TRY(c, cudaMemcpyAsync(S.data.as<uint8_t>() + doff[k], host_data + offsets[i], lens[i],
                                                cudaMemcpyHostToDevice, st));
                }
            }
        }
        uint32_t ci = 0, ti = 0, ri = 0, r8 = 0;
        uint64_t work = 0;
        for (uint32_t k = 0; k < g.count; k++) {
            const uint32_t i = g.first + k;
            GenFile f{ci, 0, work, 0};
            if (lens[i] >= kMinFile) {
                for (uint64_t pos = 0; pos < lens[i]; pos += kChunkBytes) {
                    const uint32_t m = (uint32_t)std::min<uint64_t>(kChunkBytes, lens[i] - pos);
                    GenChunk ch{doff[k] + pos, m, k, ti, 0, 0, 0, r8};
                    if (m > 64)
                        for (uint32_t t0 = 0; t0 < m - 64; t0 += kTileL) ht[ti++] = GenTile{ci, t0};
                    ch.ntiles = ti - ch.first_tile;
                    if (pre)
                        for (uint32_t s0 = 0; s0 < (m + 7) / 8 * 8; s0 += kRkSpan) hr[ri++] = make_uint2(ci, s0);
                    r8 += (m + 7) / 8;
                    hc[ci++] = ch;
                    f.nchunks++;
                }
                f.filter_cap = stream_cap(lens[i]);
                work += f.filter_cap;
            }
            hf[k] = f;
            ho[k] = k;
        }
        if (!ib)
            std::stable_sort(ho, ho + g.count,
                             [&](uint32_t a, uint32_t b) { return lens[g.first + a] > lens[g.first + b]; });
        CUDA_TRY(c, S.chunks.ensure(std::max<size_t>(1, tb_chunks)));
        CUDA_TRY(c, S.tiles.ensure(std::max<size_t>(1, tb_tiles)));
        CUDA_TRY(c, S.files.ensure(std::max<size_t>(1, tb_files)));
        CUDA_TRY(c, S.order.ensure(std::max<size_t>(1, tb_order)));
        CUDA_TRY(c, S.tile_out.ensure(std::max<uint64_t>(1, ntiles) * sizeof(TileOut)));
        CUDA_TRY(c, S.features.ensure(std::max<uint64_t>(1, ntiles) * 5ull * kTileCap * 4));
        CUDA_TRY(c, S.work.ensure(std::max<uint64_t>(1, work) * 256));
        CUDA_TRY(c, S.redo.ensure(std::max<uint64_t>(1, nchunks) * 4));
        CUDA_TRY(c, S.fix_list.ensure((ntiles + 1) * 4));
        if (tb_chunks) CUDA_TRY(c, cudaMemcpyAsync(S.chunks.p, hc, tb_chunks, cudaMemcpyHostToDevice, st));
        if (tb_tiles) CUDA_TRY(c, cudaMemcpyAsync(S.tiles.p, ht, tb_tiles, cudaMemcpyHostToDevice, st));
        CUDA_TRY(c, cudaMemcpyAsync(S.files.p, hf, tb_files, cudaMemcpyHostToDevice, st));
        CUDA_TRY(c, cudaMemcpyAsync(S.order.p, ho, tb_order, cudaMemcpyHostToDevice, st));
        if (tb_rk) CUDA_TRY(c, cudaMemcpyAsync(S.rk_items.p, hr, tb_rk, cudaMemcpyHostToDevice, st));
        GenParams P{};
        P.data = gdata;
        P.rank_tab = c->d_rank.as<uint16_t>();
        P.ent_tab = c->d_ent.as<uint32_t>();
        P.counters = c->d_counters.as<uint32_t>();
        P.lead = c->lead;
        P.phase = c->profile ? c->d_phase.as<unsigned long long>() : nullptr;
        P.chunks = S.chunks.as<GenChunk>();
        P.nchunks = (uint32_t)nchunks;
        P.tiles = S.tiles.as<GenTile>();
        P.ntiles = (uint32_t)ntiles;
        P.files = S.files.as<GenFile>();
        P.file_order = S.order.as<uint32_t>();
        P.nfiles = g.count;
        P.tile_out = S.tile_out.as<TileOut>();
        P.features = S.features.as<uint32_t>();
        P.out_filters = S.work.as<uint32_t>();
        P.out_info = c->d_binfo.as<FileInfoDev>() + g.first;
        P.chunk_redo = S.redo.as<uint32_t>();
        P.fix_list = S.fix_list.as<uint32_t>();
        if (pre) {
            P.ranks = c->d_ranks.as<uint16_t>() + (gi & 1) * (rank_half / 2);
            P.rk_items = S.rk_items.as<uint2>();
            P.nrk_items = (uint32_t)nrk;
        }
        const uint32_t cap_grid = (uint32_t)c->sms * 3 * 16;
        // the groups' tile kernels run one after another (each fills the GPU),
        // so a group's commit overlaps the next group's tiles instead of all
        // groups in flight finishing their tiles together and then waiting
        // on their commits
        if (pre) {
            CUDA_TRY(c, cudaStreamWaitEvent(st, prev2_tiles, 0));
            TIMED_LAUNCH_ON(c, "k_stream_ranks", st,
                            launch_stream_ranks(P, std::min<uint32_t>(P.nrk_items, cap_grid), st));
        }
        CUDA_TRY(c, cudaStreamWaitEvent(st, prev_tiles, 0));
        if (P.ntiles)
            TIMED_LAUNCH_ON(c, "k_stream_tiles", st, launch_stream_tiles(P, std::min<uint32_t>(P.ntiles, cap_grid), st));
        if (P.nchunks) {
            if (P.ntiles) {
                CUDA_TRY(c, cudaMemsetAsync(P.fix_list, 0, 4, st));
                TIMED_LAUNCH_ON(c, "k_stream_fails", st,
                                launch_stream_fails(P, std::min<uint32_t>((P.ntiles + 255) / 256, cap_grid), st));
                TIMED_LAUNCH_ON(c, "k_stream_fix_list", st,
                                launch_stream_fix_list(P, std::min<uint32_t>(P.ntiles, (uint32_t)c->sms * 5), st));
            }
            TIMED_LAUNCH_ON(c, "k_stream_check", st, launch_stream_check(P, (P.nchunks + 3) / 4, st));
            TIMED_LAUNCH_ON(c, "k_stream_fix", st,
                            launch_stream_fix(P, std::min<uint32_t>(P.nchunks, cap_grid), st));
        }
        CUDA_TRY(c, cudaEventRecord(c->ev_tiles[gi % depth], st));
        prev2_tiles = prev_tiles;
        prev_tiles = c->ev_tiles[gi % depth];
        if (ib) {
            P.index_bits = ib->bits;
            P.index_mask = ib->mask;
            P.index_new = ib->count;
            rc = commit_with_index(c, P, cap_grid, st);
            if (rc) return rc;
        } else {
            TIMED_LAUNCH_ON(c, "k_stream_commit", st,
                            launch_stream_commit(P, std::min<uint32_t>((g.count + kCommitWarps - 1) / kCommitWarps,
                                                                       cap_grid), st));
        }
        // output slots follow input order: scan after the previous group's scan
        CUDA_TRY(c, cudaStreamWaitEvent(st, prev_scan, 0));
        TIMED_LAUNCH_ON(c, "k_scan_offsets", st,
                        (k_scan_offsets<<<1, 1024, 0, st>>>(c->d_binfo.as<FileInfoDev>() + g.first,
                                                             c->d_boff.as<uint64_t>() + g.first, g.count,
                                                             c->d_total.as<uint64_t>()),
                         cudaGetLastError()));
        CUDA_TRY(c, cudaEventRecord(c->ev_scan[gi % depth], st));
        prev_scan = c->ev_scan[gi % depth];
        TIMED_LAUNCH_ON(c, "k_pack_filters", st,
                        (k_pack_group<<<std::min<uint32_t>(g.count, (uint32_t)c->sms * 8), 256, 0, st>>>(
                             S.work.as<uint32_t>(), S.files.as<GenFile>(), c->d_binfo.as<FileInfoDev>() + g.first,
                             c->d_boff.as<uint64_t>() + g.first, dev_out, g.count),
                         cudaGetLastError()));
        CUDA_TRY(c, cudaEventRecord(S.done, st));
    }
    // join: the caller's stream waits for both slots, then results come back
    for (int k = 0; k < kSlots; k++)
        if (c->slot[k].used) CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->slot[k].done, 0));
    std::vector<FileInfoDev> info(n);
    std::vector<uint64_t> off(n);
    uint64_t flags_total[2] = {0, 0};
    uint32_t flags[2] = {0, 0};
    if (n) {
        CUDA_TRY(c, cudaMemcpyAsync(info.data(), c->d_binfo.p, n * sizeof(FileInfoDev), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(off.data(), c->d_boff.p, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, c->stream));
    }
    CUDA_TRY(c, cudaMemcpyAsync(flags_total, c->d_total.p, 8, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(flags, c->d_counters.p, sizeof flags, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (flags[1]) return fail(c, SDBFG_ERR_CUDA, "internal error: stream digest exceeded its filter bound");
    if (flags_total[0] > out_cap)
        return fail(c, SDBFG_ERR_CAPACITY, "output capacity %llu filters < %llu needed", (unsigned long long)out_cap,
                    (unsigned long long)flags_total[0]);
    for (uint32_t i = 0; i < n; i++) {
        if (lens[i] < kMinFile) continue;
        sdbfg_digest_result& r = res[perm[i]];
        r.bf_count = info[i].bf_count;
        r.last_count = info[i].last_count;
        r.filter_offset = off[i];
    }
    if (total_out) *total_out = flags_total[0];
    return SDBFG_OK;
}

static int validate_batch(sdbfg_ctx* c, const uint64_t* offsets, const uint64_t* lens, uint32_t n, uint32_t dd,
                          sdbfg_digest_result* res) {
    if (!c || (!offsets && n) || (!lens && n) || (!res && n)) return SDBFG_ERR_ARG;
    if (dd > kMaxBlockBytes || (dd && dd < kMinFile))
        return fail(c, SDBFG_ERR_ARG, "dd_block_size %u outside [512, 16384]", dd);
    for (uint32_t i = 0; i < n; i++) {
        res[i] = sdbfg_digest_result{};
        if (lens[i] < kMinFile) res[i].status = SDBFG_DIGEST_TOO_SMALL;
        if (lens[i] >= (1ull << 40)) return fail(c, SDBFG_ERR_ARG, "input %u too large", i);
    }
    return SDBFG_OK;
}

// block mode: slots are known up front
static uint64_t assign_block_slots(const uint64_t* lens, uint32_t n, uint32_t dd, sdbfg_digest_result* res) {
    uint64_t slot = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (lens[i] < kMinFile) continue;
        res[i].filter_offset = slot;
        res[i].bf_count = (uint32_t)block_count(lens[i], dd);
        slot += res[i].bf_count;
    }
    return slot;
}

extern "C" int sdbfg_digest_batch_device(sdbfg_ctx* c, const uint8_t* dev_data, const uint64_t* offsets,
                                         const uint64_t* lens, uint32_t n, uint32_t dd, uint8_t* dev_out,
                                         uint64_t out_cap, uint16_t* dev_counts, sdbfg_digest_result* res) {
    int rc = validate_batch(c, offsets, lens, n, dd, res);
    if (rc) return rc;
    for (uint32_t i = 0; i < n; i++)
        if (offsets[i] % 16) return fail(c, SDBFG_ERR_ARG, "device input %u not 16-byte aligned", i);
    CUDA_TRY(c, cudaSetDevice(c->device));
    uint64_t next = 0;
    if (dd) {
        const uint64_t need = assign_block_slots(lens, n, dd, res);
        if (need > out_cap) return fail(c, SDBFG_ERR_CAPACITY, "need %llu filter slots", (unsigned long long)need);
        if (need && !dev_counts) return fail(c, SDBFG_ERR_ARG, "block mode needs element-count output");
    }
    if (!dd) return digest_stream_pipelined(c, nullptr, dev_data, offsets, lens, n, reinterpret_cast<uint32_t*>(dev_out),
                                            out_cap, res, nullptr);
    for (const Group& g : make_groups(lens, n, dd)) {
        std::vector<uint64_t> off(offsets + g.first, offsets + g.first + g.count);
        rc = digest_group_device(c, dev_data, off, lens, g, dd, reinterpret_cast<uint32_t*>(dev_out), dev_counts, res,
                                 &next, out_cap);
        if (rc) return rc;
    }
    return SDBFG_OK;
}

// Block-mode batch from host memory, launch group by launch group; with
// indexes, also the index-search hits of every filter slot.
static int digest_block_host(sdbfg_ctx* c, const uint8_t* host_data, const uint64_t* offsets, const uint64_t* lens,
                             uint32_t n, uint32_t dd, uint8_t* out_filters, uint16_t* out_counts,
                             sdbfg_digest_result* res, const sdbfg_index* const* indexes, uint32_t nidx,
                             uint8_t* out_hits, const IndexBuild* ib = nullptr, uint32_t* d_first = nullptr) {
    cudaStream_t st = c->stream;
    cudaPointerAttributes attr{};
    const bool pinned = cudaPointerGetAttributes(&attr, host_data) == cudaSuccess &&
                        (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    uint64_t next = 0;
    for (const Group& g : make_groups(lens, n, dd)) {
        // lay the group's inputs out 16-byte aligned on the device
        std::vector<uint64_t> off(g.count);
        uint64_t bytes = 0;
        for (uint32_t k = 0; k < g.count; k++) {
            off[k] = bytes;
            bytes += (lens[g.first + k] + 15) & ~15ull;
        }
        CUDA_TRY(c, c->d_data.ensure(std::max<uint64_t>(bytes, 16)));
        uint8_t* d = c->d_data.as<uint8_t>();
        // contiguous source range with the same layout -> one copy
        bool contiguous = true;
        for (uint32_t k = 0; k < g.count && contiguous; k++)
            contiguous = offsets[g.first + k] - offsets[g.first] == off[k];
        if (contiguous && pinned) {
            CUDA_TRY(c, cudaMemcpyAsync(d, host_data + offsets[g.first], bytes, cudaMemcpyHostToDevice, st));
        } else {
            for (uint32_t k = 0; k < g.count; k++) {
                const uint32_t i = g.first + k;
                if (lens[i] < kMinFile) continue;
                CUDA_TRY(c, cudaMemcpyAsync(d + off[k], host_data + offsets[i], lens[i], cudaMemcpyHostToDevice, st));
            }
        }
        // block mode writes its slots directly; copy back this group's range
        uint64_t group_slots = 0, group_first_slot = 0;
        bool first = true;
        for (uint32_t k = 0; k < g.count; k++) {
            const uint32_t i = g.first + k;
            if (lens[i] < kMinFile) continue;
            if (first) {
                group_first_slot = res[i].filter_offset;
                first = false;
            }
            group_slots = res[i].filter_offset + res[i].bf_count - group_first_slot;
        }
        CUDA_TRY(c, c->d_out_filters.ensure(std::max<uint64_t>(1, group_slots) * 256));
        CUDA_TRY(c, c->d_out_counts.ensure(std::max<uint64_t>(1, group_slots) * 2));
        if (nidx) {
            CUDA_TRY(c, c->d_probes.ensure(std::max<uint64_t>(1, group_slots) * kProbeWords * 4));
            CUDA_TRY(c, c->d_nprobes.ensure(std::max<uint64_t>(1, group_slots)));
            CUDA_TRY(c, c->d_hits.ensure(std::max<uint64_t>(1, group_slots) * nidx));
            c->probe_words = c->d_probes.as<uint32_t>();
            c->probe_counts = c->d_nprobes.as<uint8_t>();
        }
        if (ib) {
            CUDA_TRY(c, c->d_feats.ensure(std::max<uint64_t>(1, group_slots) * kFeatWords * 4));
            c->feat_words = c->d_feats.as<uint32_t>();
        }
        // shift slots into the group-local output buffer
        std::vector<uint64_t> saved(g.count);
        for (uint32_t k = 0; k < g.count; k++) {
            saved[k] = res[g.first + k].filter_offset;
            res[g.first + k].filter_offset -= group_first_slot;
        }
        int rc = digest_group_device(c, d, off, lens, g, dd, c->d_out_filters.as<uint32_t>(),
                                     c->d_out_counts.as<uint16_t>(), res, &next, UINT64_MAX);
        c->probe_words = nullptr;
        c->probe_counts = nullptr;
        c->feat_words = nullptr;
        for (uint32_t k = 0; k < g.count; k++) res[g.first + k].filter_offset = saved[k];
        if (rc) return rc;
        if (ib && group_slots) {
            rc = index_build_group(c, c->d_feats.as<uint32_t>(), c->d_out_counts.as<uint16_t>(), group_slots,
                                   group_first_slot, ib->mask, d_first, ib->bits, ib->count, st);
            if (rc) return rc;
        }
        if (nidx && group_slots) {
            rc = index_query(c, c->d_probes.as<uint32_t>(), c->d_nprobes.as<uint8_t>(), group_slots, indexes, nidx,
                             c->d_hits.as<uint8_t>(), st);
            if (rc) return rc;
            CUDA_TRY(c, cudaMemcpyAsync(out_hits + group_first_slot * nidx, c->d_hits.p, group_slots * nidx,
                                        cudaMemcpyDeviceToHost, st));
        }
        if (group_slots) {
            CUDA_TRY(c, cudaMemcpyAsync(out_filters + group_first_slot * 256, c->d_out_filters.p, group_slots * 256,
                                        cudaMemcpyDeviceToHost, st));
            CUDA_TRY(c, cudaMemcpyAsync(out_counts + group_first_slot, c->d_out_counts.p, group_slots * 2,
                                        cudaMemcpyDeviceToHost, st));
        }
        CUDA_TRY(c, cudaStreamSynchronize(st));
    }
    return SDBFG_OK;
}

extern "C" int sdbfg_digest_batch(sdbfg_ctx* c, const uint8_t* host_data, const uint64_t* offsets,
                                  const uint64_t* lens, uint32_t n, uint32_t dd, uint8_t* out_filters,
                                  uint64_t out_cap, uint16_t* out_counts, sdbfg_digest_result* res) {
    int rc = validate_batch(c, offsets, lens, n, dd, res);
    if (rc) return rc;
    if (n && !host_data) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    if (!dd) {
        uint64_t cap_needed = 0;
        for (uint32_t i = 0; i < n; i++)
            if (lens[i] >= kMinFile) cap_needed += stream_cap(lens[i]);
        CUDA_TRY(c, c->d_out_filters.ensure(std::max<uint64_t>(1, cap_needed) * 256));
        uint64_t total = 0;
        rc = digest_stream_pipelined(c, host_data, nullptr, offsets, lens, n, c->d_out_filters.as<uint32_t>(),
                                     std::min(cap_needed, out_cap), res, &total);
        if (rc) return rc;
        if (total) CUDA_TRY(c, cudaMemcpyAsync(out_filters, c->d_out_filters.p, total * 256, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(c, cudaStreamSynchronize(st));
        return SDBFG_OK;
    }
    const uint64_t total_slots = assign_block_slots(lens, n, dd, res);
    if (total_slots > out_cap)
        return fail(c, SDBFG_ERR_CAPACITY, "need %llu filter slots", (unsigned long long)total_slots);
    if (total_slots && !out_counts) return fail(c, SDBFG_ERR_ARG, "block mode needs element-count output");
    return digest_block_host(c, host_data, offsets, lens, n, dd, out_filters, out_counts, res, nullptr, 0, nullptr);
}

extern "C" int sdbfg_digest_batch_index(sdbfg_ctx* c, const uint8_t* host_data, const uint64_t* offsets,
                                        const uint64_t* lens, uint32_t n, uint32_t dd, uint8_t* out_filters,
                                        uint64_t out_cap, uint16_t* out_counts, sdbfg_digest_result* res,
                                        uint8_t* index_bits, uint64_t index_bytes, uint64_t* elem_count) {
    if (!index_bits || !elem_count) return SDBFG_ERR_ARG;
    // a power-of-two filter of 64 bytes .. 512 MiB (bit positions fit 32 bits)
    if (index_bytes < 64 || (index_bytes & (index_bytes - 1)) || index_bytes > (512ull << 20))
        return fail(c, SDBFG_ERR_ARG, "index size must be a power of two from 64 bytes to 512 MiB");
    int rc = validate_batch(c, offsets, lens, n, dd, res);
    if (rc) return rc;
    if (n && !host_data) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const uint64_t nbits = index_bytes * 8;
    CUDA_TRY(c, c->d_idx_bits.ensure(index_bytes));
    CUDA_TRY(c, c->d_idx_count.ensure(8));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_idx_bits.p, index_bits, index_bytes, cudaMemcpyHostToDevice, st));
    CUDA_TRY(c, cudaMemsetAsync(c->d_idx_count.p, 0, 8, st));
    const IndexBuild ib{c->d_idx_bits.as<uint32_t>(), (uint32_t)(nbits - 1), c->d_idx_count.as<unsigned long long>()};
    if (!dd) {
        uint64_t cap_needed = 0;
        for (uint32_t i = 0; i < n; i++)
            if (lens[i] >= kMinFile) cap_needed += stream_cap(lens[i]);
        CUDA_TRY(c, c->d_out_filters.ensure(std::max<uint64_t>(1, cap_needed) * 256));
        uint64_t total = 0;
        rc = digest_stream_pipelined(c, host_data, nullptr, offsets, lens, n, c->d_out_filters.as<uint32_t>(),
                                     std::min(cap_needed, out_cap), res, &total, &ib);
        if (rc) return rc;
        if (total) CUDA_TRY(c, cudaMemcpyAsync(out_filters, c->d_out_filters.p, total * 256, cudaMemcpyDeviceToHost, st));
    } else {
        const uint64_t total_slots = assign_block_slots(lens, n, dd, res);
        if (total_slots > out_cap)
            return fail(c, SDBFG_ERR_CAPACITY, "need %llu filter slots", (unsigned long long)total_slots);
        if (total_slots && !out_counts) return fail(c, SDBFG_ERR_ARG, "block mode needs element-count output");
        if ((total_slots + 1) >> 24) return fail(c, SDBFG_ERR_ARG, "index build: more than 2^24 blocks in one batch");
        CUDA_TRY(c, c->d_idx_first.ensure(nbits * 4));
        rc = index_first_init(c, ib.bits, c->d_idx_first.as<uint32_t>(), nbits, st);
        if (rc) return rc;
        rc = digest_block_host(c, host_data, offsets, lens, n, dd, out_filters, out_counts, res, nullptr, 0, nullptr,
                               &ib, c->d_idx_first.as<uint32_t>());
        if (rc) return rc;
    }
    unsigned long long added = 0;
    CUDA_TRY(c, cudaMemcpyAsync(index_bits, c->d_idx_bits.p, index_bytes, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaMemcpyAsync(&added, c->d_idx_count.p, 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaStreamSynchronize(st));
    *elem_count += added;
    return SDBFG_OK;
}

extern "C" int sdbfg_digest_batch_search(sdbfg_ctx* c, const uint8_t* host_data, const uint64_t* offsets,
                                         const uint64_t* lens, uint32_t n, uint32_t dd, uint8_t* out_filters,
                                         uint64_t out_cap, uint16_t* out_counts, sdbfg_digest_result* res,
                                         const sdbfg_index* const* indexes, uint32_t nidx, uint8_t* out_hits) {
    if (!dd) return fail(c, SDBFG_ERR_ARG, "index search needs block mode");  // sdhash.cc:241-244
    if (nidx && (!indexes || !out_hits)) return SDBFG_ERR_ARG;
    for (uint32_t i = 0; i < nidx; i++)
        if (!indexes[i] || indexes[i]->ctx != c) return fail(c, SDBFG_ERR_ARG, "index %u belongs to no/another context", i);
    int rc = validate_batch(c, offsets, lens, n, dd, res);
    if (rc) return rc;
    if (n && !host_data) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    const uint64_t total_slots = assign_block_slots(lens, n, dd, res);
    if (total_slots > out_cap)
        return fail(c, SDBFG_ERR_CAPACITY, "need %llu filter slots", (unsigned long long)total_slots);
    if (total_slots && !out_counts) return fail(c, SDBFG_ERR_ARG, "block mode needs element-count output");
    return digest_block_host(c, host_data, offsets, lens, n, dd, out_filters, out_counts, res, indexes, nidx, out_hits);
}


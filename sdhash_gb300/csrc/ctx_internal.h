// ctx_internal.h -- the context and digest-set objects behind the C ABI,
// shared by the generation (sdbf_api.cu) and comparison (compare_api.cu)
// host code.  Not part of the public interface.
#pragma once
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sdbf_gb300.h"
#include "compare_kernels.h"
#include "gen_kernels.h"

using namespace sdbfg;

namespace sdbfg_host {

constexpr uint32_t kMaxTilesPerLaunch = 1u << 18;  // 2 GiB of stream input per launch group
constexpr uint64_t kMaxBytesPerLaunch = 2ull << 30;
constexpr uint64_t kFirstHostGroupBytes = 256ull << 20;  // first group of a host-input stream batch
constexpr uint32_t kMinFile = 512;                 // MIN_FILE_SIZE (sdbf_defines.h:56)
constexpr uint64_t kPairsPerLaunch = 1ull << 22;
constexpr int kSlots = 8;  // stream-mode launch groups in flight (at most)
// pinned host-input stream batches up to this size (and half the free
// device memory) are staged whole on the device
constexpr uint64_t kStageMaxBytes = 64ull << 30;
constexpr uint64_t kStagePiece = 1ull << 20;  // work item of the staging gather
struct StagePiece {
    uint64_t dst;  // staging offset (16-byte aligned)
    uint64_t src;  // device address of the pinned host bytes
    uint64_t len;
};


// Device / pinned-host arrays that grow on demand and free themselves with
// their owner (not copyable).
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), cap(o.cap) {
        o.p = nullptr;
        o.cap = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            cap = o.cap;
            o.p = nullptr;
            o.cap = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        const size_t want = std::max(bytes, cap + cap / 2);
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    HostBuf() = default;
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
    HostBuf(HostBuf&& o) noexcept : p(o.p), cap(o.cap) {
        o.p = nullptr;
        o.cap = 0;
    }
    HostBuf& operator=(HostBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            cap = o.cap;
            o.p = nullptr;
            o.cap = 0;
        }
        return *this;
    }
    ~HostBuf() { release(); }
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMallocHost(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

}  // namespace sdbfg_host

using namespace sdbfg_host;

struct KernelTimer {
    const char* name;
    cudaEvent_t a, b;
};

struct KernelStat {
    std::string name;
    double ms = 0;
    uint64_t launches = 0;
};

struct sdbfg_ctx {
    bool profile = false;
    std::vector<KernelTimer> pending;
    std::vector<KernelStat> stats;
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    uint64_t launches = 0;
    int sms = 152;
    uint32_t lead = kDefaultLead;
    bool pre_ranks = true;  // stream mode: ranks by k_stream_ranks ahead of the tile kernel
    DevBuf d_ranks;         // their ranks (two halves, by launch-group parity)
    // constant tables
    DevBuf d_rank, d_ent, d_cut, d_cut64;
    // generation buffers
    DevBuf d_data, d_chunks, d_tiles, d_files, d_order, d_tile_out, d_features, d_work_filters, d_info, d_counters,
        d_pack_src, d_pack_dst_off, d_out_filters, d_out_counts;
    HostBuf h_stage;
    // comparison buffers
    DevBuf d_pairs, d_scores;
    // stream-mode pipeline: two launch-group slots on their own streams
    struct Slot {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        bool used = false;
        DevBuf data, chunks, tiles, files, order, tile_out, features, work, redo, fix_list;
        DevBuf rk_items;  // stretches of the group's chunks for k_stream_ranks
        HostBuf h_tables;
    } slot[kSlots];
    int depth = 4;  // launch groups in flight
    DevBuf d_binfo, d_boff, d_total, d_phase;
    // host-input stream batches staged whole on the device: per-file copies
    // in launch-group order on their own stream, one event per group
    DevBuf d_stage_in, d_stage_items;
    HostBuf h_stage_items;
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> ev_copy;
    cudaEvent_t ev_scan[kSlots] = {};
    cudaEvent_t ev_tiles[kSlots] = {};  // a group's tile kernels done
    cudaEvent_t ev_start = nullptr;
    // comparison engine: tuning and cached plans (work units + CUDA graph)
    int mat_variant = kMatVariantTc;  // tensor-core counting
    uint64_t mat_unit_work = 1ull << 22;
    bool mat_graphs = true;
    std::vector<struct MatPlan*> plans;
    DevBuf d_match_counts, d_match_offs, d_matches, d_mphase;
    // index search: per-slot probe words and counts of the group being
    // digested (set around a block-mode batch), the device index table
    uint32_t* probe_words = nullptr;
    uint8_t* probe_counts = nullptr;
    DevBuf d_probes, d_nprobes, d_hits, d_index_tab;
    // index build: counted features of the group being digested (block
    // mode), the index bits, the first setter of every bit, the new-insert count
    uint32_t* feat_words = nullptr;
    DevBuf d_feats, d_idx_bits, d_idx_first, d_idx_count;
    // stream-mode index build: fixed-point rounds before the sequential
    // commit takes over (0: sequential only), rounds the last launch group took
    uint32_t index_max_rounds = 16;
    uint32_t index_rounds_used = 0;
    DevBuf d_seen[2], d_pred, d_diff, d_ckpt, d_from;
};

// A resident index filter (bloom_filter of an index file).
struct sdbfg_index {
    sdbfg_ctx* ctx = nullptr;
    uint64_t bf_size = 0, elem_count = 0, bit_mask = 0;
    uint32_t hash_count = 0;
    std::string name;
    DevBuf d_bits;
};

// Block-mode index build over one launch group's slots [0, nslots) (global
// slots from slot0): each bit's first setter in input order, then the bits
// and the count of features that set a new one (bloom_filter::insert_sha1
// in that order, bloom_filter.cc:333-359).
int index_build_group(sdbfg_ctx* c, const uint32_t* d_feats, const uint16_t* d_counts, uint64_t nslots,
                      uint64_t slot0, uint32_t mask, uint32_t* d_first, uint32_t* d_bits,
                      unsigned long long* d_count, cudaStream_t st);
// first[p] = 0 for bits already set, ~0 otherwise.
int index_first_init(sdbfg_ctx* c, const uint32_t* d_bits, uint32_t* d_first, uint64_t nbits, cudaStream_t st);

// Hits of every probe slot against every index (k_index_query).
int index_query(sdbfg_ctx* c, const uint32_t* d_probes, const uint8_t* d_nprobes, uint64_t nslots,
                const sdbfg_index* const* indexes, uint32_t nidx, uint8_t* d_hits, cudaStream_t st);

struct sdbfg_set {
    sdbfg_ctx* ctx = nullptr;
    uint32_t n = 0;
    std::vector<std::string> names;
    std::vector<uint32_t> bf_count;
    std::vector<uint32_t> last_elem;  // element count of the last filter (swap rule)
    std::vector<uint8_t> fast;         // per digest: folded by sdbfg_set_fast
    // header fields of the SDBF text form (sdbf::to_string, sdbf_class.cc:293-334)
    std::vector<uint64_t> orig_size;
    std::vector<uint32_t> max_elem, last_count, dd_block;  // dd_block 0: stream digest
    uint64_t serial = 0;               // identifies the set in cached comparison plans
    uint64_t total_filters = 0;
    std::vector<uint32_t> first;       // first filter of each digest in d_filters
    DevBuf d_filters, d_meta, d_digests;
};

// Serial number of a new set (cached comparison plans are keyed by it).
uint64_t next_set_serial();

// A comparison job prepared for the matrix engine: work units sorted by
// size, the target list, split-pair table and slot array, and (once run) a
// CUDA graph of its launches.
struct MatPlan {
    uint64_t serial_a = 0, serial_b = 0;
    uint32_t mode = 0;
    int variant = 0;
    uint64_t unit_work = 0;
    uint32_t nunits = 0, nsplit = 0;
    uint64_t nscores = 0;
    uint64_t filter_pairs = 0;  // sum over scored pairs of n_ref * n_tgt
    DevBuf d_units, d_targets, d_refs, d_split, d_slots, d_counter;
    cudaGraphExec_t graph = nullptr;
    int32_t* graph_out = nullptr;
    cudaStream_t graph_stream = nullptr;
    uint64_t last_use = 0;
    ~MatPlan() {
        if (graph) cudaGraphExecDestroy(graph);
        for (DevBuf* b : {&d_units, &d_targets, &d_refs, &d_split, &d_slots, &d_counter}) b->release();
    }
};

// Per-kernel CUDA-event timing on the launch stream (only when enabled).
inline void timer_begin(sdbfg_ctx* c, const char* name, cudaEvent_t* a, cudaStream_t st) {
    *a = nullptr;
    if (!c->profile) return;
    cudaEventCreate(a);
    cudaEventRecord(*a, st);
    (void)name;
}

inline void timer_end(sdbfg_ctx* c, const char* name, cudaEvent_t a, cudaStream_t st) {
    if (!c->profile || !a) return;
    cudaEvent_t b;
    cudaEventCreate(&b);
    cudaEventRecord(b, st);
    c->pending.push_back({name, a, b});
}

inline void timer_collect(sdbfg_ctx* c) {
    for (KernelTimer& t : c->pending) {
        cudaEventSynchronize(t.b);
        float ms = 0;
        cudaEventElapsedTime(&ms, t.a, t.b);
        KernelStat* st = nullptr;
        for (KernelStat& k : c->stats)
            if (k.name == t.name) st = &k;
        if (!st) {
            c->stats.push_back(KernelStat{t.name, 0, 0});
            st = &c->stats.back();
        }
        st->ms += ms;
        st->launches += 1;
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    c->pending.clear();
}

#define TIMED_LAUNCH_ON(c, name, st_, expr)     \
    do {                                        \
        cudaEvent_t ev_;                        \
        timer_begin((c), (name), &ev_, (st_));  \
        cudaError_t le_ = (expr);               \
        timer_end((c), (name), ev_, (st_));     \
        if (le_ != cudaSuccess)                 \
            return fail((c), SDBFG_ERR_CUDA, "%s launch: %s", (name), cudaGetErrorString(le_)); \
        (c)->launches += 1;                     \
    } while (0)
#define TIMED_LAUNCH(c, name, expr) TIMED_LAUNCH_ON(c, name, (c)->stream, expr)

inline int fail(sdbfg_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CUDA_TRY(ctx, call)                                                                       \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? SDBFG_ERR_NOMEM : SDBFG_ERR_CUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);    \
    } while (0)


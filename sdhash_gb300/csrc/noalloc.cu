// noalloc.cu -- stream-mode digests for callers that cannot allocate GPU memory.
//
// Who needs this: code that runs where cudaMalloc is off limits -- inside a
// host callback or a framework that owns every device allocation (a custom
// allocator or memory pool it must not bypass), a signal-safe / real-time
// path that may not enter the driver's allocator, or a process with a fixed
// device-memory budget reserved up front.  Such a caller already holds its
// input and output buffers; this entry point takes those and allocates
// nothing, neither device memory nor host heap memory.
//
// The scratch the stream pipeline needs (work lists, per-tile features, the
// per-file filter workspace, the constant tables) lives in one file-scope
// __device__ array of fixed size, so every GPU that loads this library holds
// SDBFG_NOALLOC_SCRATCH_BYTES (14 MiB) of device memory until the process exits.  Its limits
// are stated in include/sdbf_gb300.h.  All calls share that one array: two
// calls whose work overlaps on the GPU (different host threads, or different
// streams without ordering between them) race on it and produce garbage.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/sdbf_gb300.h"
#include "gen_kernels.h"
#include "sdbf_tables.h"

using namespace sdbfg;

namespace {

constexpr uint32_t kMaxInputs = SDBFG_NOALLOC_MAX_INPUTS;
constexpr uint64_t kMaxBytes = SDBFG_NOALLOC_MAX_INPUT_BYTES;
// every input is at most kMaxBytes (< one 32 MiB chunk): one chunk per input;
// tiles: at most ceil((len-64)/8192) per input
constexpr uint32_t kMaxTiles = (uint32_t)(kMaxBytes / kTileL) + kMaxInputs;
constexpr uint64_t kMaxFilters = (kMaxBytes >> 11) + kMaxInputs;

constexpr uint64_t align256(uint64_t v) { return (v + 255) / 256 * 256; }

// scratch layout (byte offsets)
constexpr uint64_t kOffRank = 0;
constexpr uint64_t kOffEnt = align256(kOffRank + sizeof(uint16_t) * SDBF_RANK_BINS);
constexpr uint64_t kOffCounters = align256(kOffEnt + sizeof(uint32_t) * 65);
constexpr uint64_t kOffChunks = align256(kOffCounters + 64);
constexpr uint64_t kOffTiles = align256(kOffChunks + sizeof(GenChunk) * kMaxInputs);
constexpr uint64_t kOffFiles = align256(kOffTiles + sizeof(GenTile) * kMaxTiles);
constexpr uint64_t kOffOrder = align256(kOffFiles + sizeof(GenFile) * kMaxInputs);
constexpr uint64_t kOffInfo = align256(kOffOrder + sizeof(uint32_t) * kMaxInputs);
constexpr uint64_t kOffTileOut = align256(kOffInfo + sizeof(FileInfoDev) * kMaxInputs);
constexpr uint64_t kOffPack = align256(kOffTileOut + sizeof(TileOut) * kMaxTiles);
constexpr uint64_t kOffWork = align256(kOffPack + (8 + 8 + 4) * kMaxInputs);
constexpr uint64_t kOffRedo = align256(kOffWork + 256 * kMaxFilters);
constexpr uint64_t kOffFeat = align256(kOffRedo + sizeof(uint32_t) * kMaxInputs);
constexpr uint64_t kScratchBytes = align256(kOffFeat + 4ull * 5 * kTileCap * kMaxTiles);

static_assert(kScratchBytes <= SDBFG_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

}  // namespace

// The scratch array itself.  Host code may not use this name as an address
// (it is only a host-side stand-in); it obtains the device address with
// cudaGetSymbolAddress below.
static __device__ __align__(256) uint8_t g_noalloc_scratch[SDBFG_NOALLOC_SCRATCH_BYTES];

__global__ void k_noalloc_pack(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                               const uint64_t* __restrict__ src_off, const uint64_t* __restrict__ dst_off,
                               const uint32_t* __restrict__ words, uint32_t n) {
    for (uint32_t f = blockIdx.x; f < n; f += gridDim.x) {
        const uint4* s = reinterpret_cast<const uint4*>(src + src_off[f] * 64);
        uint4* d = reinterpret_cast<uint4*>(dst + dst_off[f] * 64);
        for (uint32_t q = threadIdx.x; q < words[f] / 4; q += blockDim.x) d[q] = s[q];
    }
}

namespace {

std::mutex g_setup_mutex;
uint8_t* g_scratch_dev[64];  // per device id: device address of g_noalloc_scratch
int g_sms[64];

// Once per device, with that device current: resolve the array's device
// address and load the constant tables into it.  The address and the tables
// belong to the device's context at that time: after cudaDeviceReset (or
// anything else that destroys the primary context) they are stale, so the
// entry point must not be called again in that process.
int setup_device(int dev, uint8_t** base, int* sms) {
    if (dev < 0 || dev >= 64) return SDBFG_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_dev[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "sdbfg_digest_stream_noalloc: cudaGetSymbolAddress failed: %s\n",
                    cudaGetErrorString(e));
            return SDBFG_ERR_CUDA;
        }
        uint8_t* b = static_cast<uint8_t*>(p);
        uint32_t ent[65];
        for (int i = 0; i < 65; i++) ent[i] = SDBF_ENTROPY64[i];
        if (cudaMemcpy(b + kOffRank, SDBF_ENTR64_RANKS, sizeof(SDBF_ENTR64_RANKS), cudaMemcpyHostToDevice) !=
                cudaSuccess ||
            cudaMemcpy(b + kOffEnt, ent, sizeof(ent), cudaMemcpyHostToDevice) != cudaSuccess)
            return SDBFG_ERR_CUDA;
        int n = 152;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_sms[dev] = n;
        g_scratch_dev[dev] = b;
    }
    *base = g_scratch_dev[dev];
    *sms = g_sms[dev];
    return SDBFG_OK;
}

}  // namespace

extern "C" int sdbfg_digest_stream_noalloc(const uint8_t* dev_data, const uint64_t* offsets, const uint64_t* lens,
                                           uint32_t n, uint8_t* dev_out_filters, uint64_t out_cap,
                                           sdbfg_digest_result* results, void* cuda_stream) {
    if ((n && (!dev_data || !offsets || !lens || !results || !dev_out_filters))) return SDBFG_ERR_ARG;
    if (n > kMaxInputs) {
        fprintf(stderr, "sdbfg_digest_stream_noalloc: %u inputs exceed the limit of %u\n", n, kMaxInputs);
        return SDBFG_ERR_CAPACITY;
    }
    // each length is checked before it is added, so no sum of huge lengths
    // can wrap below the limit
    uint64_t total = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (offsets[i] % 16) return SDBFG_ERR_ARG;
        if (lens[i] > kMaxBytes - total) {
            fprintf(stderr, "sdbfg_digest_stream_noalloc: inputs 0..%u hold more than the limit of %llu bytes\n", i,
                    (unsigned long long)kMaxBytes);
            return SDBFG_ERR_CAPACITY;
        }
        total += lens[i];
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SDBFG_ERR_CUDA;
    uint8_t* base = nullptr;
    int sms = 152;
    int rc = setup_device(dev, &base, &sms);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);

    // work lists in fixed-size host arrays (no heap)
    GenChunk chunks[kMaxInputs];
    GenFile files[kMaxInputs];
    uint32_t order[kMaxInputs];
    GenTile tiles[kMaxTiles];  // ~10 KB of stack
    uint32_t nchunks = 0, ntiles = 0;
    uint64_t work = 0;
    for (uint32_t i = 0; i < n; i++) {
        results[i] = sdbfg_digest_result{};
        GenFile f{nchunks, 0, work, 0};
        if (lens[i] < 512) {
            results[i].status = SDBFG_DIGEST_TOO_SMALL;
        } else {
            const uint32_t m = (uint32_t)lens[i];
            GenChunk ch{offsets[i], m, i, ntiles, 0, 0, 0};
            for (uint32_t t0 = 0; t0 < m - 64; t0 += kTileL) tiles[ntiles++] = GenTile{nchunks, t0};
            ch.ntiles = ntiles - ch.first_tile;
            chunks[nchunks++] = ch;
            f.nchunks = 1;
            f.filter_cap = (lens[i] >> 11) + 1;
            work += f.filter_cap;
        }
        files[i] = f;
        order[i] = i;
    }
    // largest first, insertion sort (n <= kMaxInputs)
    for (uint32_t a = 1; a < n; a++) {
        const uint32_t v = order[a];
        uint32_t b = a;
        while (b > 0 && lens[order[b - 1]] < lens[v]) {
            order[b] = order[b - 1];
            b--;
        }
        order[b] = v;
    }
#define NA_TRY(call)                                      \
    do {                                                  \
        if ((call) != cudaSuccess) return SDBFG_ERR_CUDA; \
    } while (0)
    // what must start at zero: the counters and the per-file results
    NA_TRY(cudaMemsetAsync(base + kOffCounters, 0, 64, st));
    NA_TRY(cudaMemsetAsync(base + kOffInfo, 0, sizeof(FileInfoDev) * kMaxInputs, st));
    if (nchunks) NA_TRY(cudaMemcpyAsync(base + kOffChunks, chunks, sizeof(GenChunk) * nchunks, cudaMemcpyHostToDevice, st));
    if (ntiles) NA_TRY(cudaMemcpyAsync(base + kOffTiles, tiles, sizeof(GenTile) * ntiles, cudaMemcpyHostToDevice, st));
    if (n) {
        NA_TRY(cudaMemcpyAsync(base + kOffFiles, files, sizeof(GenFile) * n, cudaMemcpyHostToDevice, st));
        NA_TRY(cudaMemcpyAsync(base + kOffOrder, order, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
    }
    GenParams P{};
    P.data = dev_data;
    P.chunks = reinterpret_cast<const GenChunk*>(base + kOffChunks);
    P.nchunks = nchunks;
    P.tiles = reinterpret_cast<const GenTile*>(base + kOffTiles);
    P.ntiles = ntiles;
    P.files = reinterpret_cast<const GenFile*>(base + kOffFiles);
    P.file_order = reinterpret_cast<const uint32_t*>(base + kOffOrder);
    P.nfiles = n;
    P.tile_out = reinterpret_cast<TileOut*>(base + kOffTileOut);
    P.features = reinterpret_cast<uint32_t*>(base + kOffFeat);
    P.out_filters = reinterpret_cast<uint32_t*>(base + kOffWork);
    P.out_info = reinterpret_cast<FileInfoDev*>(base + kOffInfo);
    P.counters = reinterpret_cast<uint32_t*>(base + kOffCounters);
    P.rank_tab = reinterpret_cast<const uint16_t*>(base + kOffRank);
    P.ent_tab = reinterpret_cast<const uint32_t*>(base + kOffEnt);
    P.chunk_redo = reinterpret_cast<uint32_t*>(base + kOffRedo);
    P.lead = kDefaultLead;
    const uint32_t cap3 = (uint32_t)sms * 3 * 16;
    if (ntiles) NA_TRY(launch_stream_tiles(P, ntiles < cap3 ? ntiles : cap3, st));
    if (nchunks) NA_TRY(launch_stream_check(P, (nchunks + 3) / 4, st));
    if (nchunks) NA_TRY(launch_stream_fix(P, nchunks < cap3 ? nchunks : cap3, st));
    if (n) NA_TRY(launch_stream_commit(P, (n + kCommitWarps - 1) / kCommitWarps, st));
    FileInfoDev info[kMaxInputs];
    uint32_t flags[2] = {0, 0};
    if (n) NA_TRY(cudaMemcpyAsync(info, base + kOffInfo, sizeof(FileInfoDev) * n, cudaMemcpyDeviceToHost, st));
    NA_TRY(cudaMemcpyAsync(flags, base + kOffCounters, sizeof flags, cudaMemcpyDeviceToHost, st));
    NA_TRY(cudaStreamSynchronize(st));
    if (flags[1]) return SDBFG_ERR_CUDA;
    // pack every digest's filters into the caller's output
    uint64_t src_off[kMaxInputs], dst_off[kMaxInputs];
    uint32_t words[kMaxInputs];
    uint32_t np = 0;
    uint64_t next = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (results[i].status) continue;
        results[i].bf_count = info[i].bf_count;
        results[i].last_count = info[i].last_count;
        results[i].filter_offset = next;
        src_off[np] = files[i].filter_base;
        dst_off[np] = next;
        words[np] = info[i].bf_count * 64;
        np++;
        next += info[i].bf_count;
    }
    if (next > out_cap) {
        fprintf(stderr, "sdbfg_digest_stream_noalloc: output holds %llu filters, %llu needed\n",
                (unsigned long long)out_cap, (unsigned long long)next);
        return SDBFG_ERR_CAPACITY;
    }
    if (np) {
        uint64_t* d_src = reinterpret_cast<uint64_t*>(base + kOffPack);
        uint64_t* d_dst = d_src + kMaxInputs;
        uint32_t* d_words = reinterpret_cast<uint32_t*>(d_dst + kMaxInputs);
        NA_TRY(cudaMemcpyAsync(d_src, src_off, 8 * np, cudaMemcpyHostToDevice, st));
        NA_TRY(cudaMemcpyAsync(d_dst, dst_off, 8 * np, cudaMemcpyHostToDevice, st));
        NA_TRY(cudaMemcpyAsync(d_words, words, 4 * np, cudaMemcpyHostToDevice, st));
        k_noalloc_pack<<<np, 256, 0, st>>>(reinterpret_cast<const uint32_t*>(base + kOffWork),
                                          reinterpret_cast<uint32_t*>(dev_out_filters), d_src, d_dst, d_words, np);
        NA_TRY(cudaGetLastError());
        NA_TRY(cudaStreamSynchronize(st));
    }
#undef NA_TRY
    return SDBFG_OK;
}

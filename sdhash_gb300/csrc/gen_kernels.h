// gen_kernels.h -- work descriptors shared by the host orchestration
// (sdbf_api.cu) and the generation kernels (gen_kernels.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace sdbfg {

constexpr int kGenThreads = 128;     // CTA size of the tile / block kernels
constexpr int kRankThreads = 96;     // threads computing ranks: 3 full warps, each lane owning
                                     // a 256-byte histogram in its own bank
constexpr int kSegs = 128;           // popularity-chain segments per tile (one per thread)
constexpr uint32_t kLead = 128;      // maximum speculative lead-in steps per segment
constexpr uint32_t kDefaultLead = 64; // default lead-in (measured best of 16..128 on the bulk stream
                                     // workload); mis-speculated segments are re-walked only until
                                     // their chain meets the speculative one
// window steps owned by a stream tile: with the 64-step credit halo and the
// 128-step maximum lead-in a tile simulates 8128 steps (127 aligned 64-step
// blocks, one per thread of the full-rescan table)
constexpr uint32_t kTileL = 7936;
// at most one selected feature per 17 credited steps (score > 16), and a
// tile's positions are credited by kTileL + 64 steps
constexpr uint32_t kTileCap = ((kTileL + 64) / 17 + 2 + 3) / 4 * 4;  // rows 16-byte aligned
constexpr int kCommitWarps = 1;      // files per commit CTA (one: its 44 KB of shared memory then
                                     // displaces a single tile CTA on its SM)
constexpr uint32_t kMaxBlockBytes = 16384;  // dd block size limit (sdhash.cc:215-219)
constexpr uint64_t kChunkBytes = 32ull << 20;  // stream chunk (sdbf_class.cc:43)

// One 32 MiB stream chunk (or the tail of a file), or one dd block.
struct GenChunk {
    uint64_t data_off;    // byte offset of the chunk in the batch buffer (16-aligned for stream)
    uint32_t n;           // bytes
    uint32_t file;        // owning file
    uint32_t first_tile;  // stream: first tile id
    uint32_t ntiles;      // stream: tiles of this chunk
    uint32_t filter;      // block: output filter index
    uint32_t kind;        // block: 0 full block (histogram threshold), 1 tail (16 / 192)
    uint32_t rank_off8;   // stream, ranks precomputed: the chunk's first rank in GenParams::ranks / 8
};

// Precomputed ranks of a stream launch group: k_stream_ranks gives each CTA
// kRkThreads x kRkPer consecutive positions of one chunk (a "stretch"); one
// work item (chunk, first position) per stretch.
constexpr int kRkThreads = 128;
constexpr uint32_t kRkPer = 312;  // positions per thread: a multiple of 8 whose word count (78) is
                                  // 2 mod 4, so a warp's byte-word reads are at most 2-way bank
                                  // conflicts; 73.3 KB per CTA still fits three CTAs per SM
constexpr uint32_t kRkSpan = kRkThreads * kRkPer;

struct GenTile {
    uint32_t chunk;
    uint32_t t0;  // first owned step (multiple of kTileL)
};

struct GenFile {
    uint32_t first_chunk;
    uint32_t nchunks;
    uint64_t filter_base;  // first output filter slot of this file
    uint64_t filter_cap;   // slots reserved for it ((len >> 11) + 1)
};

struct TileOut {
    uint64_t sig_in;   // speculative chain state entering step t0-64
    uint64_t tau_out;  // chain state entering step t0+kTileL-64
    uint32_t count;    // features selected in the tile
    uint32_t fixups;   // segments re-walked inside the tile
};

struct FileInfoDev {
    uint32_t bf_count;
    uint32_t last_count;
};

struct GenParams {
    const uint8_t* data;
    const GenChunk* chunks;
    uint32_t nchunks;
    const GenTile* tiles;
    uint32_t ntiles;
    const GenFile* files;
    const uint32_t* file_order;  // commit order (largest first)
    uint32_t nfiles;
    TileOut* tile_out;
    uint32_t* features;          // [tile][5][kTileCap]
    uint32_t* out_filters;       // 64 words per filter
    uint16_t* out_counts;        // block mode: elements per filter
    FileInfoDev* out_info;       // stream mode: per file
    uint32_t* counters;          // [0] tiles recomputed by the link check, [1] capacity overflows
    const uint16_t* rank_tab;    // device copy of SDBF_ENTR64_RANKS
    const uint32_t* ent_tab;     // device copy of SDBF_ENTROPY64
    uint32_t block_lmax;         // block mode: max window steps per block
    uint32_t lead;               // speculative lead-in steps (<= kLead)
    unsigned long long* phase;   // optional phase cycle counters (kPhase*), null = off
    uint32_t* chunk_redo;        // per chunk: first tile whose link failed (stream)
    uint32_t* fix_list;          // stream: [0] = n, then the n tiles whose link failed
    // block mode with index search: SHA-1 words of every fourth counted
    // feature of each block ([slot][kProbeWords]) and their number per slot;
    // null = no search
    uint32_t* probes;
    uint8_t* nprobes;
    // index build: stream mode inserts into index_bits (mask index_mask) and
    // counts the inserts that set a new bit in *index_new; block mode
    // records every counted feature's SHA-1 words in feats ([slot][kFeatWords])
    uint32_t* index_bits;
    uint32_t index_mask;
    unsigned long long* index_new;
    uint32_t* feats;
    // stream-mode index build by fixed-point rounds, bitmaps by feature
    // ordinal (tile * kTileCap + feature): index_pred -- the feature owns the
    // first setting of one of its index bits among the previous round's
    // inserted features (k_stream_index_pred); index_seen -- this round's
    // inserted features
    const uint32_t* index_pred;
    uint32_t* index_seen;
    // rounds after the first: only files flagged here commit again (their
    // seen bits are cleared first); null = every file.  commit_from: the
    // first feature ordinal whose predicate changed, per file; a file
    // restarts from the checkpoint (commit_ckpt, one per kCkptTiles tiles)
    // at or before it
    const uint8_t* commit_dirty;
    const uint32_t* commit_from;
    uint32_t* commit_ckpt;
    // stream mode with ranks precomputed by k_stream_ranks (null: the tile
    // kernel computes them itself): ranks of every chunk position, 16-byte
    // aligned per chunk (GenChunk::rank_off8), and the stretches to compute
    uint16_t* ranks;
    const uint2* rk_items;
    uint32_t nrk_items;
};

// Index search samples counted features 0, 4, 8, ... of a block
// (sdbf_core.cc:168-175): at most 192 / 4 = 48, five words each.
constexpr uint32_t kProbeWords = 48 * 5;
// Index build in block mode: up to 192 counted features per block, five words each.
constexpr uint32_t kFeatWords = 192 * 5;

// Phase counters (cycles summed over CTAs / warps) when GenParams::phase is set.
enum : int {
    kPhLoad = 0, kPhRanks, kPhFres, kPhWalk, kPhLink, kPhCompact, kPhSha, kPhTiles,
    kPhCommitWait, kPhCommitBusy, kPhCommitGroups, kPhCommitLoops, kPhCommitMaxFile, kPhFixups,
    kPhCkptRestarts, kPhCount
};

size_t stream_tile_smem();
size_t block_smem(uint32_t lmax);
// Ranks of every position of the group's chunks into P.ranks (P.rk_items stretches).
cudaError_t launch_stream_ranks(const GenParams& P, uint32_t grid, cudaStream_t st);
// Tile kernels: with P.ranks set they read the precomputed ranks (and the
// feature bytes from the input in global memory), else they compute ranks.
cudaError_t launch_stream_tiles(const GenParams& P, uint32_t grid, cudaStream_t st);
// Tiles whose link fails into P.fix_list (zeroed count first), then all of
// them recomputed in parallel; k_stream_check / k_stream_fix finish the job.
cudaError_t launch_stream_fails(const GenParams& P, uint32_t grid, cudaStream_t st);
cudaError_t launch_stream_fix_list(const GenParams& P, uint32_t grid, cudaStream_t st);
cudaError_t launch_stream_check(const GenParams& P, uint32_t grid, cudaStream_t st);  // 4 chunks per CTA
cudaError_t launch_stream_fix(const GenParams& P, uint32_t grid, cudaStream_t st);
cudaError_t launch_stream_commit(const GenParams& P, uint32_t grid, cudaStream_t st);
// One warp, files in file_order, index inserts (GenParams::index_bits).
cudaError_t launch_stream_commit_index(const GenParams& P, cudaStream_t st);
// One fixed-point round of a stream-mode index build: files in parallel,
// index acceptance read from GenParams::index_pred, inserted features
// recorded in GenParams::index_seen.
cudaError_t launch_stream_commit_round(const GenParams& P, uint32_t grid, cudaStream_t st);
// pred bit of every feature ordinal: first[bit] >= ordinal + 1 for one of
// its index bits (no earlier first setter).
cudaError_t launch_stream_index_pred(const GenParams& P, const uint32_t* first, uint32_t* pred, uint32_t grid,
                                     cudaStream_t st);
// first[bit] = min(first[bit], ordinal + 1) over the features in seen.
cudaError_t launch_stream_index_first(const GenParams& P, const uint32_t* seen, uint32_t* first, uint32_t grid,
                                      cudaStream_t st);
// Index bits of the features in seen; *index_new += those that own the
// first setting of one of their bits.
cudaError_t launch_stream_index_mark(const GenParams& P, const uint32_t* seen, const uint32_t* first, uint32_t grid,
                                     cudaStream_t st);
// dirty[file] = 1 for every file with a feature whose predicate bit
// differs between pred words a and b (nwords words).  *ndirty is only a
// nonzero flag: it is zero iff no file was flagged (racing threads may add
// more than once for the same file, so it is not a file count).
cudaError_t launch_pred_dirty(const GenParams& P, const uint32_t* a, const uint32_t* b, uint64_t nwords,
                              uint8_t* dirty, uint32_t* from, unsigned int* ndirty, uint32_t grid, cudaStream_t st);
// Commit-state checkpoints of the index rounds: every kCkptTiles tiles the
// 256-byte filter, the big filter and bf_count / last_count / big-filter count.
constexpr uint32_t kCkptTiles = 32;
constexpr uint32_t kCkptWords = 64 + 4096 + 4;
cudaError_t launch_block(const GenParams& P, uint32_t grid, cudaStream_t st);

}  // namespace sdbfg

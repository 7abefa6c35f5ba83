// wrs_internal.cuh -- device data layout and kernel launchers shared by the .cu files.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "wrs_device.cuh"

struct wrs_batch;

namespace wrs {

// Tile geometry of the decoupled-lookback kernels: 256 threads x 16 items.
constexpr int kTileThreads = 256;
constexpr int kTileWarps = kTileThreads / 32;
constexpr int kTileItems = 4096;
constexpr int kWarpItems = kTileItems / kTileWarps;  // 512 contiguous items per warp

// Split+pack: one split per thread (two bisections interleaved per thread measured slower on
// GB300 at N = 2^26: the kernel is issue-bound); kSplitSlots - kSplitLook - 1 subproblems
// packed per CTA, the remaining slots hold look-ahead splits (see k_split_pack).
constexpr int kSplitThreads = 512;
constexpr int kSplitPerThread = 1;
constexpr int kSplitSlots = kSplitThreads * kSplitPerThread;
constexpr int kSplitLook = 32;
constexpr int kSplitPack = kSplitSlots - kSplitLook - 1;

// Alias sampling: 256 threads x 4 samples per CTA.
constexpr int kSampleThreads = 256;
constexpr int kAliasPerThread = 4;
constexpr int kAliasPerBlock = kSampleThreads * kAliasPerThread;

// Ticket / completion / epoch of one lookback kernel kind.  The epoch selects which half
// of that kernel's double-buffered state array is live in the current launch.
struct LbCtrl {
    uint32_t ticket;  // tile tickets handed out in the current launch
    uint32_t done;    // CTAs finished in the current launch
    uint32_t epoch;
    uint32_t pad;
};

// Per-distribution control block (device memory, zero-initialised once at allocation).
// Every counter below is returned to zero by the last CTA of the kernel that used it,
// so successive builds (and CUDA-graph replays) need no memset.
struct alignas(64) BuildCtrl {
    uint32_t mass_done;  // tiles finished in the total-mass reduction
    uint32_t status;     // kStatus* bits raised by the device
    uint32_t heavy_count;
    float mean;          // (float)(total / N)
    double total;        // FP64 total mass
    LbCtrl part;         // prefix-partition launches
    LbCtrl scan;         // scan launches
    double mean64;       // total / N in FP64
    float mean_lo;       // (float)(mean64 - mean): mean64 as the float-float pair (mean, mean_lo)
    uint32_t pad0;
    unsigned long long coin_sum;  // sum of the table's coin-filter codes (k_coin_filter)
    uint32_t pad[12];
};
static_assert(sizeof(BuildCtrl) == 128, "BuildCtrl layout");

// Lookback state of one tile of the prefix-partition (128 B, 16 words).
//  compensated modes (exact fixed-point carries, two 63-bit limbs per sum):
//    agg heavy {0,1}, agg light {2,3}, agg count 4, incl count 6, incl heavy {8,9},
//    incl light {10,11}
//  FP32 mode (ff words): agg {0: heavy, 1: light}, agg count 4, incl count 6,
//    incl {8: heavy, 9: light}
struct alignas(128) PartState {
    unsigned long long q[16];
};
// Lookback state of one tile of the scan (32 B).  FP32 mode: q[0] = aggregate, q[1] =
// inclusive prefix (ff words).  Compensated mode: q[0..1] = aggregate, q[2..3] = inclusive
// prefix (fixed-point limbs).
struct alignas(32) ScanState {
    unsigned long long q[4];
};

// One distribution of a batch (device copy of wrs_dist_desc plus its place in the
// batch's tile, split and sampling grids).
struct alignas(64) DistDesc {
    const float* w;     // weights, nullptr: the table is already built
    uint2* table;       // alias table (n entries)
    uint32_t* out;      // samples, nullptr: build only
    uint64_t s;         // samples to draw
    uint64_t seed;
    uint64_t base;      // offset of this distribution in the batch's partition arrays
    uint32_t n;
    uint32_t tile0;     // first partition / total-mass tile (batch numbering)
    uint32_t split0;    // first split-pack CTA
    uint32_t sample0;   // first sampling CTA
};
static_assert(sizeof(DistDesc) == 64, "DistDesc layout");

// Device view of a batch, passed by value to the batched kernels.
struct BatchView {
    const DistDesc* dist;
    const uint32_t* tile_map;    // tile -> distribution
    const uint32_t* split_map;   // split-pack CTA -> distribution
    const uint32_t* sample_map;  // sampling CTA -> distribution
    BuildCtrl* dctrl;            // per distribution
    LbCtrl* lb;                  // partition tickets of the batch
    uint32_t* status;            // batch status word
    PartState* states;
    double* partials;            // per tile
    uint32_t* idx;               // partition arrays, distribution d at dist[d].base
    float* prefix;
    float* elems;                // nullptr: gather w[idx]
    float* prefix_lo;            // float-float mode only
    uint32_t cap_tiles;
    uint32_t tiles, split_blocks, sample_blocks;  // grid sizes of the three launches
    uint32_t split_size;
    uint32_t full_light;
    int2* descent;               // per split-pack CTA: the shared top of its bisections
};

// Grids up to this many CTAs (about one wave of 256-thread CTAs on the device) are launched
// with programmatic stream serialization; larger ones are launched plainly.  Measured on
// GB300: the small configuration's per-call build takes 20.2 us with it against 24.6 us
// without and its sampling 6.3 against 8.2 us, while a build of 2^26 weights takes 1.20
// against 1.13 ms and a batch graph of 4096 distributions 15.8 against 10.8 ms -- the early
// scheduled CTAs of a many-wave kernel cost more than the launch gap they hide.
constexpr uint64_t kPdlMaxGrid = 2048;

// Launches `kernel` (which starts with pdl_entry()) with programmatic stream serialization
// when its grid is at most kPdlMaxGrid CTAs: it may then be scheduled before its predecessor
// in the stream has finished.
template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    const uint64_t ctas = static_cast<uint64_t>(grid.x) * grid.y * grid.z;
    cfg.numAttrs = ctas <= kPdlMaxGrid ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// ---- launchers (defined in wrs_build.cu / wrs_sample.cu) -------------------------
cudaError_t launch_total_mass(cudaStream_t st, const float* w, uint32_t n, double* partials,
                              BuildCtrl* ctrl);
cudaError_t launch_prefix_partition(cudaStream_t st, bool comp, const float* w, uint32_t n,
                                    BuildCtrl* ctrl, PartState* states, uint32_t cap_tiles,
                                    uint32_t* idx_out, float* prefix_out, float* elems_out,
                                    float* prefix_lo_out);
// comp: runs k_total_mass first (into `partials`, >= tiles_for(n) doubles) for the grid of the
// exact carries
cudaError_t launch_scan(cudaStream_t st, bool comp, const float* in, uint32_t n, float* out,
                        BuildCtrl* ctrl, ScanState* states, uint32_t cap_tiles, double* partials,
                        uint32_t spin_limit = kSpinLimit);
// block-wise (reduce-then-scan) baselines; tile_scratch: 1 (scan) or 3 (partition) words per
// tile
cudaError_t launch_prefix_sum_blockwise(cudaStream_t st, const float* in, uint32_t n, float* out,
                                        float* tile_scratch);
cudaError_t launch_prefix_partition_blockwise(cudaStream_t st, const float* w, uint32_t n,
                                              BuildCtrl* ctrl, uint32_t* tile_scratch,
                                              uint32_t* idx_out, float* prefix_out,
                                              float* elems_out);
// ScalarSplit's record (split/scalar/shader.comp:12-16, std430: 12 bytes)
struct SplitRecord {
    uint32_t i, j;
    float spill;
};
static_assert(sizeof(SplitRecord) == 12, "split record layout");
// serial split-pack: records_for(n, s) = ceil(n / s) records (the last is (lc, hc, 0))
cudaError_t launch_split_records(cudaStream_t st, bool r64, bool full_light, const float* prefix,
                                 const float* prefix_lo, const BuildCtrl* ctrl, uint32_t n,
                                 uint32_t split_size, SplitRecord* records);
// full_light: the table-end rule of the full light cap (the current heavy stays in the heavy
// range), as the split-pack with split_full_light
cudaError_t launch_pack_records(cudaStream_t st, bool full_light, const float* w,
                                const uint32_t* idx, const float* elems, const BuildCtrl* ctrl,
                                uint32_t* status, uint32_t n, uint32_t split_size,
                                const SplitRecord* records, uint2* table);
cudaError_t launch_pack_records_warp(cudaStream_t st, bool full_light, const float* w,
                                     const uint32_t* idx, const float* elems,
                                     const BuildCtrl* ctrl, uint32_t* status, uint32_t n,
                                     uint32_t split_size, const SplitRecord* records,
                                     uint2* table);
// descent: scratch of descent_entries(n) int2 (or null: every bisection starts at the top)
__host__ __device__ inline uint32_t descent_entries(uint32_t max_n) {
    return max_n / kSplitPack + 2u;  // split blocks at split size 1, and more
}
cudaError_t launch_split_pack(cudaStream_t st, bool r64, bool full_light, const float* w,
                              const uint32_t* idx, const float* elems, const float* prefix,
                              const float* prefix_lo, const BuildCtrl* ctrl, uint32_t* status,
                              uint32_t n, uint32_t split_size, uint2* table, int2* descent);
// coins / coin_sum: the table's coin filter and the sum of its codes (k_coin_filter), or
// nullptr; samples are the same either way
cudaError_t launch_alias_sample(cudaStream_t st, uint32_t rng, uint32_t coop, const uint2* table,
                                const uint8_t* coins, const unsigned long long* coin_sum,
                                uint32_t n, uint64_t s, uint64_t seed, uint64_t offset,
                                uint32_t* out);
// the filter and, into *coin_sum (zeroed first, on the stream), the sum of its codes
cudaError_t launch_coin_filter(cudaStream_t st, const uint2* table, uint32_t n, uint8_t* coins,
                               unsigned long long* coin_sum);
// Tables of kCoinMinN < n <= kCoinMaxN weights get a coin filter (n bytes): a smaller table
// stays in L2 by itself, and a larger filter would not.  The sampler consults it when the
// codes average at least kCoinMinMean (out of 255): then at most ~78 % of the samples read
// their entry.  Measured at N = 2^26 on a box whose plain sampler takes 5.13 ms for 2^28
// samples, the filtered one took 0.66 + 5.45 f ms with f the share of samples reading their
// entry (f = 0.42 uniform, 0.75 log-normal(0, 2), 0.88 Zipf(1.1): 2.94 / 4.77 / 5.59 ms); on a
// box whose plain sampler takes 3.77 ms the uniform table took 2.56 ms and the log-normal one
// 4.06 ms, so tables near the threshold gain on the one and lose on the other.
constexpr uint32_t kCoinMinN = 1u << 22;
constexpr uint32_t kCoinMaxN = 1u << 26;
constexpr uint64_t kCoinMinMean = 56;
// The non-cooperative ITS sampler's bisection probes one implicit binary tree (node k, root
// 1: the range left by the decisions spelled by the bits of k below its leading one).  The
// build stores the tree's levels as blocks of three levels -- a node and its 6 descendants, 7
// probe values (slot 7: the node's range start) in one 32-byte sector -- so that one random
// read resolves three levels.  Block level b holds the 8^b blocks rooted at the nodes of tree
// level 3b, after the blocks of the levels above it.  The tree sampler keeps the top kTreeTop
// levels in each CTA's shared memory and reads the B block levels below them; a bisection
// outside that kernel (the cell search's fallback) reads all B + kTopBlockLevels of them.
constexpr uint32_t kTreeTop = 12;
constexpr uint32_t kTreeBlockLevels = 3;
constexpr uint32_t kTopBlockLevels = kTreeTop / kTreeBlockLevels;  // tree levels 0 .. 11
struct alignas(32) TreeBlock {
    float v[8];
};
static_assert(sizeof(TreeBlock) == 32, "one probe-tree block is one 32-byte sector");
// levels of the bisection of n values: ceil(log2 n)
__host__ __device__ inline uint32_t its_tree_depth(uint32_t n) {
    uint32_t t = 0;
    while (t < 32u && (1ull << t) < n) ++t;
    return t;
}
// block levels below the shared ones stored for n values (B): after them the bisection's range
// holds at most 16 values (a 64-byte stretch of the CMF), and all blocks take at most ~2/7 of
// the CMF's bytes
__host__ __device__ inline uint32_t its_tree_block_levels(uint32_t n) {
    const uint32_t t = its_tree_depth(n);
    return t >= kTreeTop + 5u ? (t - kTreeTop - 2u) / kTreeBlockLevels : 0u;
}
// block levels stored in all (the top ones too), 0 when none below the shared levels
__host__ __device__ inline uint32_t its_tree_stored_levels(uint32_t n) {
    const uint32_t B = its_tree_block_levels(n);
    return B ? B + kTopBlockLevels : 0u;
}
// blocks in the first L block levels (from the root)
__host__ __device__ constexpr size_t its_tree_blocks(uint32_t L) {
    size_t s = 0;
    for (uint32_t b = 0; b < L; ++b) s += size_t(1) << (kTreeBlockLevels * b);
    return s;
}
// blocks of the levels the shared memory holds (1 + 8 + 64 + 512)
constexpr size_t kTopBlocks = 585;
// stores the first L block levels (its_tree_stored_levels(n)) of the CMF's probe tree
cudaError_t launch_its_tree(cudaStream_t st, const float* cmf, uint32_t n, uint32_t L,
                            TreeBlock* blocks);
cudaError_t launch_its_sample(cudaStream_t st, uint32_t rng, uint32_t coop, bool parray,
                              const float* cmf, uint32_t n, uint64_t S, uint64_t seed,
                              uint64_t offset, uint32_t* out, const TreeBlock* blocks = nullptr,
                              uint32_t B = 0);

cudaError_t launch_cutpoint_guide(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                                  uint32_t* guide);
// the same table for an exactly non-decreasing CMF (galloping searches)
// (coarse: scratch of coarse_entries(G) + group_entries(G) words: every kCoarseStride-th
// entry, then every 32nd, bracketing the searches of the others)
constexpr uint32_t kCoarseStride = 1024;
__host__ __device__ inline uint32_t coarse_entries(uint32_t G) {
    return (G + kCoarseStride - 1) / kCoarseStride + 1;
}
// starts of the groups of 32 cells (the third pass's brackets), after the coarse ones
__host__ __device__ inline uint32_t group_entries(uint32_t G) { return (G + 31u) / 32u + 1u; }
cudaError_t launch_guide_monotone(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                                  uint32_t* coarse, uint32_t* guide);
// ITS on a non-decreasing CMF through cell blocks: cell k of G equal-mass cells (the Cutpoint
// guiding table's) = its candidate range [x, y] and the CMF at the last index of each of the
// range's kCellParts parts of d = ceil((y - x + 1) / kCellParts) indices; one 32-byte sector
constexpr int kCellParts = 6;
struct alignas(32) ItsCell {
    uint32_t x, y;
    float v[kCellParts];
};
static_assert(sizeof(ItsCell) == 32, "one cell block is one 32-byte sector");
cudaError_t launch_its_cells(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                             uint32_t* coarse, ItsCell* cells, bool check = false);
cudaError_t launch_its_sample_cells(cudaStream_t st, uint32_t rng, const float* cmf, uint32_t n,
                                    const ItsCell* cells, uint32_t G, uint64_t S, uint64_t seed,
                                    uint64_t offset, uint32_t* out,
                                    const TreeBlock* blocks = nullptr, uint32_t L = 0);
// FP32 CMF: marks the cells whose targets can meet a decrease of the CMF (bit 31 of y), after
// launch_its_cells with check (which marks the cells whose start is not below c_k);
// tile_scratch: 2 * tiles_for(n) floats; bad: a device word (set when every cell is marked)
cudaError_t launch_its_marks(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                             ItsCell* cells, float* tile_scratch, uint32_t* bad);
cudaError_t launch_cutpoint_sample(cudaStream_t st, uint32_t rng, const float* cmf, uint32_t n,
                                   const uint32_t* guide, uint32_t G, uint64_t S, uint64_t seed,
                                   uint64_t offset, uint32_t* out);

// batched forms (one launch each for all distributions of the batch)
cudaError_t launch_batch_maps(cudaStream_t st, const DistDesc* dist, uint32_t count,
                              uint32_t* tile_map, uint32_t* split_map, uint32_t* sample_map,
                              uint32_t split_size);
cudaError_t launch_batch_build(cudaStream_t st, uint32_t precision, bool r64,
                               const BatchView& b);
cudaError_t launch_batch_alias_sample(cudaStream_t st, uint32_t rng, uint32_t coop,
                                      const BatchView& b);

// Records `msg` as the calling thread's wrs_last_error() and returns `status`
// (defined in wrs_capi.cu).
int set_last_error(int status, const char* msg);

// Device address of a batch's status word (defined in wrs_capi.cu).
uint32_t* batch_status_word(::wrs_batch* b);

__host__ __device__ inline uint32_t tiles_for(uint32_t n) {
    return static_cast<uint32_t>((static_cast<uint64_t>(n) + kTileItems - 1) / kTileItems);
}
// number of split subproblems of a distribution of n weights
__host__ __device__ inline uint32_t splits_for(uint32_t n, uint32_t split_size) {
    const uint32_t k = n / split_size;
    return k ? k : 1u;
}
__host__ __device__ inline uint32_t split_blocks_for(uint32_t n, uint32_t split_size) {
    return (splits_for(n, split_size) + kSplitPack - 1) / kSplitPack;
}
__host__ __device__ inline uint32_t records_for(uint32_t n, uint32_t split_size) {
    const uint32_t k = static_cast<uint32_t>((static_cast<uint64_t>(n) + split_size - 1) / split_size);
    return k ? k : 1u;
}
__host__ __device__ inline uint64_t alias_blocks_for(uint64_t s) { return (s + kAliasPerBlock - 1) / kAliasPerBlock; }
// guiding-table entries of the Cutpoint method (cutpoint/Cutpoint.hpp:72-73)
__host__ __device__ inline uint32_t guide_entries(uint32_t n, uint32_t entry_size) {
    return static_cast<uint32_t>((static_cast<uint64_t>(n) + entry_size - 1) / entry_size);
}

}  // namespace wrs

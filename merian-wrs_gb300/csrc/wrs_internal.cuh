// wrs_internal.cuh -- device data layout and kernel launchers shared by the .cu files.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "wrs_device.cuh"

namespace wrs {

// Tile geometry of the decoupled-lookback kernels: 256 threads x 16 items.
constexpr int kTileThreads = 256;
constexpr int kTileWarps = kTileThreads / 32;
constexpr int kTileItems = 4096;
constexpr int kWarpItems = kTileItems / kTileWarps;  // 512 contiguous items per warp

// Total-mass reduction grid cap (152 SMs x 8); also the size of the partials array.
constexpr int kMassThreads = 256;
constexpr int kMassMaxBlocks = 152 * 8;

// Split+pack: one thread per split; kSplitThreads - kSplitLook - 1 subproblems packed per CTA,
// the remaining threads compute look-ahead splits (see k_split_pack).
constexpr int kSplitThreads = 512;
constexpr int kSplitLook = 32;

// Ticket / completion / epoch of one lookback kernel kind.  The epoch selects which half
// of that kernel's double-buffered state array is live in the current launch.
struct LbCtrl {
    uint32_t ticket;  // tile tickets handed out in the current launch
    uint32_t done;    // CTAs finished in the current launch
    uint32_t epoch;
    uint32_t pad;
};

// Per-build control block (device memory, zero-initialised once at allocation).
// Every counter below is returned to zero by the last CTA of the kernel that used it,
// so successive builds (and CUDA-graph replays) need no memset.
struct alignas(64) BuildCtrl {
    uint32_t mass_done;  // CTAs finished in the total-mass reduction
    uint32_t status;     // kStatus* bits raised by the device
    uint32_t heavy_count;
    float mean;          // (float)(total / N)
    double total;        // FP64 total mass
    LbCtrl part;         // prefix-partition launches
    LbCtrl scan;         // scan launches
    double mean64;       // total / N in FP64
    float mean_lo;       // (float)(mean64 - mean): mean64 as the float-float pair (mean, mean_lo)
    uint32_t pad[15];
};
static_assert(sizeof(BuildCtrl) == 128, "BuildCtrl layout");

// Lookback state of one tile of the prefix-partition (64 B):
//   q0 = {aggregate heavy sum, aggregate light sum}   (ff words)
//   q1 = {aggregate heavy count, inclusive heavy count} (count words)
//   q2 = {inclusive heavy sum, inclusive light sum}   (ff words)
struct alignas(64) PartState {
    unsigned long long agg_h, agg_l, agg_c, pre_c, pre_h, pre_l, pad0, pad1;
};
// Lookback state of one tile of the scan (16 B): {aggregate, inclusive prefix}.
struct alignas(16) ScanState {
    unsigned long long agg, pre;
};

// ---- launchers (defined in wrs_build.cu / wrs_sample.cu) -------------------------
cudaError_t launch_total_mass(cudaStream_t st, const float* w, uint32_t n, double* partials,
                              BuildCtrl* ctrl);
cudaError_t launch_prefix_partition(cudaStream_t st, bool comp, const float* w, uint32_t n,
                                    BuildCtrl* ctrl, PartState* states, uint32_t cap_tiles,
                                    uint32_t* idx_out, float* prefix_out, float* elems_out,
                                    float* prefix_lo_out);
cudaError_t launch_scan(cudaStream_t st, bool comp, const float* in, uint32_t n, float* out,
                        BuildCtrl* ctrl, ScanState* states, uint32_t cap_tiles,
                        uint32_t spin_limit = kSpinLimit);
cudaError_t launch_split_pack(cudaStream_t st, bool r64, bool full_light, const float* w,
                              const uint32_t* idx, const float* elems, const float* prefix,
                              const float* prefix_lo, const BuildCtrl* ctrl, uint32_t* status,
                              uint32_t n, uint32_t split_size, uint2* table);
cudaError_t launch_alias_sample(cudaStream_t st, uint32_t rng, uint32_t coop, const uint2* table,
                                uint32_t n, uint64_t s, uint64_t seed, uint64_t offset,
                                uint32_t* out);
cudaError_t launch_its_sample(cudaStream_t st, uint32_t rng, uint32_t coop, bool parray,
                              const float* cmf, uint32_t n, uint64_t s, uint64_t seed,
                              uint64_t offset, uint32_t* out);

// Records `msg` as the calling thread's wrs_last_error() and returns `status`
// (defined in wrs_capi.cu).
int set_last_error(int status, const char* msg);

inline uint32_t tiles_for(uint32_t n) {
    return static_cast<uint32_t>((static_cast<uint64_t>(n) + kTileItems - 1) / kTileItems);
}

}  // namespace wrs

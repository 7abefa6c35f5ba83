// wrs_probe.cu -- device calibration: the rate of random 8-byte gathers from a buffer.
//
// Alias sampling from a table larger than L2 is bound by random-access throughput, not by
// the bytes it needs: every gather of an 8-byte entry costs a DRAM burst of ~100+ bytes on
// GB300, whatever the access width up to 32 bytes.  wrs_probe_random_gather measures that
// rate on the device at hand (one 8-byte load per thread from a hashed index, the same access
// shape as k_alias_sample), so a benchmark can state alias sampling against the achievable
// random-gather rate next to the bandwidth roofline.
#include "../../include/wrs.h"
#include "wrs_internal.cuh"

namespace {

__device__ __forceinline__ uint32_t probe_hash(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__global__ __launch_bounds__(256) void k_probe_gather(const uint2* __restrict__ buf,
                                                      uint64_t entries, uint64_t accesses,
                                                      uint32_t* __restrict__ sink) {
    const uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (t >= accesses) return;
    const uint64_t h = (static_cast<uint64_t>(probe_hash(static_cast<uint32_t>(t))) << 32) |
                       probe_hash(static_cast<uint32_t>(t) ^ 0x9e3779b9u);
    const uint2 v = wrs::ld_entry(buf + h % entries);
    if ((v.x ^ v.y) == 0x9e3779b9u) sink[0] = v.x;  // keeps the load; never true for zeroed data
}

}  // namespace

extern "C" wrs_status wrs_probe_random_gather(void* stream, const void* buffer, uint64_t bytes,
                                              uint64_t accesses, uint32_t* sink) {
    if (!buffer || !sink || bytes < 8 || accesses == 0)
        return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_INVALID_ARG, "bad argument"));
    const uint64_t blocks = (accesses + 255) / 256;
    if (blocks > 0x7fffffffull)
        return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_INVALID_ARG, "too many accesses"));
    k_probe_gather<<<static_cast<unsigned>(blocks), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        static_cast<const uint2*>(buffer), bytes / 8, accesses, sink);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_CUDA, cudaGetErrorString(e)));
    return WRS_OK;
}

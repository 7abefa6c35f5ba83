// wrs_probe.cu -- device calibration: the rate of random 8-byte gathers from a buffer.
//
// Alias sampling from a table larger than L2 is bound by random-access throughput, not by
// the bytes it needs: every gather of an 8-byte entry costs a DRAM burst of ~100+ bytes on
// GB300, whatever the access width up to 32 bytes.  wrs_probe_random_gather measures that
// rate on the device at hand (one 8-byte load per thread from a hashed index, the same access
// shape as k_alias_sample), so a benchmark can state alias sampling against the achievable
// random-gather rate next to the bandwidth roofline.  `width` sets the bytes per load (4 to
// 128) for a sweep of the access granularity.
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

template <int W>
__global__ __launch_bounds__(256) void k_probe_gather(const unsigned char* __restrict__ buf,
                                                      uint64_t units, uint64_t accesses,
                                                      uint32_t* __restrict__ sink) {
    const uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (t >= accesses) return;
    const uint64_t h = (static_cast<uint64_t>(probe_hash(static_cast<uint32_t>(t))) << 32) |
                       probe_hash(static_cast<uint32_t>(t) ^ 0x9e3779b9u);
    const unsigned char* p = buf + (h % units) * W;  // a W-aligned W-byte unit inside the buffer
    uint32_t acc;
    if constexpr (W == 4) {
        acc = __ldg(reinterpret_cast<const uint32_t*>(p));
    } else if constexpr (W == 8) {
        const uint2 v = wrs::ld_entry(reinterpret_cast<const uint2*>(p));
        acc = v.x ^ v.y;
    } else {
        acc = 0;
#pragma unroll
        for (int k = 0; k < W / 16; ++k) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(p) + k);
            acc ^= v.x ^ v.y ^ v.z ^ v.w;
        }
    }
    if (acc == 0x9e3779b9u) sink[0] = acc;  // keeps the loads; never true for zeroed data
}

template <int W>
cudaError_t probe_launch(cudaStream_t st, const void* buffer, uint64_t bytes, uint64_t accesses,
                         uint32_t* sink) {
    const uint64_t blocks = (accesses + 255) / 256;
    k_probe_gather<W><<<static_cast<unsigned>(blocks), 256, 0, st>>>(
        static_cast<const unsigned char*>(buffer), bytes / W, accesses, sink);
    return cudaGetLastError();
}

}  // namespace

extern "C" wrs_status wrs_probe_random_gather(void* stream, const void* buffer, uint64_t bytes,
                                              uint64_t accesses, uint32_t width,
                                              uint32_t* sink) {
    if (!buffer || !sink || accesses == 0 || bytes < width)
        return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_INVALID_ARG, "bad argument"));
    if ((accesses + 255) / 256 > 0x7fffffffull)
        return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_INVALID_ARG, "too many accesses"));
    if (reinterpret_cast<uintptr_t>(buffer) % (width < 16 ? width : 16) != 0)
        return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_INVALID_ARG, "buffer misaligned"));
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e;
    switch (width) {
        case 4: e = probe_launch<4>(st, buffer, bytes, accesses, sink); break;
        case 8: e = probe_launch<8>(st, buffer, bytes, accesses, sink); break;
        case 16: e = probe_launch<16>(st, buffer, bytes, accesses, sink); break;
        case 32: e = probe_launch<32>(st, buffer, bytes, accesses, sink); break;
        case 64: e = probe_launch<64>(st, buffer, bytes, accesses, sink); break;
        case 128: e = probe_launch<128>(st, buffer, bytes, accesses, sink); break;
        default:
            return static_cast<wrs_status>(
                wrs::set_last_error(WRS_ERR_INVALID_ARG, "width must be 4, 8, 16, 32, 64 or 128"));
    }
    if (e != cudaSuccess)
        return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_CUDA, cudaGetErrorString(e)));
    return WRS_OK;
}

// wrs_prng.cu -- the standalone PRNG operator: a buffer of uniform floats from the shaders'
// Philox2x32-7 stream.
//
// PRNG::run / Philox::run (src/device/prng/PRNG.hpp:15-56, src/device/prng/philox/Philox.hpp:
// 94-108) dispatch src/device/prng/philox/shader.comp:47-55, which writes, for invocation gid,
// u = float(x1) / 2^32 with (x0, x1) = Philox2x32-7(counter (gid, 0), key = seed).  The
// reference bench uses it to fill weight buffers (src/bench/sample_throughput.cpp:151-182).
// Note the counter order: (gid, 0) here, (0, gid) in the alias sampler.
//
// One thread per 4 consecutive elements, written as one 16-byte streaming store when the
// output is 16-byte aligned; the reference's dispatch rounds up to whole workgroups and writes
// past S, this kernel writes elements [0, n) only.  Bound: the 4-byte store per element
// (HBM) and the 7 multiply rounds per element (ALU), about level on GB300.
#include "../../include/wrs.h"
#include "wrs_device.cuh"
#include "wrs_internal.cuh"

namespace wrs {

constexpr int kPrngThreads = 256;
constexpr int kPrngPerThread = 4;

__global__ __launch_bounds__(kPrngThreads) void k_philox_uniform(float* __restrict__ out,
                                                                 uint32_t n, uint32_t seed) {
    const uint64_t e0 =
        (static_cast<uint64_t>(blockIdx.x) * kPrngThreads + threadIdx.x) * kPrngPerThread;
    if (e0 >= n) return;
    float u[kPrngPerThread];
#pragma unroll
    for (int c = 0; c < kPrngPerThread; ++c)
        u[c] = unit_ref(philox2x32_7(static_cast<uint32_t>(e0 + c), 0u, seed).y);
    if (e0 + kPrngPerThread <= n && (reinterpret_cast<uintptr_t>(out) & 15u) == 0) {
        __stcs(reinterpret_cast<float4*>(out + e0), make_float4(u[0], u[1], u[2], u[3]));
    } else {
#pragma unroll
        for (int c = 0; c < kPrngPerThread; ++c)
            if (e0 + c < n) out[e0 + c] = u[c];
    }
}

}  // namespace wrs

extern "C" wrs_status wrs_philox(void* stream, uint32_t seed, uint32_t n, float* out) {
    if (n == 0) return WRS_OK;
    if (!out) return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_INVALID_ARG, "out is NULL"));
    const uint64_t threads = (static_cast<uint64_t>(n) + wrs::kPrngPerThread - 1) / wrs::kPrngPerThread;
    const uint32_t blocks =
        static_cast<uint32_t>((threads + wrs::kPrngThreads - 1) / wrs::kPrngThreads);
    wrs::k_philox_uniform<<<blocks, wrs::kPrngThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        out, n, seed);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return static_cast<wrs_status>(wrs::set_last_error(WRS_ERR_CUDA, cudaGetErrorString(e)));
    return WRS_OK;
}

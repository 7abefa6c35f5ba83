// percall_driver.cpp -- the per-call arm of the batched comparison, driven from C++.
//
// The reference builds and samples one distribution per call (WRS::build / WRS::sample,
// src/device/wrs/WRS.hpp:121-168; its benchmark loops over them, src/bench/wrs.cpp).  To time
// that usage pattern without an interpreter in the loop, wrs_percall_run drives `count`
// distributions through the C++ facade of include/wrs.hpp -- one wrs::WRS and one
// wrs::WRSBuffers sized for the largest distribution, reused -- with a build and a sample call
// per distribution, `passes` times over, and times the whole loop with CUDA events on
// `stream`.  Built next to libwrs_gb300.so as libwrs_percall.so (host code only).
#include <cuda_runtime.h>

#include <cstdint>
#include <exception>

#include "wrs.hpp"

extern "C" int wrs_percall_run(const wrs_config* cfg, void* stream, uint32_t count,
                               const float* const* weights, const uint32_t* n,
                               const uint64_t* s, const uint64_t* seeds,
                               uint32_t* const* samples, uint32_t passes, float* ms) {
    if (!cfg || !weights || !n || !s || !seeds || !samples || !ms) return WRS_ERR_INVALID_ARG;
    try {
        uint32_t max_n = 1;
        for (uint32_t d = 0; d < count; ++d) max_n = n[d] > max_n ? n[d] : max_n;
        const wrs::WRS method(*cfg);
        wrs::WRSBuffers buffers = wrs::WRSBuffers::allocate(method, max_n, nullptr, nullptr);
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        cudaEvent_t e0, e1;
        if (cudaEventCreate(&e0) != cudaSuccess) return WRS_ERR_CUDA;
        if (cudaEventCreate(&e1) != cudaSuccess) {
            cudaEventDestroy(e0);
            return WRS_ERR_CUDA;
        }
        cudaEventRecord(e0, st);
        for (uint32_t p = 0; p < passes; ++p) {
            for (uint32_t d = 0; d < count; ++d) {
                buffers.weights = weights[d];
                buffers.samples = samples[d];
                method.build(stream, buffers, n[d]);
                method.sample(stream, buffers, n[d], s[d], seeds[d]);
            }
        }
        cudaEventRecord(e1, st);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (e != cudaSuccess) return WRS_ERR_CUDA;
        uint32_t dev_status = 0;
        const wrs_status rs = wrs_buffers_status(buffers.internals(), stream, &dev_status);
        return rs;
    } catch (const wrs::Error& err) {
        return err.status;
    } catch (const std::exception&) {
        return WRS_ERR_INVALID_ARG;
    }
}

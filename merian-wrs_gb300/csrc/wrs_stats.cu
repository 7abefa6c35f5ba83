// wrs_stats.cu -- on-device sample statistics: histogram, chi-square, RMSE.
//
//   k_histogram      hist[s] += 1 per sample (64-bit atomics)
//                    (reference: src/device/statistics/histogram/atomic/shader.comp:27-38)
//   k_sample_stats   chi-square = sum over e_i > 0 of (o_i - e_i)^2 / e_i with
//                    e_i = w_i * S / total, and the squared error sum of (w_i / total - o_i / S)
//                    (src/device/statistics/chi_square/reduce/shader.comp:40-73,
//                     src/device/statistics/rmse/mse/shader.comp:41-73); also the number of
//                    draws that landed on zero-weight items (which the chi-square skips)
//
// The reference reduces with FP32 atomics (order-dependent).  Here each term is formed in FP32
// and accumulated in float-float per thread and across the CTA, the tile partials are stored
// in FP64 and the last CTA sums them in a fixed order: the statistics are deterministic.  The
// total weight comes from k_total_mass on the same scratch, so no host value is needed.
#include "../../include/wrs.h"
#include "wrs_device.cuh"
#include "wrs_internal.cuh"

using namespace wrs;

namespace {

struct StatsScratch {
    BuildCtrl* ctrl;     // total mass (k_total_mass) and the stats completion counter
    double* mass;        // per-tile mass partials
    double* part;        // per-tile {chi2, sqerr, zero hits}
};

size_t stats_bytes(uint32_t n) {
    const size_t tiles = tiles_for(n) + 1;
    return sizeof(BuildCtrl) + tiles * sizeof(double) + 3 * tiles * sizeof(double);
}

StatsScratch stats_layout(void* scratch, uint32_t n) {
    const size_t tiles = tiles_for(n) + 1;
    char* p = static_cast<char*>(scratch);
    StatsScratch s;
    s.ctrl = reinterpret_cast<BuildCtrl*>(p);
    s.mass = reinterpret_cast<double*>(p + sizeof(BuildCtrl));
    s.part = s.mass + tiles;
    return s;
}

__global__ __launch_bounds__(256) void k_histogram(const uint32_t* __restrict__ samples, uint64_t S,
                                                   uint32_t n, unsigned long long* __restrict__ hist,
                                                   uint32_t* __restrict__ status) {
    const uint64_t nth = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < S; i += nth) {
        const uint32_t s = __ldcs(samples + i);
        if (s < n)
            atomicAdd(hist + s, 1ull);
        else
            atomicOr(status, 4u);  // an index out of range: counted nowhere, reported
    }
}

// One CTA per 4096-item tile (16 items per thread), fixed-order reductions.
__global__ __launch_bounds__(kTileThreads) void k_sample_stats(
    const unsigned long long* __restrict__ hist, const float* __restrict__ w, uint32_t n,
    uint64_t S, StatsScratch sc, double* __restrict__ out) {
    __shared__ ff s_a[kTileWarps], s_b[kTileWarps];
    __shared__ unsigned long long s_z[kTileWarps];
    __shared__ bool s_last;
    const uint32_t tile = blockIdx.x;
    const double total = sc.ctrl->total;
    const float e_scale = __double2float_rn(static_cast<double>(S) / total);  // e_i = w_i * S / total
    const float p_scale = __double2float_rn(1.0 / total);                     // w_i / total
    const float inv_s = __double2float_rn(1.0 / static_cast<double>(S));
    ff chi{0.f, 0.f}, sq{0.f, 0.f};
    unsigned long long zero_hits = 0;
    const uint32_t base = tile * kTileItems + threadIdx.x;
#pragma unroll 4
    for (int r = 0; r < kTileItems / kTileThreads; ++r) {
        const uint32_t i = base + r * kTileThreads;
        if (i < n) {
            const float wi = __ldg(w + i);
            const float o = static_cast<float>(__ldcs(hist + i));
            const float e = __fmul_rn(wi, e_scale);
            if (e > 0.0f) {
                const float d = __fsub_rn(o, e);
                chi = ff_add_f(chi, __fdiv_rn(__fmul_rn(d, d), e));
            } else if (o > 0.0f) {
                zero_hits += __ldcs(hist + i);
            }
            const float diff = __fsub_rn(__fmul_rn(wi, p_scale), __fmul_rn(o, inv_s));
            sq = ff_add_f(sq, __fmul_rn(diff, diff));
        }
    }
    chi = ff_warp_total(chi);
    sq = ff_warp_total(sq);
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) zero_hits += __shfl_xor_sync(0xffffffffu, zero_hits, m);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_a[warp] = chi;
        s_b[warp] = sq;
        s_z[warp] = zero_hits;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        ff a = s_a[0], b = s_b[0];
        unsigned long long z = s_z[0];
        for (int k = 1; k < kTileWarps; ++k) {
            a = carry_add<true>(a, s_a[k]);
            b = carry_add<true>(b, s_b[k]);
            z += s_z[k];
        }
        double* p = sc.part + 3 * static_cast<size_t>(tile);
        p[0] = __dadd_rn(static_cast<double>(a.hi), static_cast<double>(a.lo));
        p[1] = __dadd_rn(static_cast<double>(b.hi), static_cast<double>(b.lo));
        p[2] = static_cast<double>(z);
        __threadfence();
        s_last = atomicAdd(&sc.ctrl->heavy_count, 1u) == gridDim.x - 1u;  // completion counter
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // last CTA: each thread sums a fixed stride of tiles, then a fixed tree
    __shared__ double s_r[3][kTileWarps];
    double c2 = 0.0, se = 0.0, zh = 0.0;
    for (uint32_t t = threadIdx.x; t < gridDim.x; t += blockDim.x) {
        const double* p = sc.part + 3 * static_cast<size_t>(t);
        c2 = __dadd_rn(c2, __ldcg(p));
        se = __dadd_rn(se, __ldcg(p + 1));
        zh = __dadd_rn(zh, __ldcg(p + 2));
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        c2 = __dadd_rn(c2, __shfl_xor_sync(0xffffffffu, c2, m));
        se = __dadd_rn(se, __shfl_xor_sync(0xffffffffu, se, m));
        zh = __dadd_rn(zh, __shfl_xor_sync(0xffffffffu, zh, m));
    }
    if (lane == 0) {
        s_r[0][warp] = c2;
        s_r[1][warp] = se;
        s_r[2][warp] = zh;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        c2 = se = zh = 0.0;
        for (int k = 0; k < kTileWarps; ++k) {
            c2 = __dadd_rn(c2, s_r[0][k]);
            se = __dadd_rn(se, s_r[1][k]);
            zh = __dadd_rn(zh, s_r[2][k]);
        }
        out[0] = c2;
        out[1] = sqrt(se / static_cast<double>(n));
        out[2] = zh;
        out[3] = total;
        sc.ctrl->heavy_count = 0u;
    }
}

wrs_status sfail(wrs_status s, const char* m) {
    set_last_error(s, m);
    return s;
}

}  // namespace

extern "C" {

wrs_status wrs_histogram(void* stream, const uint32_t* samples, uint64_t s, uint32_t n,
                         uint64_t* hist, uint32_t* device_status) {
    if ((!samples && s) || !hist || !device_status) return sfail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return sfail(WRS_ERR_INVALID_ARG, "n must be >= 1");
    if (s == 0) return WRS_OK;
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint64_t blocks = (s + 255) / 256;
    if (blocks > 152ull * 32) blocks = 152ull * 32;
    k_histogram<<<static_cast<unsigned>(blocks), 256, 0, st>>>(
        samples, s, n, reinterpret_cast<unsigned long long*>(hist), device_status);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return sfail(WRS_ERR_CUDA, cudaGetErrorString(e));
    return WRS_OK;
}

size_t wrs_statistics_scratch_bytes(uint32_t n) { return stats_bytes(n); }

wrs_status wrs_sample_statistics(void* stream, const uint64_t* hist, const float* weights,
                                 uint32_t n, uint64_t s, void* scratch, double* out) {
    if (!hist || !weights || !scratch || !out) return sfail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0 || s == 0) return sfail(WRS_ERR_INVALID_ARG, "n and s must be >= 1");
    if (reinterpret_cast<uintptr_t>(scratch) % 128 != 0)
        return sfail(WRS_ERR_INVALID_ARG, "scratch must be 128-byte aligned");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const StatsScratch sc = stats_layout(scratch, n);
    cudaError_t e = launch_total_mass(st, weights, n, sc.mass, sc.ctrl);
    if (e == cudaSuccess) {
        k_sample_stats<<<tiles_for(n), kTileThreads, 0, st>>>(
            reinterpret_cast<const unsigned long long*>(hist), weights, n, s, sc, out);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return sfail(WRS_ERR_CUDA, cudaGetErrorString(e));
    return WRS_OK;
}

}  // extern "C"

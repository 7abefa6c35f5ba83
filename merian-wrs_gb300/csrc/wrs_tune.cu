// wrs_tune.cu -- launch-configuration autotuner for the alias method.
//
// Two knobs decide the speed of a build + sample on a given workload:
//   * the PSA split size (PSAConfig's InlineSplitPackConfig::splitSize,
//     src/device/wrs/alias/psa/PSA.hpp:19-41): the number of pack items per split, which
//     trades the split bisections (N / splitSize of them, latency-bound) against the serial
//     pack walk of each subproblem.  It is part of the table's definition: the split points
//     move with it, so the table bits are a function of (weights, split size).
//   * the context's L2 fetch granularity (cudaLimitMaxL2FetchGranularity): how many bytes
//     the L2 fetches from HBM per miss.  Alias sampling from a table larger than L2 is one
//     random 8-byte gather per sample, so the over-fetch of each miss bounds it.  A
//     context-wide hint that lasts as long as the CUDA context; it changes no result.
// The tuner measures candidates with CUDA events on the caller's stream (a coordinate
// search: the L2 granularity at the configured split size, then the split sizes at the
// chosen granularity), objective = build + sample time per call, and leaves the context's
// L2 limit at the chosen value.  No counterpart in the reference, whose configurations are
// fixed at construction.
#include <cuda_runtime.h>

#include <cstdio>
#include <iterator>
#include <vector>

#include "../../include/wrs.h"
#include "wrs_internal.cuh"

namespace {

const uint32_t kDefaultSplits[] = {4, 6, 8, 12, 16, 24, 32};
const uint32_t kDefaultL2[] = {32, 64, 128};

wrs_status tfail(wrs_status s, const char* m) {
    wrs::set_last_error(s, m);
    return s;
}

wrs_status tcuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return WRS_OK;
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return tfail(WRS_ERR_CUDA, buf);
}

struct Events {
    cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
    ~Events() {
        for (cudaEvent_t x : e)
            if (x) cudaEventDestroy(x);
    }
    cudaError_t create() {
        for (cudaEvent_t& x : e) {
            const cudaError_t r = cudaEventCreate(&x);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    }
};

// The search space with the defaults filled in.
struct Space {
    std::vector<uint32_t> splits, l2;
    uint32_t warmup, reps;
};

wrs_status make_space(const wrs_tune_space* sp, uint32_t base_split, Space& out) {
    out.splits.clear();
    out.l2.clear();
    if (sp && sp->split_sizes) {
        out.splits.assign(sp->split_sizes, sp->split_sizes + sp->split_count);
    } else if (!sp || sp->split_count != 0) {
        out.splits.assign(std::begin(kDefaultSplits), std::end(kDefaultSplits));
    }
    if (sp && sp->l2_fetch) {
        out.l2.assign(sp->l2_fetch, sp->l2_fetch + sp->l2_count);
    } else if (!sp || sp->l2_count != 0) {
        out.l2.assign(std::begin(kDefaultL2), std::end(kDefaultL2));
    }
    for (uint32_t s : out.splits)
        if (s < 1u) return tfail(WRS_ERR_INVALID_ARG, "split sizes must be >= 1");
    for (uint32_t b : out.l2)
        if (b > 128u) return tfail(WRS_ERR_INVALID_ARG, "L2 fetch granularity must be <= 128 bytes");
    if (out.splits.empty()) out.splits.push_back(base_split);
    out.warmup = sp && sp->warmup ? sp->warmup : 1u;
    out.reps = sp && sp->reps ? sp->reps : 3u;
    return WRS_OK;
}

// One candidate's timing: `build` and `sample` enqueue one call each on `st`; the mean
// milliseconds per repetition land in *bms and *sms.
template <class B, class S>
wrs_status time_pair(cudaStream_t st, const Space& sp, B&& build, S&& sample, float* bms,
                     float* sms) {
    Events ev;
    wrs_status s = tcuda(ev.create(), "event create");
    if (s != WRS_OK) return s;
    for (uint32_t r = 0; r < sp.warmup; ++r) {
        if ((s = build()) != WRS_OK || (s = sample()) != WRS_OK) return s;
    }
    float tb = 0.f, ts = 0.f;
    for (uint32_t r = 0; r < sp.reps; ++r) {
        if ((s = tcuda(cudaEventRecord(ev.e[0], st), "event record")) != WRS_OK) return s;
        if ((s = build()) != WRS_OK) return s;
        if ((s = tcuda(cudaEventRecord(ev.e[1], st), "event record")) != WRS_OK) return s;
        if ((s = sample()) != WRS_OK) return s;
        if ((s = tcuda(cudaEventRecord(ev.e[2], st), "event record")) != WRS_OK) return s;
        if ((s = tcuda(cudaEventSynchronize(ev.e[2]), "event synchronize")) != WRS_OK) return s;
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, ev.e[0], ev.e[1]);
        cudaEventElapsedTime(&b, ev.e[1], ev.e[2]);
        tb += a;
        ts += b;
    }
    *bms = tb / static_cast<float>(sp.reps);
    *sms = ts / static_cast<float>(sp.reps);
    return WRS_OK;
}

// The coordinate search shared by the per-call and batch tuners.  trial(cfg, &b, &s)
// measures one configuration.
template <class Trial>
wrs_status search(const wrs_config& base, const Space& sp, Trial&& trial, wrs_tune_result* out,
                  wrs_tune_trial* trials, uint32_t max_trials) {
    uint32_t done = 0;
    auto record = [&](uint32_t split, uint32_t l2, float b, float s) {
        if (trials && done < max_trials) trials[done] = wrs_tune_trial{split, l2, b, s};
        ++done;
    };
    wrs_config cfg = base;
    uint32_t best_l2 = 0;
    float best = -1.f, best_b = 0.f, best_s = 0.f;
    // 1) L2 fetch granularity at the configured split size
    for (uint32_t l2 : sp.l2) {
        wrs_status s = wrs_set_l2_fetch_granularity(l2);
        if (s != WRS_OK) return s;
        float b = 0.f, sm = 0.f;
        if ((s = trial(cfg, &b, &sm)) != WRS_OK) return s;
        record(cfg.split_size, l2, b, sm);
        if (best < 0.f || b + sm < best) {
            best = b + sm;
            best_l2 = l2;
            best_b = b;
            best_s = sm;
        }
    }
    if (!sp.l2.empty()) {
        const wrs_status s = wrs_set_l2_fetch_granularity(best_l2);
        if (s != WRS_OK) return s;
    }
    // 2) split sizes at that granularity (the configured size is not measured twice)
    uint32_t best_split = base.split_size;
    for (uint32_t split : sp.splits) {
        if (!sp.l2.empty() && split == base.split_size) continue;
        cfg.split_size = split;
        float b = 0.f, sm = 0.f;
        const wrs_status s = trial(cfg, &b, &sm);
        if (s != WRS_OK) return s;
        record(split, sp.l2.empty() ? 0u : best_l2, b, sm);
        if (best < 0.f || b + sm < best) {
            best = b + sm;
            best_split = split;
            best_b = b;
            best_s = sm;
        }
    }
    out->split_size = best_split;
    out->l2_fetch = sp.l2.empty() ? 0u : best_l2;
    out->build_ms = best_b;
    out->sample_ms = best_s;
    out->trials = done;
    return WRS_OK;
}

wrs_status check_base(const wrs_config* base) {
    if (!base) return tfail(WRS_ERR_INVALID_ARG, "config is NULL");
    if (base->method != WRS_METHOD_ALIAS_TABLE)
        return tfail(WRS_ERR_NOT_IMPLEMENTED, "the tuner covers the alias method");
    return WRS_OK;
}

}  // namespace

extern "C" {

wrs_status wrs_set_l2_fetch_granularity(uint32_t bytes) {
    if (bytes > 128u) return tfail(WRS_ERR_INVALID_ARG, "L2 fetch granularity must be <= 128 bytes");
    return tcuda(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, bytes),
                 "cudaDeviceSetLimit(MaxL2FetchGranularity)");
}

wrs_status wrs_get_l2_fetch_granularity(uint32_t* bytes) {
    if (!bytes) return tfail(WRS_ERR_INVALID_ARG, "NULL argument");
    size_t v = 0;
    const wrs_status s = tcuda(cudaDeviceGetLimit(&v, cudaLimitMaxL2FetchGranularity),
                               "cudaDeviceGetLimit(MaxL2FetchGranularity)");
    if (s == WRS_OK) *bytes = static_cast<uint32_t>(v);
    return s;
}

wrs_status wrs_autotune_alias(const wrs_config* base, void* stream, const float* weights,
                              uint32_t n, uint64_t s, uint32_t* samples,
                              const wrs_tune_space* space, wrs_tune_result* out,
                              wrs_tune_trial* trials, uint32_t max_trials) {
    wrs_status st = check_base(base);
    if (st != WRS_OK) return st;
    if (!weights || !out || (s && !samples)) return tfail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return tfail(WRS_ERR_INVALID_ARG, "n must be >= 1");
    Space sp;
    if ((st = make_space(space, base->split_size, sp)) != WRS_OK) return st;
    const cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    auto trial = [&](const wrs_config& cfg, float* bms, float* sms) -> wrs_status {
        wrs_handle* h = nullptr;
        wrs_buffers* b = nullptr;
        wrs_status r = wrs_create(&cfg, &h);
        if (r == WRS_OK) r = wrs_buffers_create(h, n, &b);
        if (r == WRS_OK)
            r = time_pair(
                cs, sp, [&] { return wrs_build(h, stream, weights, n, b); },
                [&] { return s ? wrs_sample(h, stream, b, n, s, 1u, samples) : WRS_OK; }, bms,
                sms);
        uint32_t dev = 0;
        if (r == WRS_OK) r = wrs_buffers_status(b, stream, &dev);
        wrs_buffers_destroy(b);
        wrs_destroy(h);
        return r;
    };
    return search(*base, sp, trial, out, trials, max_trials);
}

wrs_status wrs_autotune_batch(const wrs_config* base, void* stream, const wrs_dist_desc* descs,
                              uint32_t count, const wrs_tune_space* space, wrs_tune_result* out,
                              wrs_tune_trial* trials, uint32_t max_trials) {
    wrs_status st = check_base(base);
    if (st != WRS_OK) return st;
    if (!descs || !out || count == 0) return tfail(WRS_ERR_INVALID_ARG, "no distributions");
    uint64_t weights = 0, samples = 0;
    for (uint32_t d = 0; d < count; ++d) {
        if (descs[d].weights) weights += descs[d].n;
        if (descs[d].samples) samples += descs[d].s;
    }
    Space sp;
    if ((st = make_space(space, base->split_size, sp)) != WRS_OK) return st;
    const cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);
    auto trial = [&](const wrs_config& cfg, float* bms, float* sms) -> wrs_status {
        wrs_handle* h = nullptr;
        wrs_batch* b = nullptr;
        wrs_status r = wrs_create(&cfg, &h);
        if (r == WRS_OK) r = wrs_batch_create(h, count, weights, samples, &b);
        if (r == WRS_OK) r = wrs_batch_set(b, stream, descs, count);
        if (r == WRS_OK)
            r = time_pair(
                cs, sp, [&] { return wrs_batch_build(h, stream, b); },
                [&] { return wrs_batch_sample(h, stream, b); }, bms, sms);
        uint32_t dev = 0;
        if (r == WRS_OK) r = wrs_batch_status(b, stream, &dev);
        wrs_batch_destroy(b);
        wrs_destroy(h);
        return r;
    };
    return search(*base, sp, trial, out, trials, max_trials);
}

}  // extern "C"

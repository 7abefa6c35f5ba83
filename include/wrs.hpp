// wrs.hpp -- header-only C++ mirror of merian-wrs's device::WRS operator facade
// (src/device/wrs/WRS.hpp:14-172) on top of the C ABI in wrs.h.
//
//   reference                                         here
//   WRSConfig = variant<ITS::Config, AliasTable::Config,        wrs::WRSConfig (+ AliasTableConfig(),
//                       Cutpoint::Config>                       ITSConfig(), CutpointConfig() factories)
//   WRSBuffers::allocate(alloc, mapping, N, S, config)          wrs::WRSBuffers::allocate(wrs, N, weights, samples)
//   WRS(context, shaderCompiler, config)                        wrs::WRS(config)
//   WRS::build(cmd, buffers, N, profiler)                       wrs::WRS::build(stream, buffers, N)
//   WRS::sample(cmd, buffers, N, S, seed = 12345)               wrs::WRS::sample(stream, buffers, N, S, seed = 12345)
//
// The reference records into a caller-owned command buffer; here every call is enqueued
// on a caller-owned CUDA stream (passed as void*).  Weights and samples are caller-owned
// device buffers, as in the reference.  Failures throw wrs::Error carrying the status
// code, where the reference throws std::runtime_error.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>

#include "wrs.h"

namespace wrs {

class Error : public std::runtime_error {
  public:
    Error(wrs_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    wrs_status status;
};

inline void check(wrs_status s) {
    if (s != WRS_OK)
        throw Error(s, std::string(wrs_status_string(s)) + ": " + wrs_last_error());
}

using WRSConfig = wrs_config;

inline WRSConfig AliasTableConfig(uint32_t split_size = 2, uint32_t coop_size = 0,
                                  bool use_partition_elements = true,
                                  uint32_t split_pack_mode = WRS_SPLITPACK_INLINE) {
    WRSConfig c;
    check(wrs_config_init(&c, WRS_METHOD_ALIAS_TABLE));
    c.split_size = split_size;
    c.coop_size = coop_size;
    c.use_partition_elements = use_partition_elements ? 1u : 0u;
    c.split_pack_mode = split_pack_mode;
    return c;
}

inline WRSConfig ITSConfig(uint32_t coop_size = 0, bool parray = false) {
    WRSConfig c;
    check(wrs_config_init(&c, WRS_METHOD_ITS));
    c.coop_size = coop_size;
    c.its_parray = parray ? 1u : 0u;
    return c;
}

inline WRSConfig CutpointConfig(uint32_t guiding_entry_size = 32) {
    WRSConfig c;
    check(wrs_config_init(&c, WRS_METHOD_CUTPOINT));
    c.guiding_entry_size = guiding_entry_size;
    return c;
}

class WRS;

// Caller-owned weights [N] and samples [S] plus the method's internals.
class WRSBuffers {
  public:
    const float* weights = nullptr;
    uint32_t* samples = nullptr;

    static WRSBuffers allocate(const WRS& wrs, uint32_t N, const float* weights,
                               uint32_t* samples);

    WRSBuffers() = default;
    WRSBuffers(const WRSBuffers&) = delete;
    WRSBuffers& operator=(const WRSBuffers&) = delete;
    WRSBuffers(WRSBuffers&& o) noexcept { *this = std::move(o); }
    WRSBuffers& operator=(WRSBuffers&& o) noexcept {
        std::swap(weights, o.weights);
        std::swap(samples, o.samples);
        std::swap(internals_, o.internals_);
        return *this;
    }
    ~WRSBuffers() { wrs_buffers_destroy(internals_); }

    wrs_buffers* internals() const { return internals_; }
    const wrs_alias_entry* aliasTable() const { return wrs_buffers_alias_table(internals_); }
    const float* cmf() const { return wrs_buffers_cmf(internals_); }

  private:
    wrs_buffers* internals_ = nullptr;
};

class WRS {
  public:
    using Config = WRSConfig;
    using Buffers = WRSBuffers;

    explicit WRS(const Config& config) { check(wrs_create(&config, &handle_)); }
    WRS(const WRS&) = delete;
    WRS& operator=(const WRS&) = delete;
    ~WRS() { wrs_destroy(handle_); }

    void build(void* stream, const Buffers& buffers, uint32_t N) const {
        check(wrs_build(handle_, stream, buffers.weights, N, buffers.internals()));
    }

    void sample(void* stream, const Buffers& buffers, uint32_t N, uint64_t S,
                uint64_t seed = 12345u) const {
        check(wrs_sample(handle_, stream, buffers.internals(), N, S, seed, buffers.samples));
    }

    const wrs_handle* handle() const { return handle_; }

  private:
    wrs_handle* handle_ = nullptr;
};

inline WRSBuffers WRSBuffers::allocate(const WRS& wrs, uint32_t N, const float* weights,
                                       uint32_t* samples) {
    WRSBuffers b;
    b.weights = weights;
    b.samples = samples;
    check(wrs_buffers_create(wrs.handle(), N, &b.internals_));
    return b;
}

}  // namespace wrs

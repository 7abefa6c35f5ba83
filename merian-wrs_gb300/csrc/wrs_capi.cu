// wrs_capi.cu -- host side of the C ABI declared in include/wrs.h.
//
// The handle holds the configuration (the reference's WRSConfig variant); a buffers
// object holds the internals of one distribution (the reference's WRSBuffers minus the
// caller-owned weights and samples) in a single device allocation.  Launch sequences:
//   alias build : k_total_mass -> k_prefix_partition -> k_split_pack
//                 (PSA::run, src/device/wrs/alias/psa/PSA.hpp:170-237)
//   ITS build   : k_scan_bulk, or k_total_mass -> k_scan_exact in the compensated precisions
//                 (ITS::build, src/device/wrs/its/ITS.hpp:90-108), then with a cell size
//                 k_its_cells (the cell blocks k_its_sample_cells reads); on the FP32 CMF also
//                 the cell marks (k_cmf_tile_min -> k_tile_suffix_min -> k_cmf_mark) and
//                 k_its_tree (the probe-tree blocks the marked cells and cell size 0 bisect in)
//   Cutpoint    : the same scan -> k_cutpoint_guide, or k_guide_monotone on the compensated CMF
//                 (Cutpoint::build, src/device/wrs/cutpoint/Cutpoint.hpp:108-138)
//   sample      : k_alias_sample | k_its_sample (k_its_sample_cells) | k_cutpoint_sample
//                 (WRS::sample, src/device/wrs/WRS.hpp:145-168)
//   batch       : k_batch_maps (wrs_batch_set), then the same three build kernels and the
//                 alias sampler over all distributions of a batch, one launch each
// Stream order replaces the reference's pipeline barriers.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/wrs.h"
#include "wrs_device.cuh"
#include "wrs_internal.cuh"

using namespace wrs;

struct wrs_handle {
    wrs_config cfg;
};

struct wrs_buffers {
    wrs_config cfg;
    uint32_t max_n = 0;
    uint32_t cap_tiles = 0;
    void* base = nullptr;
    size_t bytes = 0;
    BuildCtrl* ctrl = nullptr;
    double* partials = nullptr;
    PartState* part_states = nullptr;
    ScanState* scan_states = nullptr;
    uint32_t* idx = nullptr;
    float* prefix = nullptr;
    float* elems = nullptr;
    float* prefix_lo = nullptr;
    uint2* table = nullptr;
    SplitRecord* records = nullptr;  // serial split-pack
    float* cmf = nullptr;
    uint32_t* guide = nullptr;
    ItsCell* cells = nullptr;
    TreeBlock* tree = nullptr;   // ITS bisection: the probe tree's stored block levels
    uint32_t tree_n = 0;         // the n the last build stored them for (0: none)
    uint32_t cells_n = 0;        // the n the last build wrote the ITS cell blocks for (0: none)
    uint8_t* coins = nullptr;    // alias: the table's coin filter (n bytes, kCoinMinN < n)
    uint32_t coins_n = 0;        // the n the last build wrote the coin filter for (0: none)
    uint32_t* coarse = nullptr;  // scratch of the guiding-table / cell construction
    uint32_t* tile_scratch = nullptr;  // block-wise baselines: 3 words per tile
    int2* descent = nullptr;           // split-pack: shared bisection tops per CTA
};

namespace {

thread_local std::string g_last_error;

wrs_status fail(wrs_status s, const char* what) {
    g_last_error = what;
    return s;
}

wrs_status cuda_fail(cudaError_t e, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return WRS_ERR_CUDA;
}

#define WRS_CUDA(call, where)                      \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, where); \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct Layout {
    size_t ctrl, partials, part_states, scan_states, idx, prefix, elems, prefix_lo, table, records,
        coins, cmf, guide, cells, tree, coarse, tile_scratch, descent, total;
};

// ITS bisects the whole CMF with the non-cooperative sampler, and its CMF is deep enough for
// stored block levels below the probe tree's shared-memory ones: the build stores them
// (k_its_tree)
bool its_tree_levels(const wrs_config& cfg, uint32_t n) {
    // the compensated CMF's cells serve every sample; an FP32 CMF's cells send the marked ones
    // to the bisection through the blocks
    const bool cells_alone = cfg.guiding_entry_size != 0 && cfg.scan_precision != WRS_SCAN_FP32;
    return cfg.method == WRS_METHOD_ITS && cfg.coop_size == 0 && !cells_alone &&
           its_tree_block_levels(n) > 0;
}

Layout layout_for(const wrs_config& cfg, uint32_t max_n) {
    const uint32_t cap_tiles = tiles_for(max_n) + 1;
    Layout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off = align_up(off + bytes, 256);
        return at;
    };
    L.ctrl = take(sizeof(BuildCtrl));
    L.partials = take(sizeof(double) * static_cast<size_t>(cap_tiles));
    const bool alias = cfg.method == WRS_METHOD_ALIAS_TABLE;
    L.part_states = alias ? take(sizeof(PartState) * 2 * static_cast<size_t>(cap_tiles)) : 0;
    L.scan_states = take(sizeof(ScanState) * 2 * static_cast<size_t>(cap_tiles));
    const size_t zero_end = off;  // everything above starts zeroed
    L.tile_scratch = take(3 * sizeof(uint32_t) * static_cast<size_t>(cap_tiles));
    (void)zero_end;
    if (alias) {
        L.idx = take(sizeof(uint32_t) * static_cast<size_t>(max_n));
        L.prefix = take(sizeof(float) * static_cast<size_t>(max_n));
        L.elems = cfg.use_partition_elements ? take(sizeof(float) * static_cast<size_t>(max_n)) : 0;
        L.prefix_lo = cfg.scan_precision == WRS_SCAN_FLOAT_FLOAT
                          ? take(sizeof(float) * static_cast<size_t>(max_n))
                          : 0;
        L.table = take(sizeof(uint2) * static_cast<size_t>(max_n));
        L.coins = max_n > kCoinMinN ? take(std::min(max_n, kCoinMaxN)) : 0;
        L.descent = take(sizeof(int2) * static_cast<size_t>(descent_entries(max_n)));
        L.records = cfg.split_pack_mode != WRS_SPLITPACK_INLINE
                        ? take(sizeof(SplitRecord) * records_for(max_n, cfg.split_size))
                        : 0;
    } else {
        L.cmf = take(sizeof(float) * static_cast<size_t>(max_n));
        // Cutpoint: its guiding table; ITS: the cell blocks that steer sampling (none with
        // guiding_entry_size 0) and their construction scratch
        const uint32_t G = cfg.guiding_entry_size ? guide_entries(max_n, cfg.guiding_entry_size) : 0;
        const bool its = cfg.method == WRS_METHOD_ITS;
        if (!its)
            L.guide = take(sizeof(uint32_t) * G);
        else if (G)
            L.cells = take(sizeof(ItsCell) * G);
        if (G && (its || cfg.scan_precision != WRS_SCAN_FP32))
            L.coarse = take(sizeof(uint32_t) * (coarse_entries(G) + group_entries(G)));
        // ITS bisecting the whole CMF (FP32, or no cells): the probe tree's deeper levels
        if (its_tree_levels(cfg, max_n))
            L.tree = take(sizeof(TreeBlock) * its_tree_blocks(its_tree_stored_levels(max_n)));
    }
    L.total = off;
    return L;
}

size_t zeroed_bytes(const wrs_config& cfg, uint32_t max_n) {
    const Layout L = layout_for(cfg, max_n);
    const uint32_t cap_tiles = tiles_for(max_n) + 1;
    return L.scan_states + sizeof(ScanState) * 2 * static_cast<size_t>(cap_tiles);
}

wrs_status check_config(const wrs_config* c) {
    if (!c) return fail(WRS_ERR_INVALID_ARG, "config is NULL");
    if (c->method != WRS_METHOD_ALIAS_TABLE && c->method != WRS_METHOD_ITS &&
        c->method != WRS_METHOD_CUTPOINT)
        return fail(WRS_ERR_INVALID_ARG, "unknown method");
    if (c->method == WRS_METHOD_CUTPOINT && c->guiding_entry_size == 0)
        return fail(WRS_ERR_INVALID_ARG, "guiding_entry_size must be >= 1");
    if (c->method == WRS_METHOD_CUTPOINT && c->coop_size != 0)
        return fail(WRS_ERR_INVALID_ARG,
                    "the Cutpoint method has no cooperative-size setting (coop_size must be 0)");
    if (c->method == WRS_METHOD_ALIAS_TABLE && c->split_size == 0)
        return fail(WRS_ERR_INVALID_ARG, "split_size must be >= 1");
    if (c->split_pack_mode > WRS_SPLITPACK_SERIAL_SUBGROUP)
        return fail(WRS_ERR_INVALID_ARG, "unknown split_pack_mode");
    if (c->rng > WRS_RNG_PHILOX4X32_10) return fail(WRS_ERR_INVALID_ARG, "unknown rng");
    if (c->scan_precision > WRS_SCAN_FLOAT_FLOAT)
        return fail(WRS_ERR_INVALID_ARG, "unknown scan precision");
    if (c->method == WRS_METHOD_ITS && c->coop_size != 0 && c->coop_size < 32)
        return fail(WRS_ERR_INVALID_ARG, "ITS coop_size must be 0 or >= 32");
    if (c->coop_size != 0 && c->rng != WRS_RNG_REFERENCE)
        return fail(WRS_ERR_INVALID_ARG, "cooperative sampling exists only with the reference RNG");
    if (c->coop_size > (1u << 30)) return fail(WRS_ERR_INVALID_ARG, "coop_size too large");
    return WRS_OK;
}

constexpr uint32_t kMaxN = 0x7fffffffu;  // indices are handled as int where the shaders use int

}  // namespace

int wrs::set_last_error(int status, const char* msg) {
    g_last_error = msg;
    return status;
}

extern "C" {

int wrs_version(void) { return WRS_VERSION; }

const char* wrs_status_string(wrs_status s) {
    switch (s) {
        case WRS_OK: return "ok";
        case WRS_ERR_INVALID_ARG: return "invalid argument";
        case WRS_ERR_OOM: return "out of device memory";
        case WRS_ERR_TIMEOUT: return "a lookback wait gave up";
        case WRS_ERR_CUDA: return "CUDA error";
        case WRS_ERR_NOT_IMPLEMENTED: return "not implemented";
        case WRS_ERR_CAPACITY: return "n exceeds the buffers' capacity";
    }
    return "unknown status";
}

const char* wrs_last_error(void) { return g_last_error.c_str(); }

wrs_status wrs_config_init(wrs_config* cfg, uint32_t method) {
    if (!cfg) return fail(WRS_ERR_INVALID_ARG, "config is NULL");
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->method = method;
    cfg->split_size = 2;
    cfg->use_partition_elements = 1;
    cfg->coop_size = 0;
    cfg->its_parray = 0;
    cfg->rng = WRS_RNG_REFERENCE;
    cfg->scan_precision = WRS_SCAN_FP32;
    cfg->split_residual_f64 = 0;
    cfg->split_full_light = 0;
    cfg->guiding_entry_size = method == WRS_METHOD_ITS ? 4u : 32u;
    return check_config(cfg);
}

wrs_status wrs_create(const wrs_config* cfg, wrs_handle** out) {
    if (!out) return fail(WRS_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    wrs_status s = check_config(cfg);
    if (s != WRS_OK) return s;
    wrs_handle* h = new (std::nothrow) wrs_handle;
    if (!h) return fail(WRS_ERR_OOM, "host allocation failed");
    h->cfg = *cfg;
    *out = h;
    return WRS_OK;
}

void wrs_destroy(wrs_handle* h) { delete h; }

size_t wrs_buffers_bytes(const wrs_handle* h, uint32_t max_n) {
    if (!h) return 0;
    return layout_for(h->cfg, max_n).total;
}

wrs_status wrs_buffers_create(const wrs_handle* h, uint32_t max_n, wrs_buffers** out) {
    if (!h || !out) return fail(WRS_ERR_INVALID_ARG, "handle or out is NULL");
    *out = nullptr;
    if (max_n == 0 || max_n > kMaxN) return fail(WRS_ERR_INVALID_ARG, "max_n out of range");
    const Layout L = layout_for(h->cfg, max_n);
    wrs_buffers* b = new (std::nothrow) wrs_buffers;
    if (!b) return fail(WRS_ERR_OOM, "host allocation failed");
    b->cfg = h->cfg;
    b->max_n = max_n;
    b->cap_tiles = tiles_for(max_n) + 1;
    cudaError_t e = cudaMalloc(&b->base, L.total);
    if (e != cudaSuccess) {
        delete b;
        (void)cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? fail(WRS_ERR_OOM, "cudaMalloc failed")
                                              : cuda_fail(e, "cudaMalloc");
    }
    b->bytes = L.total;
    char* p = static_cast<char*>(b->base);
    b->ctrl = reinterpret_cast<BuildCtrl*>(p + L.ctrl);
    b->partials = reinterpret_cast<double*>(p + L.partials);
    const bool alias = h->cfg.method == WRS_METHOD_ALIAS_TABLE;
    b->part_states = alias ? reinterpret_cast<PartState*>(p + L.part_states) : nullptr;
    b->scan_states = reinterpret_cast<ScanState*>(p + L.scan_states);
    b->tile_scratch = reinterpret_cast<uint32_t*>(p + L.tile_scratch);
    if (alias) {
        b->idx = reinterpret_cast<uint32_t*>(p + L.idx);
        b->prefix = reinterpret_cast<float*>(p + L.prefix);
        b->elems = h->cfg.use_partition_elements ? reinterpret_cast<float*>(p + L.elems) : nullptr;
        b->prefix_lo = h->cfg.scan_precision == WRS_SCAN_FLOAT_FLOAT
                           ? reinterpret_cast<float*>(p + L.prefix_lo)
                           : nullptr;
        b->table = reinterpret_cast<uint2*>(p + L.table);
        b->coins = L.coins ? reinterpret_cast<uint8_t*>(p + L.coins) : nullptr;
        b->descent = reinterpret_cast<int2*>(p + L.descent);
        b->records = L.records ? reinterpret_cast<SplitRecord*>(p + L.records) : nullptr;
    } else {
        b->cmf = reinterpret_cast<float*>(p + L.cmf);
        b->guide = L.guide ? reinterpret_cast<uint32_t*>(p + L.guide) : nullptr;
        b->cells = L.cells ? reinterpret_cast<ItsCell*>(p + L.cells) : nullptr;
        b->tree = L.tree ? reinterpret_cast<TreeBlock*>(p + L.tree) : nullptr;
        b->coarse = L.coarse ? reinterpret_cast<uint32_t*>(p + L.coarse) : nullptr;
    }
    e = cudaMemset(b->base, 0, zeroed_bytes(h->cfg, max_n));
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        cudaFree(b->base);
        delete b;
        return cuda_fail(e, "cudaMemset");
    }
    *out = b;
    return WRS_OK;
}

void wrs_buffers_destroy(wrs_buffers* b) {
    if (!b) return;
    if (b->base) cudaFree(b->base);
    delete b;
}

static wrs_status check_n(const wrs_buffers* b, uint32_t n) {
    if (!b) return fail(WRS_ERR_INVALID_ARG, "buffers is NULL");
    if (n == 0) return fail(WRS_ERR_INVALID_ARG, "n must be >= 1");
    if (n > b->max_n) return fail(WRS_ERR_CAPACITY, "n exceeds the buffers' capacity");
    return WRS_OK;
}

wrs_status wrs_total_mass(const wrs_handle* h, void* stream, const float* weights, uint32_t n,
                          wrs_buffers* b) {
    if (!h || !weights) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    WRS_CUDA(launch_total_mass(as_stream(stream), weights, n, b->partials, b->ctrl), "total mass");
    return WRS_OK;
}

wrs_status wrs_prefix_sum(const wrs_handle* h, void* stream, const float* in, uint32_t n,
                          float* out, wrs_buffers* b) {
    if (!h || !in || !out) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    WRS_CUDA(launch_scan(as_stream(stream), h->cfg.scan_precision != WRS_SCAN_FP32, in, n,
                         out, b->ctrl, b->scan_states, b->cap_tiles, b->partials),
             "prefix sum");
    return WRS_OK;
}

static bool float_float(const wrs_handle* h) {
    return h->cfg.scan_precision == WRS_SCAN_FLOAT_FLOAT;
}
static bool compensated(const wrs_handle* h) {
    return h->cfg.scan_precision != WRS_SCAN_FP32;
}
// ITS sampling steered by a guiding table: the compensated CMF is exactly non-decreasing, so
// any lower-bound search returns the bisection's index
static bool its_guided(const wrs_handle* h) {
    return h->cfg.method == WRS_METHOD_ITS && h->cfg.coop_size == 0 &&
           h->cfg.guiding_entry_size != 0;
}
// the guiding table / cell blocks the handle will use exist in b and have its size
static wrs_status check_tables(const wrs_handle* h, const wrs_buffers* b) {
    if ((h->cfg.method == WRS_METHOD_CUTPOINT || its_guided(h)) &&
        b->cfg.guiding_entry_size != h->cfg.guiding_entry_size)
        return fail(WRS_ERR_INVALID_ARG, "buffers were created for another guiding_entry_size");
    if ((its_guided(h) && (!b->cells || !b->coarse)) ||
        (h->cfg.method == WRS_METHOD_CUTPOINT && compensated(h) && !b->coarse))
        return fail(WRS_ERR_INVALID_ARG,
                    "buffers were created without the cell blocks or the construction scratch "
                    "this handle's search uses");
    return WRS_OK;
}

wrs_status wrs_prefix_partition(const wrs_handle* h, void* stream, const float* weights,
                                uint32_t n, uint32_t* partition_indices, float* partition_prefix,
                                float* partition_elements, float* partition_prefix_lo,
                                wrs_buffers* b) {
    if (!h || !weights || !partition_indices || !partition_prefix)
        return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    if ((partition_prefix_lo != nullptr) != float_float(h))
        return fail(WRS_ERR_INVALID_ARG,
                    "partition_prefix_lo is required exactly with WRS_SCAN_FLOAT_FLOAT");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    if (!b->part_states) return fail(WRS_ERR_INVALID_ARG, "buffers were not created for the alias method");
    WRS_CUDA(launch_prefix_partition(as_stream(stream), compensated(h), weights, n, b->ctrl,
                                     b->part_states, b->cap_tiles, partition_indices,
                                     partition_prefix, partition_elements, partition_prefix_lo),
             "prefix partition");
    return WRS_OK;
}

wrs_status wrs_split_pack(const wrs_handle* h, void* stream, const float* weights,
                          const uint32_t* partition_indices, const float* partition_prefix,
                          const float* partition_elements, const float* partition_prefix_lo,
                          uint32_t n, wrs_alias_entry* table, wrs_buffers* b) {
    if (!h || !weights || !partition_indices || !partition_prefix || !table)
        return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    if ((partition_prefix_lo != nullptr) != float_float(h))
        return fail(WRS_ERR_INVALID_ARG,
                    "partition_prefix_lo is required exactly with WRS_SCAN_FLOAT_FLOAT");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    if (h->cfg.split_size == 0) return fail(WRS_ERR_INVALID_ARG, "split_size must be >= 1");
    b->coins_n = 0;  // the table may be the buffers' own: its coin filter no longer holds
    WRS_CUDA(launch_split_pack(as_stream(stream), h->cfg.split_residual_f64 != 0,
                               h->cfg.split_full_light != 0, weights, partition_indices,
                               partition_elements, partition_prefix, partition_prefix_lo, b->ctrl,
                               &b->ctrl->status, n, h->cfg.split_size,
                               reinterpret_cast<uint2*>(table), b->descent),
             "split pack");
    return WRS_OK;
}

wrs_status wrs_prefix_sum_blockwise(const wrs_handle* h, void* stream, const float* in,
                                    uint32_t n, float* out, wrs_buffers* b) {
    if (!h || !in || !out) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    WRS_CUDA(launch_prefix_sum_blockwise(as_stream(stream), in, n, out,
                                         reinterpret_cast<float*>(b->tile_scratch)),
             "block-wise prefix sum");
    return WRS_OK;
}

wrs_status wrs_prefix_partition_blockwise(const wrs_handle* h, void* stream, const float* weights,
                                          uint32_t n, uint32_t* partition_indices,
                                          float* partition_prefix, float* partition_elements,
                                          wrs_buffers* b) {
    if (!h || !weights || !partition_indices || !partition_prefix)
        return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    WRS_CUDA(launch_prefix_partition_blockwise(as_stream(stream), weights, n, b->ctrl,
                                               b->tile_scratch, partition_indices,
                                               partition_prefix, partition_elements),
             "block-wise prefix partition");
    return WRS_OK;
}

uint32_t wrs_split_records_count(uint32_t n, uint32_t split_size) {
    return split_size ? records_for(n, split_size) : 0u;
}

wrs_status wrs_split(const wrs_handle* h, void* stream, const float* partition_prefix,
                     const float* partition_prefix_lo, uint32_t n, wrs_split_record* records,
                     wrs_buffers* b) {
    if (!h || !partition_prefix || !records) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    if ((partition_prefix_lo != nullptr) != float_float(h))
        return fail(WRS_ERR_INVALID_ARG,
                    "partition_prefix_lo is required exactly with WRS_SCAN_FLOAT_FLOAT");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    if (h->cfg.split_size == 0) return fail(WRS_ERR_INVALID_ARG, "split_size must be >= 1");
    WRS_CUDA(launch_split_records(as_stream(stream), h->cfg.split_residual_f64 != 0,
                                  h->cfg.split_full_light != 0, partition_prefix,
                                  partition_prefix_lo, b->ctrl, n, h->cfg.split_size,
                                  reinterpret_cast<SplitRecord*>(records)),
             "split records");
    return WRS_OK;
}

wrs_status wrs_pack(const wrs_handle* h, void* stream, const float* weights,
                    const uint32_t* partition_indices, const float* partition_elements,
                    const wrs_split_record* records, uint32_t n, wrs_alias_entry* table,
                    wrs_buffers* b) {
    if (!h || !weights || !partition_indices || !records || !table)
        return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    if (h->cfg.split_size == 0) return fail(WRS_ERR_INVALID_ARG, "split_size must be >= 1");
    const SplitRecord* r = reinterpret_cast<const SplitRecord*>(records);
    uint2* t = reinterpret_cast<uint2*>(table);
    b->coins_n = 0;  // the table may be the buffers' own: its coin filter no longer holds
    const bool fl = h->cfg.split_full_light != 0;
    WRS_CUDA(h->cfg.split_pack_mode == WRS_SPLITPACK_SERIAL_SUBGROUP
                 ? launch_pack_records_warp(as_stream(stream), fl, weights, partition_indices,
                                            partition_elements, b->ctrl, &b->ctrl->status, n,
                                            h->cfg.split_size, r, t)
                 : launch_pack_records(as_stream(stream), fl, weights, partition_indices,
                                       partition_elements, b->ctrl, &b->ctrl->status, n,
                                       h->cfg.split_size, r, t),
             "pack");
    return WRS_OK;
}

wrs_status wrs_alias_sample(const wrs_handle* h, void* stream, const wrs_alias_entry* table,
                            uint32_t n, uint64_t s, uint64_t seed, uint64_t offset,
                            uint32_t* samples) {
    if (!h || !table || (!samples && s)) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0 || n > kMaxN) return fail(WRS_ERR_INVALID_ARG, "n out of range");
    if (s == 0) return WRS_OK;
    WRS_CUDA(launch_alias_sample(as_stream(stream), h->cfg.rng, h->cfg.coop_size,
                                 reinterpret_cast<const uint2*>(table), nullptr, nullptr, n, s,
                                 seed, offset, samples),
             "alias sample");
    return WRS_OK;
}

wrs_status wrs_its_sample(const wrs_handle* h, void* stream, const float* cmf, uint32_t n,
                          uint64_t s, uint64_t seed, uint64_t offset, uint32_t* samples) {
    if (!h || !cmf || (!samples && s)) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0 || n > kMaxN) return fail(WRS_ERR_INVALID_ARG, "n out of range");
    if (s == 0) return WRS_OK;
    WRS_CUDA(launch_its_sample(as_stream(stream), h->cfg.rng, h->cfg.coop_size,
                               h->cfg.its_parray != 0, cmf, n, s, seed, offset, samples),
             "its sample");
    return WRS_OK;
}

wrs_status wrs_cutpoint_guide(const wrs_handle* h, void* stream, const float* cmf, uint32_t n,
                              uint32_t* guide) {
    if (!h || !cmf || !guide) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0 || n > kMaxN) return fail(WRS_ERR_INVALID_ARG, "n out of range");
    if (h->cfg.method != WRS_METHOD_CUTPOINT)
        return fail(WRS_ERR_INVALID_ARG, "the handle is not configured for the Cutpoint method");
    WRS_CUDA(launch_cutpoint_guide(as_stream(stream), cmf, n,
                                   guide_entries(n, h->cfg.guiding_entry_size), guide),
             "guiding table");
    return WRS_OK;
}

wrs_status wrs_cutpoint_sample(const wrs_handle* h, void* stream, const float* cmf, uint32_t n,
                               const uint32_t* guide, uint64_t s, uint64_t seed, uint64_t offset,
                               uint32_t* samples) {
    if (!h || !cmf || !guide || (!samples && s)) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0 || n > kMaxN) return fail(WRS_ERR_INVALID_ARG, "n out of range");
    if (h->cfg.method != WRS_METHOD_CUTPOINT)
        return fail(WRS_ERR_INVALID_ARG, "the handle is not configured for the Cutpoint method");
    if (s == 0) return WRS_OK;
    WRS_CUDA(launch_cutpoint_sample(as_stream(stream), h->cfg.rng, cmf, n, guide,
                                    guide_entries(n, h->cfg.guiding_entry_size), s, seed, offset,
                                    samples),
             "cutpoint sample");
    return WRS_OK;
}

wrs_status wrs_build(const wrs_handle* h, void* stream, const float* weights, uint32_t n,
                     wrs_buffers* b) {
    if (!h || !weights) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    if (b->cfg.method != h->cfg.method)
        return fail(WRS_ERR_INVALID_ARG, "buffers were created for another method");
    if ((s = check_tables(h, b)) != WRS_OK) return s;
    const cudaStream_t st = as_stream(stream);
    const bool comp = compensated(h);
    if (h->cfg.method != WRS_METHOD_ALIAS_TABLE) {
        WRS_CUDA(launch_scan(st, comp, weights, n, b->cmf, b->ctrl, b->scan_states, b->cap_tiles,
                             b->partials),
                 "ITS build");
        // the compensated CMF is exactly non-decreasing: the galloping construction gives
        // the bisection's entries
        const uint32_t G = guide_entries(n, h->cfg.guiding_entry_size);
        if (h->cfg.method == WRS_METHOD_CUTPOINT)
            WRS_CUDA(comp ? launch_guide_monotone(st, b->cmf, n, G, b->coarse, b->guide)
                          : launch_cutpoint_guide(st, b->cmf, n, G, b->guide),
                     "guiding table");
        else if (its_guided(h)) {
            // an FP32 CMF need not be monotone: mark the cells the search cannot serve
            b->cells_n = 0;
            WRS_CUDA(launch_its_cells(st, b->cmf, n, G, b->coarse, b->cells, !comp), "ITS cells");
            if (!comp)
                WRS_CUDA(launch_its_marks(st, b->cmf, n, G, b->cells,
                                          reinterpret_cast<float*>(b->tile_scratch),
                                          b->tile_scratch + 2u * b->cap_tiles),
                         "ITS cell marks");
            b->cells_n = n;
        }
        b->tree_n = 0;
        if (b->tree && its_tree_levels(h->cfg, n)) {
            WRS_CUDA(launch_its_tree(st, b->cmf, n, its_tree_stored_levels(n), b->tree),
                     "ITS probe tree");
            b->tree_n = n;
        }
        return WRS_OK;
    }
    if (h->cfg.use_partition_elements && !b->elems)
        return fail(WRS_ERR_INVALID_ARG, "buffers were created without partition elements");
    if (float_float(h) && !b->prefix_lo)
        return fail(WRS_ERR_INVALID_ARG, "buffers were created without the float-float prefix");
    float* elems = h->cfg.use_partition_elements ? b->elems : nullptr;
    float* lo = float_float(h) ? b->prefix_lo : nullptr;
    b->coins_n = 0;
    WRS_CUDA(launch_total_mass(st, weights, n, b->partials, b->ctrl), "total mass");
    WRS_CUDA(launch_prefix_partition(st, comp, weights, n, b->ctrl, b->part_states, b->cap_tiles,
                                     b->idx, b->prefix, elems, lo),
             "prefix partition");
    if (h->cfg.split_pack_mode != WRS_SPLITPACK_INLINE) {
        // SerialSplitPack: the split records, then the pack from them
        if (!b->records || b->cfg.split_size != h->cfg.split_size)
            return fail(WRS_ERR_INVALID_ARG,
                        "buffers were created without split records for this split size");
        WRS_CUDA(launch_split_records(st, h->cfg.split_residual_f64 != 0,
                                      h->cfg.split_full_light != 0, b->prefix, lo, b->ctrl, n,
                                      h->cfg.split_size, b->records),
                 "split records");
        const bool fl = h->cfg.split_full_light != 0;
        WRS_CUDA(h->cfg.split_pack_mode == WRS_SPLITPACK_SERIAL_SUBGROUP
                     ? launch_pack_records_warp(st, fl, weights, b->idx, elems, b->ctrl,
                                                &b->ctrl->status, n, h->cfg.split_size,
                                                b->records, b->table)
                     : launch_pack_records(st, fl, weights, b->idx, elems, b->ctrl,
                                           &b->ctrl->status, n, h->cfg.split_size, b->records,
                                           b->table),
                 "pack");
    } else {
        WRS_CUDA(launch_split_pack(st, h->cfg.split_residual_f64 != 0,
                                   h->cfg.split_full_light != 0, weights, b->idx, elems, b->prefix,
                                   lo, b->ctrl, &b->ctrl->status, n, h->cfg.split_size, b->table,
                                   b->descent),
                 "split pack");
    }
    if (b->coins && n > kCoinMinN && n <= kCoinMaxN) {
        WRS_CUDA(launch_coin_filter(st, b->table, n, b->coins, &b->ctrl->coin_sum), "coin filter");
        b->coins_n = n;
    }
    return WRS_OK;
}

wrs_status wrs_sample_at(const wrs_handle* h, void* stream, const wrs_buffers* b, uint32_t n,
                         uint64_t s, uint64_t seed, uint64_t offset, uint32_t* samples) {
    if (!h) return fail(WRS_ERR_INVALID_ARG, "handle is NULL");
    wrs_status st = check_n(b, n);
    if (st != WRS_OK) return st;
    if (b->cfg.method != h->cfg.method)
        return fail(WRS_ERR_INVALID_ARG, "buffers were created for another method");
    if ((st = check_tables(h, b)) != WRS_OK) return st;
    if (h->cfg.method == WRS_METHOD_ITS) {
        if (its_guided(h) && s && b->cells_n == n) {
            // the cell-block search returns the bisection's index: for every target on the
            // compensated (non-decreasing) CMF, for the unmarked cells' targets on an FP32 one;
            // the marked cells bisect, through the stored probe tree when the build made it.
            // Cells written for another n (or none yet) are not read: the bisections below
            // give the same samples
            if (!samples) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
            const bool tree = !compensated(h) && b->tree && b->tree_n == n;
            WRS_CUDA(launch_its_sample_cells(as_stream(stream), h->cfg.rng, b->cmf, n, b->cells,
                                             guide_entries(n, h->cfg.guiding_entry_size), s,
                                             seed, offset, samples, tree ? b->tree : nullptr,
                                             tree ? its_tree_stored_levels(n) : 0u),
                     "its sample");
            return WRS_OK;
        }
        if (b->tree && b->tree_n == n && its_tree_levels(h->cfg, n) && s) {
            // the bisection with the probe tree's block levels read from the build's copy
            if (!samples) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
            WRS_CUDA(launch_its_sample(as_stream(stream), h->cfg.rng, 0, false, b->cmf, n, s, seed,
                                       offset, samples, b->tree + kTopBlocks,
                                       its_tree_block_levels(n)),
                     "its sample");
            return WRS_OK;
        }
        return wrs_its_sample(h, stream, b->cmf, n, s, seed, offset, samples);
    }
    if (h->cfg.method == WRS_METHOD_CUTPOINT)
        return wrs_cutpoint_sample(h, stream, b->cmf, n, b->guide, s, seed, offset, samples);
    if (b->coins && b->coins_n == n && s) {
        // the table's coin filter, written by the last build for this n: the same samples with
        // the table read only where the coin does not decide
        if (!samples) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
        WRS_CUDA(launch_alias_sample(as_stream(stream), h->cfg.rng, h->cfg.coop_size, b->table,
                                     b->coins, &b->ctrl->coin_sum, n, s, seed, offset, samples),
                 "alias sample");
        return WRS_OK;
    }
    return wrs_alias_sample(h, stream, reinterpret_cast<const wrs_alias_entry*>(b->table), n, s,
                            seed, offset, samples);
}

wrs_status wrs_sample(const wrs_handle* h, void* stream, const wrs_buffers* b, uint32_t n,
                      uint64_t s, uint64_t seed, uint32_t* samples) {
    return wrs_sample_at(h, stream, b, n, s, seed, 0, samples);
}

wrs_status wrs_buffers_status(wrs_buffers* b, void* stream, uint32_t* device_status) {
    if (!b) return fail(WRS_ERR_INVALID_ARG, "buffers is NULL");
    const cudaStream_t st = as_stream(stream);
    WRS_CUDA(cudaStreamSynchronize(st), "stream synchronize");
    uint32_t v = 0;
    WRS_CUDA(cudaMemcpy(&v, &b->ctrl->status, sizeof(v), cudaMemcpyDeviceToHost), "status read");
    if (v) WRS_CUDA(cudaMemset(&b->ctrl->status, 0, sizeof(v)), "status clear");
    if (device_status) *device_status = v;
    if (v & kStatusTimeout) return fail(WRS_ERR_TIMEOUT, "a lookback wait gave up");
    return WRS_OK;
}

wrs_status wrs_test_prefix_sum_stalled(const wrs_handle* h, void* stream, const float* in,
                                       uint32_t n, float* out, wrs_buffers* b,
                                       uint32_t spin_limit) {
    if (!h || !in || !out) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    wrs_status s = check_n(b, n);
    if (s != WRS_OK) return s;
    if (spin_limit == 0 || spin_limit > kSpinLimit)
        return fail(WRS_ERR_INVALID_ARG, "spin_limit out of range");
    const cudaStream_t st = as_stream(stream);
    const uint32_t one = 1;
    WRS_CUDA(cudaMemcpyAsync(&b->ctrl->scan.ticket, &one, sizeof(one), cudaMemcpyHostToDevice, st),
             "ticket preset");
    WRS_CUDA(launch_scan(st, h->cfg.scan_precision != WRS_SCAN_FP32, in, n, out, b->ctrl,
                         b->scan_states, b->cap_tiles, b->partials, spin_limit),
             "stalled prefix sum");
    return WRS_OK;
}

wrs_status wrs_buffers_set_partition_info(wrs_buffers* b, void* stream, float mean,
                                          double mean64, uint32_t heavy_count) {
    if (!b) return fail(WRS_ERR_INVALID_ARG, "buffers is NULL");
    const cudaStream_t st = as_stream(stream);
    WRS_CUDA(cudaMemcpyAsync(&b->ctrl->mean, &mean, sizeof(float), cudaMemcpyHostToDevice, st),
             "mean upload");
    WRS_CUDA(cudaMemcpyAsync(&b->ctrl->mean64, &mean64, sizeof(double), cudaMemcpyHostToDevice,
                             st),
             "mean64 upload");
    WRS_CUDA(cudaMemcpyAsync(&b->ctrl->heavy_count, &heavy_count, sizeof(uint32_t),
                             cudaMemcpyHostToDevice, st),
             "heavy count upload");
    WRS_CUDA(cudaStreamSynchronize(st), "stream synchronize");
    return WRS_OK;
}

const double* wrs_buffers_mean64(const wrs_buffers* b) { return b ? &b->ctrl->mean64 : nullptr; }

const wrs_alias_entry* wrs_buffers_alias_table(const wrs_buffers* b) {
    return b ? reinterpret_cast<const wrs_alias_entry*>(b->table) : nullptr;
}
const float* wrs_buffers_cmf(const wrs_buffers* b) { return b ? b->cmf : nullptr; }
const uint32_t* wrs_buffers_guide_table(const wrs_buffers* b) { return b ? b->guide : nullptr; }
const wrs_split_record* wrs_buffers_split_records(const wrs_buffers* b) {
    return b ? reinterpret_cast<const wrs_split_record*>(b->records) : nullptr;
}
const uint32_t* wrs_buffers_partition_indices(const wrs_buffers* b) { return b ? b->idx : nullptr; }
const float* wrs_buffers_partition_prefix(const wrs_buffers* b) { return b ? b->prefix : nullptr; }
const float* wrs_buffers_partition_elements(const wrs_buffers* b) { return b ? b->elems : nullptr; }
const float* wrs_buffers_partition_prefix_lo(const wrs_buffers* b) {
    return b ? b->prefix_lo : nullptr;
}
const float* wrs_buffers_mean(const wrs_buffers* b) { return b ? &b->ctrl->mean : nullptr; }
const double* wrs_buffers_total(const wrs_buffers* b) { return b ? &b->ctrl->total : nullptr; }
const uint32_t* wrs_buffers_heavy_count(const wrs_buffers* b) {
    return b ? &b->ctrl->heavy_count : nullptr;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------------

struct wrs_batch {
    wrs_config cfg;
    uint32_t max_dists = 0;
    uint64_t max_weights = 0, max_samples = 0;
    uint32_t cap_tiles = 0, cap_split = 0, cap_sample = 0;
    void* base = nullptr;
    size_t bytes = 0;
    BuildCtrl* bctrl = nullptr;  // batch tickets (part) and status
    DistDesc* staging = nullptr; // pinned host copy of the descriptors
    cudaEvent_t staged = nullptr;
    bool staged_pending = false;
    BatchView view{};
    uint32_t count = 0;
};

namespace {

struct BatchCaps {
    uint32_t tiles, split, sample;
};

bool batch_caps(const wrs_config& cfg, uint32_t max_dists, uint64_t max_weights,
                uint64_t max_samples, BatchCaps& c) {
    const uint64_t tiles = max_weights / kTileItems + max_dists + 1;
    const uint64_t split = max_weights / (static_cast<uint64_t>(cfg.split_size) * kSplitPack) +
                           max_dists + 1;
    const uint64_t sample = max_samples / kAliasPerBlock + max_dists + 1;
    if (tiles > 0x7fffffffull || split > 0x7fffffffull || sample > 0x7fffffffull) return false;
    c = {static_cast<uint32_t>(tiles), static_cast<uint32_t>(split),
         static_cast<uint32_t>(sample)};
    return true;
}

struct BatchLayout {
    size_t bctrl, dctrl, states, dist, partials, tile_map, split_map, descent, sample_map, idx,
        prefix,
        elems, prefix_lo, zero_end, total;
};

BatchLayout batch_layout(const wrs_config& cfg, uint32_t max_dists, uint64_t max_weights,
                         const BatchCaps& c) {
    BatchLayout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off = align_up(off + bytes, 256);
        return at;
    };
    L.bctrl = take(sizeof(BuildCtrl));
    L.dctrl = take(sizeof(BuildCtrl) * static_cast<size_t>(max_dists));
    L.states = take(sizeof(PartState) * 2 * static_cast<size_t>(c.tiles));
    L.zero_end = off;
    L.dist = take(sizeof(DistDesc) * static_cast<size_t>(max_dists));
    L.partials = take(sizeof(double) * static_cast<size_t>(c.tiles));
    L.tile_map = take(sizeof(uint32_t) * static_cast<size_t>(c.tiles));
    L.split_map = take(sizeof(uint32_t) * static_cast<size_t>(c.split));
    L.descent = take(sizeof(int2) * static_cast<size_t>(c.split));
    L.sample_map = take(sizeof(uint32_t) * static_cast<size_t>(c.sample));
    L.idx = take(sizeof(uint32_t) * max_weights);
    L.prefix = take(sizeof(float) * max_weights);
    L.elems = cfg.use_partition_elements ? take(sizeof(float) * max_weights) : 0;
    L.prefix_lo = cfg.scan_precision == WRS_SCAN_FLOAT_FLOAT ? take(sizeof(float) * max_weights) : 0;
    L.total = off;
    return L;
}

wrs_status check_batch_handle(const wrs_handle* h, const wrs_batch* b) {
    if (!h || !b) return fail(WRS_ERR_INVALID_ARG, "handle or batch is NULL");
    if (h->cfg.method != WRS_METHOD_ALIAS_TABLE)
        return fail(WRS_ERR_NOT_IMPLEMENTED, "batches exist for the alias method only");
    if (h->cfg.split_pack_mode != WRS_SPLITPACK_INLINE)
        return fail(WRS_ERR_NOT_IMPLEMENTED, "batches use the inline split-pack");
    if (h->cfg.split_size != b->cfg.split_size ||
        h->cfg.use_partition_elements != b->cfg.use_partition_elements ||
        h->cfg.scan_precision != b->cfg.scan_precision)
        return fail(WRS_ERR_INVALID_ARG,
                    "the batch was created for another split size, element or precision setting");
    return WRS_OK;
}

}  // namespace

extern "C" {

size_t wrs_batch_bytes(const wrs_handle* h, uint32_t max_dists, uint64_t max_weights,
                       uint64_t max_samples) {
    BatchCaps c;
    if (!h || h->cfg.method != WRS_METHOD_ALIAS_TABLE ||
        !batch_caps(h->cfg, max_dists, max_weights, max_samples, c))
        return 0;
    return batch_layout(h->cfg, max_dists, max_weights, c).total;
}

wrs_status wrs_batch_create(const wrs_handle* h, uint32_t max_dists, uint64_t max_weights,
                            uint64_t max_samples, wrs_batch** out) {
    if (!h || !out) return fail(WRS_ERR_INVALID_ARG, "handle or out is NULL");
    *out = nullptr;
    if (h->cfg.method != WRS_METHOD_ALIAS_TABLE)
        return fail(WRS_ERR_NOT_IMPLEMENTED, "batches exist for the alias method only");
    if (h->cfg.split_pack_mode != WRS_SPLITPACK_INLINE)
        return fail(WRS_ERR_NOT_IMPLEMENTED, "batches use the inline split-pack");
    if (max_dists == 0 || max_dists > (1u << 24))
        return fail(WRS_ERR_INVALID_ARG, "max_dists out of range");
    BatchCaps c;
    if (!batch_caps(h->cfg, max_dists, max_weights, max_samples, c))
        return fail(WRS_ERR_INVALID_ARG, "batch capacity out of range");
    const BatchLayout L = batch_layout(h->cfg, max_dists, max_weights, c);
    wrs_batch* b = new (std::nothrow) wrs_batch;
    if (!b) return fail(WRS_ERR_OOM, "host allocation failed");
    b->cfg = h->cfg;
    b->max_dists = max_dists;
    b->max_weights = max_weights;
    b->max_samples = max_samples;
    b->cap_tiles = c.tiles;
    b->cap_split = c.split;
    b->cap_sample = c.sample;
    cudaError_t e = cudaMalloc(&b->base, L.total);
    if (e != cudaSuccess) {
        delete b;
        (void)cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? fail(WRS_ERR_OOM, "cudaMalloc failed")
                                              : cuda_fail(e, "cudaMalloc");
    }
    b->bytes = L.total;
    e = cudaHostAlloc(reinterpret_cast<void**>(&b->staging), sizeof(DistDesc) * max_dists,
                      cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMemset(b->base, 0, L.zero_end);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        wrs_batch_destroy(b);
        return cuda_fail(e, "batch setup");
    }
    char* p = static_cast<char*>(b->base);
    b->bctrl = reinterpret_cast<BuildCtrl*>(p + L.bctrl);
    BatchView& v = b->view;
    v.dist = reinterpret_cast<const DistDesc*>(p + L.dist);
    v.tile_map = reinterpret_cast<const uint32_t*>(p + L.tile_map);
    v.split_map = reinterpret_cast<const uint32_t*>(p + L.split_map);
    v.descent = reinterpret_cast<int2*>(p + L.descent);
    v.sample_map = reinterpret_cast<const uint32_t*>(p + L.sample_map);
    v.dctrl = reinterpret_cast<BuildCtrl*>(p + L.dctrl);
    v.lb = &b->bctrl->part;
    v.status = &b->bctrl->status;
    v.states = reinterpret_cast<PartState*>(p + L.states);
    v.partials = reinterpret_cast<double*>(p + L.partials);
    v.idx = reinterpret_cast<uint32_t*>(p + L.idx);
    v.prefix = reinterpret_cast<float*>(p + L.prefix);
    v.elems = h->cfg.use_partition_elements ? reinterpret_cast<float*>(p + L.elems) : nullptr;
    v.prefix_lo = h->cfg.scan_precision == WRS_SCAN_FLOAT_FLOAT
                      ? reinterpret_cast<float*>(p + L.prefix_lo)
                      : nullptr;
    v.cap_tiles = c.tiles;
    v.split_size = h->cfg.split_size;
    v.full_light = h->cfg.split_full_light ? 1u : 0u;
    *out = b;
    return WRS_OK;
}

void wrs_batch_destroy(wrs_batch* b) {
    if (!b) return;
    if (b->staged) {
        cudaEventSynchronize(b->staged);
        cudaEventDestroy(b->staged);
    }
    if (b->staging) cudaFreeHost(b->staging);
    if (b->base) cudaFree(b->base);
    delete b;
}

wrs_status wrs_batch_set(wrs_batch* b, void* stream, const wrs_dist_desc* descs, uint32_t count) {
    if (!b) return fail(WRS_ERR_INVALID_ARG, "batch is NULL");
    if (count && !descs) return fail(WRS_ERR_INVALID_ARG, "descs is NULL");
    if (count > b->max_dists) return fail(WRS_ERR_CAPACITY, "more distributions than max_dists");
    uint64_t weights = 0, tiles = 0, split = 0, sample = 0, samples = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const wrs_dist_desc& d = descs[i];
        if (d.n == 0 || d.n > kMaxN) return fail(WRS_ERR_INVALID_ARG, "a distribution's n is out of range");
        if (!d.table) return fail(WRS_ERR_INVALID_ARG, "a distribution has no table");
        if (d.s && !d.samples) return fail(WRS_ERR_INVALID_ARG, "s > 0 with samples NULL");
        if (d.weights) {
            weights += d.n;
            tiles += tiles_for(d.n);
            split += split_blocks_for(d.n, b->cfg.split_size);
        }
        if (d.samples) {
            sample += alias_blocks_for(d.s);
            samples += d.s;
        }
    }
    if (weights > b->max_weights || tiles > b->cap_tiles || split > b->cap_split)
        return fail(WRS_ERR_CAPACITY, "the distributions' weights exceed max_weights");
    if (samples > b->max_samples || sample > b->cap_sample)
        return fail(WRS_ERR_CAPACITY, "the distributions' samples exceed max_samples");
    if (b->staged_pending) {
        WRS_CUDA(cudaEventSynchronize(b->staged), "staging wait");
        b->staged_pending = false;
    }
    uint64_t base = 0;
    uint32_t t0 = 0, s0 = 0, m0 = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const wrs_dist_desc& d = descs[i];
        DistDesc& o = b->staging[i];
        o.w = d.weights;
        o.table = reinterpret_cast<uint2*>(d.table);
        o.out = d.samples;
        o.s = d.samples ? d.s : 0;
        o.seed = d.seed;
        o.base = base;
        o.n = d.n;
        o.tile0 = t0;
        o.split0 = s0;
        o.sample0 = m0;
        if (d.weights) {
            base += d.n;
            t0 += tiles_for(d.n);
            s0 += split_blocks_for(d.n, b->cfg.split_size);
        }
        if (d.samples) m0 += static_cast<uint32_t>(alias_blocks_for(d.s));
    }
    const cudaStream_t st = as_stream(stream);
    BatchView& v = b->view;
    if (count) {
        WRS_CUDA(cudaMemcpyAsync(const_cast<DistDesc*>(v.dist), b->staging, sizeof(DistDesc) * count,
                                 cudaMemcpyHostToDevice, st),
                 "descriptor upload");
        WRS_CUDA(cudaEventRecord(b->staged, st), "staging event");
        b->staged_pending = true;
        WRS_CUDA(launch_batch_maps(st, v.dist, count, const_cast<uint32_t*>(v.tile_map),
                                   const_cast<uint32_t*>(v.split_map),
                                   const_cast<uint32_t*>(v.sample_map), b->cfg.split_size),
                 "batch maps");
    }
    v.tiles = t0;
    v.split_blocks = s0;
    v.sample_blocks = m0;
    b->count = count;
    return WRS_OK;
}

wrs_status wrs_batch_build(const wrs_handle* h, void* stream, wrs_batch* b) {
    wrs_status s = check_batch_handle(h, b);
    if (s != WRS_OK) return s;
    WRS_CUDA(launch_batch_build(as_stream(stream), h->cfg.scan_precision,
                                h->cfg.split_residual_f64 != 0, b->view),
             "batch build");
    return WRS_OK;
}

wrs_status wrs_batch_sample(const wrs_handle* h, void* stream, wrs_batch* b) {
    wrs_status s = check_batch_handle(h, b);
    if (s != WRS_OK) return s;
    WRS_CUDA(launch_batch_alias_sample(as_stream(stream), h->cfg.rng, h->cfg.coop_size, b->view),
             "batch sample");
    return WRS_OK;
}

wrs_status wrs_batch_status(wrs_batch* b, void* stream, uint32_t* device_status) {
    if (!b) return fail(WRS_ERR_INVALID_ARG, "batch is NULL");
    const cudaStream_t st = as_stream(stream);
    WRS_CUDA(cudaStreamSynchronize(st), "stream synchronize");
    uint32_t v = 0;
    WRS_CUDA(cudaMemcpy(&v, &b->bctrl->status, sizeof(v), cudaMemcpyDeviceToHost), "status read");
    if (v) WRS_CUDA(cudaMemset(&b->bctrl->status, 0, sizeof(v)), "status clear");
    if (device_status) *device_status = v;
    if (v & kStatusTimeout) return fail(WRS_ERR_TIMEOUT, "a lookback wait gave up");
    return WRS_OK;
}

uint32_t wrs_batch_count(const wrs_batch* b) { return b ? b->count : 0u; }

}  // extern "C"

uint32_t* wrs::batch_status_word(wrs_batch* b) { return &b->bctrl->status; }

/*
 * wrs.h -- C ABI of the GB300-native weighted-random-sampling hot path.
 *
 * This is the drop-in boundary for kistenklaus/merian-wrs's operator facade
 * `device::WRS` (src/device/wrs/WRS.hpp:91-172) and the kernels behind it.  Plain
 * pointers and sizes only: device pointers are CUDA device addresses, `stream` is a
 * cudaStream_t passed as void* (NULL = legacy default stream).  Every call is
 * asynchronous on `stream` unless stated otherwise and returns a wrs_status.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   wrs_config / wrs_config_init  WRSConfig = variant<ITS::Config, AliasTable::Config,
 *                                 Cutpoint::Config>            src/device/wrs/WRS.hpp:14
 *                                 PSAConfig                     src/device/wrs/alias/psa/PSA.hpp:19-41
 *                                 SampleAliasTableConfig        src/device/wrs/alias/sampling/AliasTableSampling.hpp:26-32
 *                                 InverseTransformSamplingConfig src/device/wrs/its/sampling/InverseTransformSampling.hpp:69-80
 *   wrs_create / wrs_destroy      WRS::WRS(context, shaderCompiler, config)  src/device/wrs/WRS.hpp:116-119
 *   wrs_buffers_create / _destroy WRSBuffers::allocate(alloc, mapping, N, S, config)
 *                                                               src/device/wrs/WRS.hpp:60-88
 *                                 (weights and samples stay caller-owned; the internals
 *                                  -- mean, heavyCount, partition arrays, table or CMF,
 *                                  lookback states -- live in wrs_buffers)
 *   wrs_build                     WRS::build(cmd, buffers, N, profiler)  src/device/wrs/WRS.hpp:121-143
 *   wrs_sample / wrs_sample_at    WRS::sample(cmd, buffers, N, S, seed = 12345)
 *                                                               src/device/wrs/WRS.hpp:145-168
 *   wrs_total_mass                Mean<float>::run              src/device/mean/Mean.hpp (AtomicMean::run)
 *   wrs_prefix_sum                PrefixSum<float>::run / DecoupledPrefixSum::run
 *                                                               src/device/prefix_sum/decoupled/DecoupledPrefixSum.hpp:174-199
 *   wrs_prefix_partition          PrefixPartition<float>::run / DecoupledPrefixPartition::run
 *                                                               src/device/prefix_partition/decoupled/DecoupledPrefixPartition.hpp:185-216
 *   wrs_split_pack                SplitPack::run / InlineSplitPack::run
 *                                                               src/device/wrs/alias/psa/splitpack/inline/InlineSplitPack.hpp:105-150
 *   wrs_alias_sample              SampleAliasTable::run         src/device/wrs/alias/sampling/AliasTableSampling.hpp:75-84
 *   wrs_its_sample                InverseTransformSampling::run src/device/wrs/its/sampling/InverseTransformSampling.hpp
 *   wrs_cutpoint_guide            CutpointGuidingTable::run     src/device/wrs/cutpoint/guiding_table/CutpointGuidingTable.hpp
 *   wrs_cutpoint_sample           CutpointSampling::run         src/device/wrs/cutpoint/sampling/CutpointSampling.hpp
 *                                 (Cutpoint::build / ::sample,  src/device/wrs/cutpoint/Cutpoint.hpp:108-158)
 *   wrs_philox                    PRNG::run / Philox::run       src/device/prng/PRNG.hpp:15-56,
 *                                                               src/device/prng/philox/Philox.hpp:94-108
 *   wrs_histogram,                Histogram, ChiSquare, RMSE    src/device/statistics
 *   wrs_sample_statistics
 *   wrs_batch_*, wrs_server_*,    no counterpart (the reference builds and samples one
 *   wrs_autotune_*                distribution per call, with a configuration fixed at
 *                                 construction)
 * The last section (test and calibration hooks) is not part of the drop-in path.
 *
 * Errors: the reference throws std::runtime_error("NOT-IMPLEMENTED") for unknown
 * variants (src/device/wrs/WRS.hpp:40,111,141,166); here every entry point returns a
 * status code instead, and wrs_last_error() gives the message of the calling thread's
 * last failure.  Device-side conditions (a lookback wait that ran out of budget,
 * overlapping PSA subproblems) are raised in a status word read by
 * wrs_buffers_status().
 *
 * Threading: a handle and a buffers object are not thread-safe; distinct objects are
 * independent.
 */
#ifndef WRS_GB300_H
#define WRS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WRS_VERSION 100

typedef enum wrs_status {
    WRS_OK = 0,
    WRS_ERR_INVALID_ARG = 1,
    WRS_ERR_OOM = 2,
    WRS_ERR_TIMEOUT = 3,         /* a lookback wait gave up (device status bit 1) */
    WRS_ERR_CUDA = 4,
    WRS_ERR_NOT_IMPLEMENTED = 5, /* e.g. a batch of a method other than the alias table */
    WRS_ERR_CAPACITY = 6         /* N larger than the buffers were created for */
} wrs_status;

/* the WRSConfig alternatives */
typedef enum wrs_method {
    WRS_METHOD_ALIAS_TABLE = 0, /* AliasTable: PSA build + alias sampling */
    WRS_METHOD_ITS = 1,         /* ITS: decoupled scan + inverse transform sampling */
    WRS_METHOD_CUTPOINT = 2     /* Cutpoint: decoupled scan + guiding table + guided sampling */
} wrs_method;

typedef enum wrs_rng {
    WRS_RNG_REFERENCE = 0,     /* the shaders' streams: Philox2x32-7 (alias), wang_hash (ITS,
                                  Cutpoint) */
    WRS_RNG_PHILOX4X32_10 = 1  /* Philox4x32-10, key = seed, counter = sample index */
} wrs_rng;

typedef enum wrs_scan_precision {
    WRS_SCAN_FP32 = 0,         /* FP32 carry through the lookback, as the reference */
    WRS_SCAN_COMPENSATED = 1,  /* FP32 with a two-sum (float-float) carry */
    WRS_SCAN_FLOAT_FLOAT = 2   /* alias method: compensated carry, and the partition prefix is
                                  kept as a float-float pair (an extra low-word array) so the
                                  split search decides on exact sums and the split residual
                                  is exact to FP64 rounding; ITS: as COMPENSATED */
} wrs_scan_precision;

/* PSA split + pack (PSAConfig::splitPack, src/device/wrs/alias/psa/splitpack/SplitPack.hpp) */
typedef enum wrs_split_pack_mode {
    WRS_SPLITPACK_INLINE = 0,         /* InlineSplitPack: splits computed and packed in one kernel
                                         (splitpack/inline/shader.comp), N / splitSize splits */
    WRS_SPLITPACK_SERIAL = 1,         /* SerialSplitPack = ScalarSplit + ScalarPack: ceil(N /
                                         splitSize) split records written to device memory
                                         (split/scalar/shader.comp), then one thread per
                                         subproblem packs from them (pack/scalar/float.comp) */
    WRS_SPLITPACK_SERIAL_SUBGROUP = 2 /* ScalarSplit + SubgroupPack's strategy: one warp per
                                         subproblem, items loaded 32 at a time and shuffled to the
                                         lockstep walk (pack/subgroup/shader.comp); the table is
                                         bit-identical to WRS_SPLITPACK_SERIAL's */
} wrs_split_pack_mode;

/* device status bits (wrs_buffers_status) */
#define WRS_DEVICE_TIMEOUT 1u
#define WRS_DEVICE_NONMONOTONE_SPLIT 2u

typedef struct wrs_config {
    uint32_t method;                 /* wrs_method */
    uint32_t split_size;             /* PSA InlineSplitPackConfig(splitSize); reference default 2 */
    uint32_t use_partition_elements; /* PSAConfig::usePartitionElements */
    uint32_t coop_size;              /* alias: SampleAliasTableConfig::cooperativeSampleSize;
                                        ITS: InverseTransformSamplingConfig::cooperativeSamplingSize
                                        (0 = off; otherwise >= 32) */
    uint32_t its_parray;             /* ITS: InverseTransformSamplingConfig::pArraySearch */
    uint32_t rng;                    /* wrs_rng */
    uint32_t scan_precision;         /* wrs_scan_precision */
    uint32_t split_residual_f64;     /* PSA split-point residual (spill) in FP64; the search
                                        keeps the shader's FP32 comparisons */
    uint32_t split_full_light;       /* PSA split caps the light count at lightCount instead of
                                        the shader's lightCount - 1
                                        (splitpack/inline/shader.comp:90,104), which at the end
                                        of the table can leave i + j < n and give the last
                                        light bucket extra mass; 0 = reference behaviour */
    uint32_t guiding_entry_size;     /* Cutpoint: CutpointConfig::guidingEntrySize, weights per
                                        guiding-table entry (table size ceil(N / this));
                                        default 32.  ITS with coop 0: the CMF is cut into as
                                        many equal-mass cells, each stored as a 32-byte block
                                        (its index range and 6 CMF values), and each sample
                                        reads the block of its cell instead of bisecting the
                                        whole CMF, with the same index: the compensated CMF is
                                        exactly non-decreasing; on an FP32 CMF the build marks
                                        the cells whose targets can meet a decrease of the CMF,
                                        and those samples bisect.  Default 4 for ITS; 0 = no
                                        cells (the bisection through the stored probe tree) */
    uint32_t split_pack_mode;        /* wrs_split_pack_mode: PSAConfig's splitPack alternative;
                                        default WRS_SPLITPACK_INLINE */
} wrs_config;

typedef struct wrs_alias_entry {
    float p;    /* keep-probability of the bucket (alias_table.hpp layout, 8 bytes) */
    uint32_t a; /* alias index */
} wrs_alias_entry;

/* A split between PSA subproblems: i light and j heavy items before it, spill = the residual of
 * heavy j (host::Split<float, uint32>, src/host/types/split.hpp:9-37; the std430 layout of the
 * shaders' Split, 12 bytes). */
typedef struct wrs_split_record {
    uint32_t i;
    uint32_t j;
    float spill;
} wrs_split_record;

typedef struct wrs_handle wrs_handle;
typedef struct wrs_buffers wrs_buffers;

int wrs_version(void);
const char* wrs_status_string(wrs_status s);
const char* wrs_last_error(void);

/* Defaults: alias = PSA split size 2, partition elements on, coop 0, reference RNG, FP32
 * scan; ITS = coop 0, reference RNG, FP32 scan; Cutpoint = guiding entry size 32, reference
 * RNG, FP32 scan. */
wrs_status wrs_config_init(wrs_config* cfg, uint32_t method);

wrs_status wrs_create(const wrs_config* cfg, wrs_handle** out);
void wrs_destroy(wrs_handle* h);

/* Internals for distributions of up to max_n weights (one cudaMalloc).  For ITS on the FP32
 * CMF above 2^16 weights they include the bisection's stored probe-tree blocks (at most ~2/7
 * of the CMF's bytes), which wrs_build writes and wrs_sample reads for the n built last; the
 * primitive wrs_its_sample probes the CMF alone (same samples).  For the alias method above
 * 2^22 weights they include the table's coin filter (one byte per weight up to 2^26): wrs_build
 * writes it after the table and wrs_sample reads it for the n built last, so that samples whose
 * coin decides skip the table read (same samples; wrs_split_pack and wrs_pack into the buffers
 * retire it until the next build, and the primitive wrs_alias_sample reads the table alone). */
size_t wrs_buffers_bytes(const wrs_handle* h, uint32_t max_n);
wrs_status wrs_buffers_create(const wrs_handle* h, uint32_t max_n, wrs_buffers** out);
void wrs_buffers_destroy(wrs_buffers* b);

/* Build the sampler (alias table or CMF) of `weights[0..n)` (device, FP32, >= 0) into b. */
wrs_status wrs_build(const wrs_handle* h, void* stream, const float* weights, uint32_t n,
                     wrs_buffers* b);
/* Draw s samples (uint32 indices) for sample indices [0, s).  `samples` is any address the
 * device can store to: device memory, or pinned host memory (cudaHostAlloc /
 * cudaHostRegister; on NVLink-C2C systems the kernel then writes the samples straight into
 * host memory, with no separate device-to-host copy). */
wrs_status wrs_sample(const wrs_handle* h, void* stream, const wrs_buffers* b, uint32_t n,
                      uint64_t s, uint64_t seed, uint32_t* samples);
/* Same for sample indices [offset, offset + s) of the stream. */
wrs_status wrs_sample_at(const wrs_handle* h, void* stream, const wrs_buffers* b, uint32_t n,
                         uint64_t s, uint64_t seed, uint64_t offset, uint32_t* samples);

/* Synchronises `stream`, returns WRS_DEVICE_* bits raised since the last call (and clears
 * them) in *device_status; WRS_ERR_TIMEOUT if a lookback wait gave up. */
wrs_status wrs_buffers_status(wrs_buffers* b, void* stream, uint32_t* device_status);

/* Device views of the internals (valid while b lives). */
const wrs_alias_entry* wrs_buffers_alias_table(const wrs_buffers* b);
const float* wrs_buffers_cmf(const wrs_buffers* b);              /* ITS and Cutpoint */
const uint32_t* wrs_buffers_guide_table(const wrs_buffers* b);   /* Cutpoint: ceil(N / entry) */
/* serial split-pack modes: the split records of the last build (wrs_split_records_count) */
const wrs_split_record* wrs_buffers_split_records(const wrs_buffers* b);
const uint32_t* wrs_buffers_partition_indices(const wrs_buffers* b);
const float* wrs_buffers_partition_prefix(const wrs_buffers* b);
const float* wrs_buffers_partition_elements(const wrs_buffers* b);
const float* wrs_buffers_partition_prefix_lo(const wrs_buffers* b); /* FLOAT_FLOAT only */
const float* wrs_buffers_mean(const wrs_buffers* b);        /* 1 float */
const double* wrs_buffers_total(const wrs_buffers* b);      /* 1 double */
const uint32_t* wrs_buffers_heavy_count(const wrs_buffers* b); /* 1 uint32 */

/* ---- primitives (device pointers; b supplies control block and scratch) ---------- */
wrs_status wrs_total_mass(const wrs_handle* h, void* stream, const float* weights, uint32_t n,
                          wrs_buffers* b);
wrs_status wrs_prefix_sum(const wrs_handle* h, void* stream, const float* in, uint32_t n,
                          float* out, wrs_buffers* b);
/* pivot = the mean held in b (run wrs_total_mass first); heavy count lands in b.
 * partition_elements may be NULL; partition_prefix_lo (the low words of the float-float
 * prefix) must be non-NULL exactly when the handle's precision is WRS_SCAN_FLOAT_FLOAT. */
wrs_status wrs_prefix_partition(const wrs_handle* h, void* stream, const float* weights,
                                uint32_t n, uint32_t* partition_indices,
                                float* partition_prefix, float* partition_elements,
                                float* partition_prefix_lo, wrs_buffers* b);
/* mean and heavy count are read from b; pointers as for wrs_prefix_partition */
wrs_status wrs_split_pack(const wrs_handle* h, void* stream, const float* weights,
                          const uint32_t* partition_indices, const float* partition_prefix,
                          const float* partition_elements, const float* partition_prefix_lo,
                          uint32_t n, wrs_alias_entry* table, wrs_buffers* b);
/* Block-wise (reduce-then-scan) baselines of the two decoupled-lookback kernels, kept for
 * comparison as the reference keeps BlockWiseScan (src/device/prefix_sum/block_wise/
 * BlockWiseScan.hpp:183-215) and BlockWisePrefixPartition (src/device/prefix_partition/
 * block_wise/BlockWisePrefixPartition.hpp:226-329): every 4096-weight tile is reduced, the tile
 * reductions are scanned, and every tile is scanned again with its offset (3 launches, the
 * weights read twice).  FP32 carries (the handle's precision does not apply); the partition's
 * pivot is the mean held in b (run wrs_total_mass first) and its heavy count lands in b. */
wrs_status wrs_prefix_sum_blockwise(const wrs_handle* h, void* stream, const float* in,
                                    uint32_t n, float* out, wrs_buffers* b);
wrs_status wrs_prefix_partition_blockwise(const wrs_handle* h, void* stream, const float* weights,
                                          uint32_t n, uint32_t* partition_indices,
                                          float* partition_prefix, float* partition_elements,
                                          wrs_buffers* b);
/* Serial split-pack (SerialSplitPack::run, src/device/wrs/alias/psa/splitpack/serial/
 * SerialSplitPack.hpp:52-93): wrs_split writes the K = wrs_split_records_count(n, split_size)
 * = ceil(n / split_size) records of ScalarSplit (split/scalar/shader.comp:72-133): record k - 1
 * for k in [1, K) at n_k = ceil(n * k / K), record K - 1 = (lightCount, heavyCount, 0); mean and
 * heavy count are read from b, the precision options are the handle's.  wrs_pack packs the K
 * subproblems [record k - 1, record k) from them (ScalarPack, pack/scalar/float.comp; with
 * WRS_SPLITPACK_SERIAL_SUBGROUP the warp-cooperative strategy of SubgroupPack, same table). */
uint32_t wrs_split_records_count(uint32_t n, uint32_t split_size);
wrs_status wrs_split(const wrs_handle* h, void* stream, const float* partition_prefix,
                     const float* partition_prefix_lo, uint32_t n, wrs_split_record* records,
                     wrs_buffers* b);
wrs_status wrs_pack(const wrs_handle* h, void* stream, const float* weights,
                    const uint32_t* partition_indices, const float* partition_elements,
                    const wrs_split_record* records, uint32_t n, wrs_alias_entry* table,
                    wrs_buffers* b);
wrs_status wrs_alias_sample(const wrs_handle* h, void* stream, const wrs_alias_entry* table,
                            uint32_t n, uint64_t s, uint64_t seed, uint64_t offset,
                            uint32_t* samples);
wrs_status wrs_its_sample(const wrs_handle* h, void* stream, const float* cmf, uint32_t n,
                          uint64_t s, uint64_t seed, uint64_t offset, uint32_t* samples);
/* Cutpoint guiding table of a CMF: guide[k] = first index with cmf >= (total / G) * k for
 * k < G = ceil(n / guiding_entry_size) (cutpoint/guiding_table/shader.comp:40-55). */
wrs_status wrs_cutpoint_guide(const wrs_handle* h, void* stream, const float* cmf, uint32_t n,
                              uint32_t* guide);
/* Cutpoint sampling (cutpoint/sampling/shader.comp:100-140): each group of 32 consecutive
 * samples picks one guiding-table cell, each sample bisects inside it. */
wrs_status wrs_cutpoint_sample(const wrs_handle* h, void* stream, const float* cmf, uint32_t n,
                               const uint32_t* guide, uint64_t s, uint64_t seed,
                               uint64_t offset, uint32_t* samples);
/* The standalone PRNG operator (PRNG::run with PhiloxConfig, src/device/prng/PRNG.hpp:15-56;
 * src/device/prng/philox/shader.comp:47-55): out[i] = float(x1) / 2^32 for i < n, with
 * (x0, x1) = the shaders' Philox2x32-7 (7 rounds, multiplier 0xD256D193, Weyl 0x9E3779B9) of
 * counter (i, 0) and key = seed; the float conversion rounds to nearest, so 1.0f can occur.
 * (The alias sampler's stream uses counter (0, i).)  out: n device floats. */
wrs_status wrs_philox(void* stream, uint32_t seed, uint32_t n, float* out);
/* Inclusive prefix sum (the scan of wrs_prefix_sum) that allocates no device memory, for
 * callers that cannot call cudaMalloc -- e.g. code running under a host application whose
 * pool already holds all device memory, code that must not take the device-wide
 * synchronisation of cudaMalloc/cudaFree, or code called from inside another allocator.  No
 * counterpart in the reference.  Instead of a wrs_buffers object it uses one fixed array
 * of about 1.2 MiB in this library's own device memory, so n must be <= 2^26 (67,108,864;
 * larger n returns WRS_ERR_CAPACITY).  The first call on a device looks up that array's
 * address and caches it; make that first call before capturing the stream into a CUDA
 * graph.  All calls share the array: each call clears it on `stream` before use, and calls
 * whose work overlaps on the GPU (different streams, or concurrent host threads) race and
 * give wrong results.  scan_precision is WRS_SCAN_FP32 or WRS_SCAN_COMPENSATED.  If
 * device_status is not NULL, the WRS_DEVICE_* bits of this call are copied to that
 * caller-owned device word on `stream`. */
wrs_status wrs_prefix_sum_noalloc(void* stream, const float* in, uint32_t n, float* out,
                                  uint32_t scan_precision, uint32_t* device_status);
/* Host helper: upload the FP32 mean, the FP64 mean (total / N, used by the float-float
 * mode's split targets) and the heavy count into b, for driving wrs_split_pack directly. */
wrs_status wrs_buffers_set_partition_info(wrs_buffers* b, void* stream, float mean,
                                          double mean64, uint32_t heavy_count);
/* device view of the FP64 mean (1 double) */
const double* wrs_buffers_mean64(const wrs_buffers* b);

/* ---- batches ------------------------------------------------------------------------
 * Many independent distributions of any sizes, built and sampled with one launch per
 * stage for the whole batch (4 build launches, 1 sampling launch), e.g. captured once into
 * a CUDA graph and replayed.  No counterpart in the reference, whose WRS::build and
 * WRS::sample (src/device/wrs/WRS.hpp:121-168) handle one distribution per call.  Each
 * distribution's table and samples are bit-for-bit those of wrs_build + wrs_sample on the
 * same weights, seed and handle configuration (total mass, partition and carries are
 * deterministic in the compensated precisions), whatever else the batch holds.  Alias
 * method only. */
typedef struct wrs_batch wrs_batch;

typedef struct wrs_dist_desc {
    const float* weights;   /* device, n FP32 weights >= 0; NULL: the table is already built
                               (sample only) */
    wrs_alias_entry* table; /* device, n entries: written by wrs_batch_build (if weights),
                               read by wrs_batch_sample (if samples) */
    uint32_t* samples;      /* device, s indices for sample indices [0, s); NULL: build only */
    uint64_t s;
    uint64_t seed;
    uint32_t n;             /* >= 1 */
    uint32_t reserved;      /* 0 */
} wrs_dist_desc;

/* Capacity: at most max_dists distributions, max_weights weights summed over the
 * distributions with weights, max_samples samples summed over all. */
size_t wrs_batch_bytes(const wrs_handle* h, uint32_t max_dists, uint64_t max_weights,
                       uint64_t max_samples);
wrs_status wrs_batch_create(const wrs_handle* h, uint32_t max_dists, uint64_t max_weights,
                            uint64_t max_samples, wrs_batch** out);
void wrs_batch_destroy(wrs_batch* b);
/* Sets the batch's distributions: copies the descriptors to the device and lays out the
 * batch's tile, split and sampling grids (one small kernel) on `stream`.  The pointers the
 * descriptors hold must stay valid while the batch is built or sampled.  Waits on the host
 * until the previous wrs_batch_set of this batch has finished its upload; not for use
 * inside a stream capture. */
wrs_status wrs_batch_set(wrs_batch* b, void* stream, const wrs_dist_desc* descs,
                         uint32_t count);
uint32_t wrs_batch_count(const wrs_batch* b);
/* Builds the table of every distribution with weights: 4 launches.  No host
 * synchronisation and no allocation, so the call can be captured into a CUDA graph. */
wrs_status wrs_batch_build(const wrs_handle* h, void* stream, wrs_batch* b);
/* Samples every distribution with samples: 1 launch; capturable like wrs_batch_build. */
wrs_status wrs_batch_sample(const wrs_handle* h, void* stream, wrs_batch* b);
/* As wrs_buffers_status, for the batch's device status word. */
wrs_status wrs_batch_status(wrs_batch* b, void* stream, uint32_t* device_status);

/* ---- served request loop --------------------------------------------------------------
 * Continuous batching of build+sample requests on top of the batches above.  No
 * counterpart in the reference.  Requests queue on the host (wrs_server_submit); each
 * wrs_server_progress call reaps finished batches, then admits queued requests in arrival
 * order into a batch for a free slot (one CUDA stream and one wrs_batch per slot) while
 * the device memory budget allows, and launches it, so that requests arriving while others
 * run on the GPU join the next batch and their work overlaps with the batches in flight.
 * Alias tables stay resident by table_id: a request naming a resident table only samples;
 * otherwise its table is built into the server's table arena, evicting the least recently
 * used tables that no batch in flight uses.  The budget covers the table arena and every
 * slot's batch scratch; weights and sample buffers are the caller's.  Each request's
 * samples equal those of a per-call wrs_build + wrs_sample of its weights and seed, in the
 * compensated precisions (see the batches above).  A server is not thread-safe. */
typedef struct wrs_server wrs_server;

typedef struct wrs_server_config {
    uint64_t memory_budget;     /* device bytes: table arena + batch scratch (default 16 GiB) */
    uint32_t slots;             /* batches in flight, one stream each (default 3) */
    uint32_t max_batch_dists;   /* requests per batch (default 1024) */
    uint64_t max_batch_weights; /* weights built per batch; bounds a request's n
                                   (default 2^25) */
    uint64_t max_batch_samples; /* samples per batch; bounds a request's s (default 2^24) */
} wrs_server_config;

typedef struct wrs_request {
    uint64_t table_id;     /* requests naming the same id share one table (same weights) */
    const float* weights;  /* device, n weights >= 0; read only when the table is built */
    uint32_t* samples;     /* device, s indices (sample indices [0, s) of the stream) */
    uint64_t s;
    uint64_t seed;
    uint32_t n;            /* 1 <= n <= max_batch_weights */
    uint32_t reserved;     /* 0 */
} wrs_request;

typedef struct wrs_completion {
    uint64_t ticket;   /* from wrs_server_submit */
    double submit_s;   /* host steady clock, seconds: submission (or trace arrival) */
    double done_s;     /* host steady clock, seconds: the batch was seen complete */
    uint32_t built;    /* 1: the table was built for this request; 0: a resident one */
    uint32_t status;   /* wrs_status of the request */
} wrs_completion;

typedef struct wrs_server_stats {
    uint64_t submitted, completed, batches, builds, reuses, evictions;
    uint64_t table_arena_bytes, table_bytes_peak, scratch_bytes;
    uint64_t device_status; /* OR of the batches' WRS_DEVICE_* bits */
} wrs_server_stats;

wrs_status wrs_server_config_init(wrs_server_config* c);
wrs_status wrs_server_create(const wrs_handle* h, const wrs_server_config* c,
                             wrs_server** out);
void wrs_server_destroy(wrs_server* s);
/* Queues a request (host only, no GPU work). */
wrs_status wrs_server_submit(wrs_server* s, const wrs_request* r, uint64_t* ticket);
/* One non-blocking scheduling step (reap, admit, launch); writes up to max_out completions. */
wrs_status wrs_server_progress(wrs_server* s, wrs_completion* out, uint32_t max_out,
                               uint32_t* count);
/* Number of submitted requests not yet reported complete. */
uint64_t wrs_server_pending(const wrs_server* s);
wrs_status wrs_server_get_stats(const wrs_server* s, wrs_server_stats* st);
/* Replays a trace in real time: request i is submitted arrival_s[i] seconds after the call
 * starts (arrival_s ascending), progress runs until every request completed, and out[i]
 * receives request i's completion with submit_s = the call's start + arrival_s[i]. */
wrs_status wrs_server_run_trace(wrs_server* s, const wrs_request* reqs,
                                const double* arrival_s, uint32_t count,
                                wrs_completion* out);

/* ---- sample statistics on the device (src/device/statistics) --------------------------
 * wrs_histogram: hist[samples[i]] += 1 for i < s (Histogram / AtomicHistogram,
 * statistics/histogram/atomic/shader.comp); hist is n device uint64 counters the caller zeroes
 * first; an index >= n is counted nowhere and ORs 4 into *device_status (a device word).
 * wrs_sample_statistics: from a histogram of s samples and the n weights, writes four device
 * doubles to out: the chi-square statistic sum over e_i > 0 of (o_i - e_i)^2 / e_i with
 * e_i = w_i * s / total (ChiSquare, statistics/chi_square/reduce/shader.comp), the RMSE
 * sqrt(mean((w_i / total - o_i / s)^2)) (statistics/rmse/mse/shader.comp), the number of
 * draws on zero-weight items, and the total weight.  Deterministic (fixed-order reductions,
 * where the reference adds with FP32 atomics).  scratch: wrs_statistics_scratch_bytes(n)
 * device bytes, 128-byte aligned, zeroed before its first use (the kernels leave it reusable). */
wrs_status wrs_histogram(void* stream, const uint32_t* samples, uint64_t s, uint32_t n,
                         uint64_t* hist, uint32_t* device_status);
size_t wrs_statistics_scratch_bytes(uint32_t n);
wrs_status wrs_sample_statistics(void* stream, const uint64_t* hist, const float* weights,
                                 uint32_t n, uint64_t s, void* scratch, double* out);

/* ---- autotuning (alias method) -----------------------------------------------------------
 * No counterpart in the reference, whose WRSConfig is fixed at construction
 * (src/device/wrs/WRS.hpp:116-119).  Two knobs are tuned by measurement (CUDA events on
 * `stream`, objective = build + sample milliseconds per call):
 *   split size  PSA InlineSplitPackConfig::splitSize (src/device/wrs/alias/psa/PSA.hpp:19-41):
 *               pack items per split.  Part of the table's definition: tables built with
 *               different split sizes differ in their bits, so per-call and batched builds
 *               that must agree use the same value.
 *   L2 fetch    the CUDA context's cudaLimitMaxL2FetchGranularity hint (bytes the L2 fetches
 *               from HBM per miss; alias sampling from tables larger than L2 is bound by
 *               it).  Context-wide, lasts as long as the context, changes no result.
 * The search is coordinate-wise: each L2 candidate at the configured split size, then each
 * split size at the best L2 value; the context's L2 limit is left at the chosen value.  The
 * tuner allocates (one handle and buffers or batch per candidate), synchronises the stream,
 * and overwrites the samples (and, for batches, the tables) its inputs name; not for use
 * inside a stream capture. */
typedef struct wrs_tune_space {
    const uint32_t* split_sizes; /* candidates; NULL = 4, 6, 8, 12, 16, 24, 32 (with count
                                    0 and NULL: only the configured size) */
    uint32_t split_count;
    const uint32_t* l2_fetch;    /* candidate granularities in bytes (0..128); NULL = 32, 64,
                                    128 (with count 0 and NULL: the L2 limit is not touched) */
    uint32_t l2_count;
    uint32_t warmup;             /* untimed calls per candidate (0 = 1) */
    uint32_t reps;               /* timed calls per candidate (0 = 3) */
} wrs_tune_space;

typedef struct wrs_tune_trial {
    uint32_t split_size;
    uint32_t l2_fetch;           /* 0 when the L2 limit was not tuned */
    float build_ms;              /* mean per call */
    float sample_ms;
} wrs_tune_trial;

typedef struct wrs_tune_result {
    uint32_t split_size;         /* the fastest candidate */
    uint32_t l2_fetch;           /* its L2 fetch granularity (0 when not tuned) */
    float build_ms;
    float sample_ms;
    uint32_t trials;             /* candidates measured */
} wrs_tune_result;

/* Sets / reads the current CUDA context's L2 fetch-granularity hint (bytes, <= 128). */
wrs_status wrs_set_l2_fetch_granularity(uint32_t bytes);
wrs_status wrs_get_l2_fetch_granularity(uint32_t* bytes);
/* Tunes one distribution: n device weights, s samples into `samples` (device, s entries;
 * s = 0 tunes the build alone).  `base` is an alias-method configuration; space NULL = the
 * defaults above; up to max_trials measurements are written to trials (may be NULL). */
wrs_status wrs_autotune_alias(const wrs_config* base, void* stream, const float* weights,
                              uint32_t n, uint64_t s, uint32_t* samples,
                              const wrs_tune_space* space, wrs_tune_result* out,
                              wrs_tune_trial* trials, uint32_t max_trials);
/* Tunes a batch: the distributions are those wrs_batch_set would take. */
wrs_status wrs_autotune_batch(const wrs_config* base, void* stream, const wrs_dist_desc* descs,
                              uint32_t count, const wrs_tune_space* space, wrs_tune_result* out,
                              wrs_tune_trial* trials, uint32_t max_trials);

/* ---- test and calibration hooks ------------------------------------------------------
 * Not part of the drop-in path: used by this library's own tests and benchmark. */
/* Test hook for the bounded-wait path: runs the scan of wrs_prefix_sum with its first
 * tile never scheduled (the tile ticket starts at 1) and a wait budget of `spin_limit`
 * polls, so every other tile's lookback runs out of budget.  The kernel still ends;
 * wrs_buffers_status then reports WRS_ERR_TIMEOUT and the context stays usable.
 * No counterpart in the reference (its DecoupledMean lookback breaks silently after
 * MAX_IT polls, src/device/mean/decoupled/float.comp:143). */
wrs_status wrs_test_prefix_sum_stalled(const wrs_handle* h, void* stream, const float* in,
                                       uint32_t n, float* out, wrs_buffers* b,
                                       uint32_t spin_limit);
/* Test hook for the server's table arena (host only, no device work): `iterations` random
 * allocations and releases of up to 4 MiB in a 1 GiB arena, checked against a shadow map
 * (no two live blocks overlap, the used byte count matches, everything released coalesces
 * back into one block).  Returns 0 when every check held, else the number of the first
 * check that failed. */
int wrs_test_arena(uint64_t seed, uint32_t iterations);
/* Device calibration: launches one `width`-byte load (4, 8, 16, 32, 64 or 128) per thread
 * from a hashed, width-aligned position in `buffer` (device memory, `bytes` long), `accesses`
 * threads in all; `sink` is a device word the kernel may write.  Time it with events on `stream`: with
 * width 8 the result is the device's random-gather rate, the bound of alias sampling from
 * tables larger than L2.  No counterpart in the reference. */
wrs_status wrs_probe_random_gather(void* stream, const void* buffer, uint64_t bytes,
                                   uint64_t accesses, uint32_t width, uint32_t* sink);

#ifdef __cplusplus
}
#endif
#endif /* WRS_GB300_H */

/*
 * wrs_oracle.h -- CPU oracle for the weighted-random-sampling hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path is
 * compared against (and the timed CPU baseline); the product never links,
 * loads or calls it.  Every function restates, in plain C, the arithmetic of
 * one reference shader or host routine of kistenklaus/merian-wrs and cites
 * the file:line it follows.  Floating-point code is compiled with
 * -ffp-contract=off so that every operation rounds once, exactly as the
 * device code (which uses __fadd_rn/__fmul_rn/__fdiv_rn) does.
 */
#ifndef WRS_ORACLE_H
#define WRS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    float p;    /* probability of keeping the bucket's own index */
    uint32_t a; /* alias index */
} wrso_entry;

/* RNG modes */
#define WRSO_RNG_REFERENCE 0u     /* Philox2x32-7 variant (alias) / wang_hash (ITS), as the shaders */
#define WRSO_RNG_PHILOX4X32_10 1u /* Random123 Philox4x32-10, key=seed, counter=sample index */

/* ---- counter-based generators ------------------------------------------------ */
void wrso_philox2x32_7(uint32_t c0, uint32_t c1, uint32_t key, uint32_t out[2]);
void wrso_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint32_t wrso_wang_hash(uint32_t seed);
float wrso_unit_ref(uint32_t x); /* float(x) / 2^32, round-to-nearest conversion */
/* the PRNG operator (prng/philox/shader.comp:47-55): out[i] = unit(Philox2x32-7((i, 0), seed).y) */
void wrso_philox_uniform(uint32_t seed, uint32_t n, float* out);

/* ---- build pieces ---------------------------------------------------------------- */
double wrso_total_mass(const float* w, uint64_t N);
float wrso_mean(const float* w, uint64_t N); /* (float)(sum_f64 / N) */
void wrso_partition(const float* w, uint32_t N, float pivot, uint32_t* idx, float* elems,
                    uint32_t* heavy_count);
void wrso_partition_prefix_f64(const float* w, uint32_t N, float pivot, double* prefix);
void wrso_prefix_f64(const float* w, uint64_t N, double* out);
void wrso_prefix_kahan(const float* w, uint64_t N, float* out);
void wrso_prefix_seq_f32(const float* w, uint64_t N, float* out);

/* split flags */
#define WRSO_SPLIT_F64 1          /* split-point residual (spill) in FP64 */
#define WRSO_SPLIT_FULL_LIGHT 2   /* light count capped at lightCount, not lightCount - 1 */
#define WRSO_SPLIT_FLOAT_FLOAT 4  /* wrso_psa_build: float-float prefix for the split search */

/* prefix_lo: low words of a float-float prefix (prefix = high words), or NULL.
 * mean64: total / N in FP64, the float-float mode's split targets (unused otherwise). */
void wrso_split(const float* prefix, const float* prefix_lo, uint32_t N, uint32_t heavy_count,
                float mean, double mean64, uint32_t n, int flags, uint32_t* i_out,
                uint32_t* j_out, float* spill_out);
void wrso_split_pack(const float* w, const uint32_t* idx, const float* elems, const float* prefix,
                     const float* prefix_lo, uint32_t heavy_count, float mean, double mean64,
                     uint32_t N, uint32_t split_size, int flags, wrso_entry* table,
                     uint32_t* splits /* 3*(K+1) or NULL */);
/* the same with the split searches on nthreads threads (the same table and splits) */
void wrso_split_pack_mt(const float* w, const uint32_t* idx, const float* elems,
                        const float* prefix, const float* prefix_lo, uint32_t heavy_count,
                        float mean, double mean64, uint32_t N, uint32_t split_size, int flags,
                        int nthreads, wrso_entry* table, uint32_t* splits);
/* Serial split-pack: ScalarSplit's ceil(N / split_size) records {i, j, spill} (3 words each)
 * and ScalarPack from them. */
void wrso_scalar_split(const float* prefix, const float* prefix_lo, uint32_t N, uint32_t heavy_count,
                       float mean, double mean64, uint32_t split_size, int flags,
                       uint32_t* records);
void wrso_scalar_pack(const float* w, const uint32_t* idx, const float* elems, uint32_t heavy_count,
                      float mean, uint32_t N, uint32_t split_size, int flags /* FULL_LIGHT */,
                      const uint32_t* records, wrso_entry* table);
/* Full PSA build on the CPU (mean -> partition -> prefix -> split+pack) with nthreads
 * worker threads.  Used as the timed CPU port of the reference path. */
void wrso_psa_build(const float* w, uint32_t N, uint32_t split_size, int flags, int nthreads,
                    wrso_entry* table, float* mean_out, uint32_t* heavy_count_out);

/* ---- sampling -------------------------------------------------------------------- */
void wrso_alias_sample(const wrso_entry* table, uint32_t N, uint64_t S, uint64_t seed,
                       uint64_t offset, uint32_t rng, uint32_t coop, int nthreads, uint32_t* out);
void wrso_its_sample(const float* cmf, uint32_t N, uint64_t S, uint64_t seed, uint64_t offset,
                     uint32_t rng, uint32_t coop, int parray, int nthreads, uint32_t* out);
void wrso_cutpoint_guide(const float* cmf, uint32_t N, uint32_t G, uint32_t* guide);
void wrso_cutpoint_sample(const float* cmf, uint32_t N, const uint32_t* guide, uint32_t G,
                          uint64_t S, uint64_t seed, uint64_t offset, uint32_t rng, int nthreads,
                          uint32_t* out);

/* ---- statistics ------------------------------------------------------------------ */
void wrso_histogram(const uint32_t* samples, uint64_t S, uint32_t N, uint64_t* hist);
double wrso_chi_square(const uint64_t* hist, const float* w, uint32_t N, uint64_t S);
double wrso_chi_square_binned(const uint64_t* hist, const float* w, uint32_t N, uint64_t S,
                              double min_expected, uint64_t* bins_out);
double wrso_chi2_sf(double x, double df);
double wrso_rmse(const uint64_t* hist, const float* w, uint32_t N, uint64_t S);
double wrso_js_divergence(const uint64_t* hist, const float* w, uint32_t N, uint64_t S);
void wrso_alias_to_weights(const wrso_entry* table, uint32_t N, double* out);

#ifdef __cplusplus
}
#endif
#endif

/*
 * wrs_oracle.c -- CPU oracle for the weighted-random-sampling hot path.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the CPU legs of
 * bench.py call this as the checker / CPU baseline.  The CUDA product never
 * links or calls it.
 *
 * Each function restates one routine of kistenklaus/merian-wrs (paths relative
 * to that project):
 *   Philox2x32-7 variant    src/device/wrs/alias/sampling/shader.comp:34-66
 *   wang_hash               src/device/wrs/its/sampling/shader.comp:70-78
 *   stable partition        src/device/prefix_partition/decoupled/shader.comp:329-361
 *                           (== src/host/reference/partition.hpp:37-52 + reversed light run)
 *   Kahan prefix            src/host/reference/prefix_sum.hpp:17-34
 *   split                   src/device/wrs/alias/psa/splitpack/inline/shader.comp:81-114
 *   pack                    src/device/wrs/alias/psa/splitpack/inline/shader.comp:130-223
 *   split+pack driver       src/device/wrs/alias/psa/splitpack/inline/shader.comp:225-270,
 *                           K = N / splitSize from .../inline/InlineSplitPack.hpp:116
 *   alias sampling          src/device/wrs/alias/sampling/shader.comp:68-111
 *   ITS sampling            src/device/wrs/its/sampling/shader.comp:80-177
 *   Cutpoint guiding table  src/device/wrs/cutpoint/guiding_table/shader.comp:40-55
 *   Cutpoint sampling       src/device/wrs/cutpoint/sampling/shader.comp:100-140
 *   chi-square statistic    src/host/statistics/chi_square.hpp:17-37
 *   RMSE                    src/dep/eval/rms.hpp:24-63
 *   JS divergence           src/host/statistics/js_divergence.hpp:48-92
 *   alias -> weights        src/host/reference/inverse_alias_table.hpp:15-30
 * Philox4x32-10 follows Salmon et al., "Parallel random numbers: as easy as
 * 1, 2, 3" (SC'11), the Random123 reference construction.
 */
#include "wrs_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* generators                                                                */
/* ------------------------------------------------------------------------- */

/* shader.comp:39-54 (alias sampling): 7 rounds of
 *   (hi,lo) = mulExtended(x0, 0xD256D193); x0 = x1 ^ hi; x1 = lo + k; k += 0x9E3779B9 */
void wrso_philox2x32_7(uint32_t c0, uint32_t c1, uint32_t key, uint32_t out[2]) {
    uint32_t x0 = c0, x1 = c1, k = key;
    for (int r = 0; r < 7; ++r) {
        uint64_t m = (uint64_t)x0 * 0xD256D193u;
        uint32_t hi = (uint32_t)(m >> 32), lo = (uint32_t)m;
        x0 = x1 ^ hi;
        x1 = lo + k;
        k += 0x9E3779B9u;
    }
    out[0] = x0;
    out[1] = x1;
}

/* src/device/prng/philox/shader.comp:47-55 (the PRNG operator): out[i] = float(x1) / 2^32 of
 * Philox2x32-7 at counter (i, 0), key = seed; the conversion rounds to nearest. */
void wrso_philox_uniform(uint32_t seed, uint32_t n, float* out) {
    uint32_t r[2];
    for (uint32_t i = 0; i < n; ++i) {
        wrso_philox2x32_7(i, 0u, seed, r);
        out[i] = wrso_unit_ref(r[1]);
    }
}

/* Random123 Philox4x32 with 10 rounds; key schedule bumped between rounds. */
void wrso_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t m0 = (uint64_t)0xD2511F53u * c0;
        uint64_t m1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(m0 >> 32), lo0 = (uint32_t)m0;
        uint32_t hi1 = (uint32_t)(m1 >> 32), lo1 = (uint32_t)m1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* its/sampling/shader.comp:70-78 (returns the hashed bits; the shader divides by 2^32). */
uint32_t wrso_wang_hash(uint32_t seed) {
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    return seed;
}

/* float(x) / 4294967296.0: the conversion rounds to nearest, the division by a
 * power of two is exact. */
float wrso_unit_ref(uint32_t x) {
    volatile float f = (float)x;
    return f * 2.3283064365386963e-10f;
}

/* ------------------------------------------------------------------------- */
/* threads                                                                   */
/* ------------------------------------------------------------------------- */

typedef void (*wrso_task_fn)(void* ctx, int t, int nt);
typedef struct {
    wrso_task_fn fn;
    void* ctx;
    int t, nt;
} wrso_task;

static void* wrso_task_main(void* p) {
    wrso_task* task = (wrso_task*)p;
    task->fn(task->ctx, task->t, task->nt);
    return NULL;
}

static void wrso_parallel(wrso_task_fn fn, void* ctx, int nt) {
    if (nt <= 1) {
        fn(ctx, 0, 1);
        return;
    }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
    wrso_task* tasks = (wrso_task*)malloc(sizeof(wrso_task) * (size_t)nt);
    for (int t = 0; t < nt; ++t) {
        tasks[t].fn = fn;
        tasks[t].ctx = ctx;
        tasks[t].t = t;
        tasks[t].nt = nt;
        if (t > 0) pthread_create(&th[t], NULL, wrso_task_main, &tasks[t]);
    }
    fn(ctx, 0, nt);
    for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
    free(th);
    free(tasks);
}

static void wrso_range(uint64_t n, int t, int nt, uint64_t* lo, uint64_t* hi) {
    uint64_t chunk = (n + (uint64_t)nt - 1) / (uint64_t)nt;
    *lo = chunk * (uint64_t)t;
    *hi = *lo + chunk;
    if (*lo > n) *lo = n;
    if (*hi > n) *hi = n;
}

/* ------------------------------------------------------------------------- */
/* build pieces                                                              */
/* ------------------------------------------------------------------------- */

double wrso_total_mass(const float* w, uint64_t N) {
    double s = 0.0;
    for (uint64_t i = 0; i < N; ++i) s += (double)w[i];
    return s;
}

float wrso_mean(const float* w, uint64_t N) {
    if (N == 0) return 0.0f;
    return (float)(wrso_total_mass(w, N) / (double)N);
}

/* Heavy items (w > pivot) ascending at [0, h); light items at N-1-lightRank, i.e.
 * the light run is stored in reverse: prefix_partition/decoupled/shader.comp:337-351. */
void wrso_partition(const float* w, uint32_t N, float pivot, uint32_t* idx, float* elems,
                    uint32_t* heavy_count) {
    uint32_t h = 0, l = 0;
    for (uint32_t i = 0; i < N; ++i) {
        if (w[i] > pivot) {
            idx[h] = i;
            if (elems) elems[h] = w[i];
            ++h;
        } else {
            idx[N - 1 - l] = i;
            if (elems) elems[N - 1 - l] = w[i];
            ++l;
        }
    }
    *heavy_count = h;
}

void wrso_partition_prefix_f64(const float* w, uint32_t N, float pivot, double* prefix) {
    uint32_t h = 0, l = 0;
    double hs = 0.0, ls = 0.0;
    for (uint32_t i = 0; i < N; ++i) {
        if (w[i] > pivot) {
            hs += (double)w[i];
            prefix[h++] = hs;
        } else {
            ls += (double)w[i];
            prefix[N - 1 - l] = ls;
            ++l;
        }
    }
}

void wrso_prefix_f64(const float* w, uint64_t N, double* out) {
    double s = 0.0;
    for (uint64_t i = 0; i < N; ++i) {
        s += (double)w[i];
        out[i] = s;
    }
}

/* src/host/reference/prefix_sum.hpp:17-34 with T = float. */
void wrso_prefix_kahan(const float* w, uint64_t N, float* out) {
    volatile float sum = 0.0f, c = 0.0f;
    for (uint64_t i = 0; i < N; ++i) {
        volatile float y = w[i] - c;
        volatile float t = sum + y;
        c = (t - sum) - y;
        sum = t;
        out[i] = sum;
    }
}

void wrso_prefix_seq_f32(const float* w, uint64_t N, float* out) {
    float s = 0.0f;
    for (uint64_t i = 0; i < N; ++i) {
        s += w[i];
        out[i] = s;
    }
}

/* splitpack/inline/shader.comp:81-114 (computeSplit).  Bisection over the number
 * of heavy items j in [0, heavyCount-1] with the shader's exact probe sequence and FP32
 * comparisons.
 * flags & WRSO_SPLIT_F64: evaluate the split-point residual (the spill) in FP64 and round
 * it once to FP32, instead of the shader's FP32 spill.
 * flags & WRSO_SPLIT_FULL_LIGHT: cap the light count at lightCount instead of the
 * shader's lightCount - 1 (shader.comp:90,104).  With the shader's cap a split near the
 * end of the table can have i + j < n, after which the last heavy bucket aliases a light
 * item that then gains mass; the full range keeps i + j = n.
 * prefix_lo != NULL (float-float prefix, prefix[] holding the high words): each comparison
 * sigma <= target and the final spill are evaluated in FP32 float-float arithmetic
 * (wrso_ff_sigma_minus) against target = (mean + mean_lo) * n as a float-float pair
 * (wrso_ff_target), where mean_lo = (float)(mean64 - mean) and mean64 = total / N in FP64.
 * This is the kernel's arithmetic operation for operation.
 * Guard beyond the shader: if every probe exceeds the target (b would wrap to
 * 0xFFFFFFFF in the shader), j = 0 is used. */
static inline float wrso_ff_sigma_minus(float h, float hl, float l, float ll, float t, float tl) {
    volatile float s = h + l;
    volatile float bp = s - h;
    volatile float ap = s - bp;
    volatile float e1 = h - ap, e2 = l - bp;
    volatile float e = e1 + e2;
    volatile float lo1 = e + hl;
    volatile float lo = lo1 + ll;
    volatile float d = s - t;
    volatile float dl = lo - tl;
    return d + dl;
}

static inline void wrso_ff_target(float m, float ml, uint32_t n, float* t, float* tl) {
    const float n1 = (float)(n & ~0xffu), n2 = (float)(n & 0xffu);
    volatile float p1 = m * n1;
    volatile float e1 = fmaf(m, n1, -p1);
    volatile float p2 = m * n2;
    volatile float e2 = fmaf(m, n2, -p2);
    volatile float p3 = ml * (float)n;
    volatile float s = p1 + p2;
    volatile float bp = s - p1;
    volatile float ap = s - bp;
    volatile float x1 = p1 - ap, x2 = p2 - bp;
    volatile float sl = x1 + x2;
    volatile float e12 = e1 + e2;
    volatile float e123 = e12 + p3;
    volatile float lo = sl + e123;
    volatile float hi = s + lo; /* fast two-sum */
    volatile float hs = hi - s;
    *t = hi;
    *tl = lo - hs;
}

void wrso_split(const float* prefix, const float* prefix_lo, uint32_t N, uint32_t hc, float mean,
                double mean64, uint32_t n, int flags, uint32_t* i_out, uint32_t* j_out,
                float* spill_out) {
    const uint32_t lc = N - hc;
    const uint32_t lcap = (flags & WRSO_SPLIT_FULL_LIGHT) ? lc : lc - 1;
    const int residual_f64 = (flags & WRSO_SPLIT_F64) != 0;
    int64_t a = 0, b = (int64_t)hc - 1;
    const float target = mean * (float)n;
    float t_hi = 0.0f, t_lo = 0.0f;
    if (prefix_lo) wrso_ff_target(mean, (float)(mean64 - (double)mean), n, &t_hi, &t_lo);
    while (a <= b) {
        uint32_t j = (uint32_t)((a + b) / 2);
        uint32_t i = (j > n) ? lcap : ((n - j) < lcap ? (n - j) : lcap);
        float heavy = j == 0 ? 0.0f : prefix[j - 1];
        float light = i == 0 ? 0.0f : prefix[N - i];
        int le;
        if (prefix_lo) {
            const float hl = j == 0 ? 0.0f : prefix_lo[j - 1];
            const float ll = i == 0 ? 0.0f : prefix_lo[N - i];
            le = wrso_ff_sigma_minus(heavy, hl, light, ll, t_hi, t_lo) <= 0.0f;
        } else {
            volatile float sigma = light + heavy;
            le = sigma <= target;
        }
        if (le)
            a = (int64_t)j + 1;
        else
            b = (int64_t)j - 1;
    }
    uint32_t j = b < 0 ? 0u : (uint32_t)b;
    uint32_t i = (j > n) ? lcap : ((n - j) < lcap ? (n - j) : lcap);
    float light = i == 0 ? 0.0f : prefix[N - i];
    float heavy2 = prefix[j];
    float spill;
    if (prefix_lo) {
        const float ll = i == 0 ? 0.0f : prefix_lo[N - i];
        spill = wrso_ff_sigma_minus(heavy2, prefix_lo[j], light, ll, t_hi, t_lo);
    } else if (residual_f64) {
        spill = (float)(((double)heavy2 + (double)light) - (double)mean * (double)n);
    } else {
        volatile float sigma2 = heavy2 + light;
        spill = sigma2 - target;
    }
    *i_out = i;
    *j_out = j;
    *spill_out = spill;
}

typedef struct {
    const float* w;
    const uint32_t* idx;
    const float* elems;
    uint32_t N, hc, lc;
    float mean;
    wrso_entry* table;
    int close_last; /* table-end rule (flags & WRSO_SPLIT_FULL_LIGHT), see wrso_pack */
} wrso_pack_ctx;

static inline float wrso_elem(const wrso_pack_ctx* c, uint32_t pos) {
    return c->elems ? c->elems[pos] : c->w[c->idx[pos]];
}

/* splitpack/inline/shader.comp:130-223 (pack).  Every arithmetic step rounds once.
 * close_last (the table-end rule that goes with the full light cap): the shader reads the
 * current heavy h = idx[j] and the next heavy idx[j + 1] even at j + 1 = heavyCount, where
 * position j + 1 holds the first light item, so the last heavy bucket's residual and every
 * light bucket packed after the heavies ran out alias a light item (possibly of weight zero).
 * With close_last, h = idx[min(j, heavyCount - 1)] and a heavy step at j + 1 = heavyCount
 * writes (1, h): the residual stays on the last heavy item. */
static void wrso_pack(const wrso_pack_ctx* c, uint32_t i0, uint32_t i1, uint32_t j0, uint32_t j1,
                      float spill) {
    const uint32_t N = c->N, hc = c->hc, lc = c->lc;
    const uint32_t lastLight = N - 1;
    const float mean = c->mean;
    uint32_t i = i0, j = j0;
    float w = spill;
    if (w == 0.0f) w = wrso_elem(c, j);
    while (i < i1 || j < j1) {
        int packHeavy;
        if (j == j1 || j == hc)
            packHeavy = 0;
        else if (i == i1 || i == lc)
            packHeavy = 1;
        else
            packHeavy = w <= mean;
        uint32_t h = c->idx[(c->close_last && j >= hc) ? hc - 1 : j];
        const int last = c->close_last && j + 1 == hc;
        uint32_t weightIdx;
        float weight;
        if (packHeavy) {
            weightIdx = c->idx[j + 1];
            weight = wrso_elem(c, j + 1);
        } else {
            weightIdx = c->idx[lastLight - i];
            weight = wrso_elem(c, lastLight - i);
        }
        float p;
        uint32_t idx, a;
        if (packHeavy) {
            p = last ? 1.0f : w / mean;
            a = last ? h : weightIdx;
            idx = h;
            j += 1;
        } else {
            p = weight / mean;
            a = h;
            idx = weightIdx;
            i += 1;
        }
        c->table[idx].p = p;
        c->table[idx].a = a;
        volatile float t = w + weight;
        w = t - mean;
    }
    if (j1 == hc - 1) {
        uint32_t h = c->idx[j];
        c->table[h].p = 1.0f;
        c->table[h].a = h;
    }
}

typedef struct {
    const float* prefix;
    const float* prefix_lo;
    uint32_t N, hc, split_size, K;
    float mean;
    double mean64;
    int flags;
    uint32_t* si;
    uint32_t* sj;
    float* ss;
} wrso_splits_ctx;

/* splits k in [1, K) of one thread's share (each split is independent of the others) */
static void wrso_splits_task(void* p, int t, int nt) {
    wrso_splits_ctx* c = (wrso_splits_ctx*)p;
    uint64_t lo, hi;
    wrso_range(c->K - 1u, t, nt, &lo, &hi);
    for (uint64_t k = lo + 1; k < hi + 1; ++k)
        wrso_split(c->prefix, c->prefix_lo, c->N, c->hc, c->mean, c->mean64,
                   (uint32_t)k * c->split_size, c->flags, &c->si[k], &c->sj[k], &c->ss[k]);
}

/* Driver of splitpack/inline/shader.comp:225-270: split k packs [split_k, split_{k+1})
 * for k in [0, K) with K = N / splitSize; split_0 = (0,0,0), split_K = (lc, hc, 0);
 * i1 = max(split_{k+1}.i, i0), j1 = max(split_{k+1}.j, j0).  Subproblems run in
 * increasing k, so where two subproblems write one entry the later k wins.
 * Guards beyond the shader (which is undefined there): heavyCount == 0 or N gives
 * table[i] = (1, i); K == 0 (N < splitSize) is treated as K = 1.
 * The K - 1 split searches (independent of each other) are spread over nthreads threads; the
 * pack loop then runs once, in increasing k, so the table does not depend on nthreads. */
void wrso_split_pack_mt(const float* w, const uint32_t* idx, const float* elems,
                        const float* prefix, const float* prefix_lo, uint32_t hc, float mean,
                        double mean64, uint32_t N, uint32_t split_size, int flags, int nthreads,
                        wrso_entry* table, uint32_t* splits) {
    if (N == 0) return;
    if (hc == 0 || hc == N) {
        for (uint32_t i = 0; i < N; ++i) {
            table[i].p = 1.0f;
            table[i].a = i;
        }
        return;
    }
    uint32_t K = N / split_size;
    if (K == 0) K = 1;
    wrso_splits_ctx sc = {prefix, prefix_lo, N, hc, split_size, K, mean, mean64, flags,
                          (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)K + 1)),
                          (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)K + 1)),
                          (float*)malloc(sizeof(float) * ((size_t)K + 1))};
    sc.si[0] = 0;
    sc.sj[0] = 0;
    sc.ss[0] = 0.0f;
    sc.si[K] = N - hc;
    sc.sj[K] = hc;
    sc.ss[K] = 0.0f;
    if (K > 1) wrso_parallel(wrso_splits_task, &sc, nthreads < 1 ? 1 : nthreads);
    wrso_pack_ctx c = {w, idx, elems, N, hc, N - hc, mean, table,
                       (flags & WRSO_SPLIT_FULL_LIGHT) != 0};
    for (uint32_t k = 0; k <= K; ++k) {
        if (splits) {
            splits[3 * k + 0] = sc.si[k];
            splits[3 * k + 1] = sc.sj[k];
            memcpy(&splits[3 * k + 2], &sc.ss[k], 4);
        }
        if (k == 0) continue;
        const uint32_t pi = sc.si[k - 1], pj = sc.sj[k - 1];
        const uint32_t i1 = sc.si[k] > pi ? sc.si[k] : pi;
        const uint32_t j1 = sc.sj[k] > pj ? sc.sj[k] : pj;
        wrso_pack(&c, pi, i1, pj, j1, sc.ss[k - 1]);
    }
    free(sc.si);
    free(sc.sj);
    free(sc.ss);
}

/* wrso_split_pack_mt on one thread */
void wrso_split_pack(const float* w, const uint32_t* idx, const float* elems, const float* prefix,
                     const float* prefix_lo, uint32_t hc, float mean, double mean64, uint32_t N,
                     uint32_t split_size, int flags, wrso_entry* table, uint32_t* splits) {
    wrso_split_pack_mt(w, idx, elems, prefix, prefix_lo, hc, mean, mean64, N, split_size, flags,
                       1, table, splits);
}

/* split/scalar/shader.comp:72-133 (ScalarSplit, the split half of SerialSplitPack):
 * K = ceil(N / splitSize) records of {i, j, spill}; record k - 1 for k in [1, K) is computeSplit
 * at n = ceilMulDiv(N, k, K) = ceil(N * k / K) in 64 bits (shader.comp:63-64), record K - 1 =
 * (lightCount, heavyCount, 0) (shader.comp:125-129).  Each split is wrso_split (the same
 * bisection, light cap and precision flags as the inline shader's computeSplit, which this
 * shader's computeSplit equals).  Guard beyond the shader: heavyCount == 0 or N makes every
 * record the final one. */
void wrso_scalar_split(const float* prefix, const float* prefix_lo, uint32_t N, uint32_t hc,
                       float mean, double mean64, uint32_t split_size, int flags,
                       uint32_t* records) {
    uint32_t K = (uint32_t)(((uint64_t)N + split_size - 1) / split_size);
    if (K == 0) K = 1;
    const uint32_t h = hc < N ? hc : N;
    for (uint32_t t = 0; t < K; ++t) {
        uint32_t ri = N - h, rj = h;
        float rs = 0.0f;
        if (t + 1 < K && hc != 0 && hc < N) {
            const uint32_t nk = (uint32_t)(((uint64_t)N * (t + 1) + K - 1) / K);
            wrso_split(prefix, prefix_lo, N, hc, mean, mean64, nk, flags, &ri, &rj, &rs);
        }
        records[3 * t + 0] = ri;
        records[3 * t + 1] = rj;
        memcpy(&records[3 * t + 2], &rs, 4);
    }
}

/* pack/scalar/float.comp:154-180 (ScalarPack, the pack half of SerialSplitPack): subproblem k in
 * [0, K) packs [split_k, split_{k+1}) with split_0 = (0, 0, 0) and split_k = record k - 1, by
 * the same loop as the inline shader (wrso_pack, float.comp:56-152 equals
 * splitpack/inline/shader.comp:130-223), subproblems in increasing k.  Where FP32 rounding
 * makes a split step back the shader's invocations write the same entries in no defined order;
 * here i1 = max(split_{k+1}.i, i0), j1 = max(split_{k+1}.j, j0) and the later k's write stands,
 * as for the inline split-pack.  Guard: heavyCount == 0 or N gives table[i] = (1, i). */
void wrso_scalar_pack(const float* w, const uint32_t* idx, const float* elems, uint32_t hc,
                      float mean, uint32_t N, uint32_t split_size, int flags,
                      const uint32_t* records, wrso_entry* table) {
    if (N == 0) return;
    if (hc == 0 || hc >= N) {
        for (uint32_t i = 0; i < N; ++i) {
            table[i].p = 1.0f;
            table[i].a = i;
        }
        return;
    }
    uint32_t K = (uint32_t)(((uint64_t)N + split_size - 1) / split_size);
    if (K == 0) K = 1;
    wrso_pack_ctx c = {w, idx, elems, N, hc, N - hc, mean, table,
                       (flags & WRSO_SPLIT_FULL_LIGHT) != 0};
    uint32_t pi = 0, pj = 0;
    float pspill = 0.0f;
    for (uint32_t k = 0; k < K; ++k) {
        const uint32_t ni = records[3 * k + 0], nj = records[3 * k + 1];
        float nspill;
        memcpy(&nspill, &records[3 * k + 2], 4);
        const uint32_t i1 = ni > pi ? ni : pi;
        const uint32_t j1 = nj > pj ? nj : pj;
        wrso_pack(&c, pi, i1, pj, j1, pspill);
        pi = ni;
        pj = nj;
        pspill = nspill;
    }
}

/* ---- threaded PSA build (timed CPU port) ---------------------------------- */

typedef struct {
    const float* w;
    uint32_t N;
    uint32_t split_size;
    int flags;
    float mean;
    double mean64;
    double* part_sum;
    uint32_t* part_heavy;
    double* part_hsum;
    double* part_lsum;
    uint32_t* idx;
    float* elems;
    float* prefix;
    float* prefix_lo; /* the FP64 prefix kept as a float-float pair (prefix = high word) */
    uint32_t hc;
    uint32_t K;
    wrso_entry* table;
} wrso_psa_ctx;

static void psa_sum_task(void* p, int t, int nt) {
    wrso_psa_ctx* c = (wrso_psa_ctx*)p;
    uint64_t lo, hi;
    wrso_range(c->N, t, nt, &lo, &hi);
    double s = 0.0;
    uint32_t h = 0;
    (void)h;
    for (uint64_t i = lo; i < hi; ++i) s += (double)c->w[i];
    c->part_sum[t] = s;
}

static void psa_count_task(void* p, int t, int nt) {
    wrso_psa_ctx* c = (wrso_psa_ctx*)p;
    uint64_t lo, hi;
    wrso_range(c->N, t, nt, &lo, &hi);
    uint32_t h = 0;
    double hs = 0.0, ls = 0.0;
    for (uint64_t i = lo; i < hi; ++i) {
        float x = c->w[i];
        if (x > c->mean) {
            ++h;
            hs += (double)x;
        } else {
            ls += (double)x;
        }
    }
    c->part_heavy[t] = h;
    c->part_hsum[t] = hs;
    c->part_lsum[t] = ls;
}

static void psa_scatter_task(void* p, int t, int nt) {
    wrso_psa_ctx* c = (wrso_psa_ctx*)p;
    uint64_t lo, hi;
    wrso_range(c->N, t, nt, &lo, &hi);
    uint32_t h = 0, l = 0;
    double hs = 0.0, ls = 0.0;
    for (int u = 0; u < t; ++u) {
        h += c->part_heavy[u];
        hs += c->part_hsum[u];
        ls += c->part_lsum[u];
    }
    l = (uint32_t)lo - h;
    const uint32_t N = c->N;
    for (uint64_t i = lo; i < hi; ++i) {
        float x = c->w[i];
        if (x > c->mean) {
            hs += (double)x;
            c->idx[h] = (uint32_t)i;
            c->elems[h] = x;
            c->prefix[h] = (float)hs;
            c->prefix_lo[h] = (float)(hs - (double)c->prefix[h]);
            ++h;
        } else {
            ls += (double)x;
            c->idx[N - 1 - l] = (uint32_t)i;
            c->elems[N - 1 - l] = x;
            c->prefix[N - 1 - l] = (float)ls;
            c->prefix_lo[N - 1 - l] = (float)(ls - (double)c->prefix[N - 1 - l]);
            ++l;
        }
    }
}

static void psa_splitpack_task(void* p, int t, int nt) {
    wrso_psa_ctx* c = (wrso_psa_ctx*)p;
    uint64_t lo, hi;
    wrso_range(c->K, t, nt, &lo, &hi);
    if (lo >= hi) return;
    wrso_pack_ctx pc = {c->w,    c->idx,  c->elems, c->N, c->hc, c->N - c->hc, c->mean,
                        c->table, (c->flags & WRSO_SPLIT_FULL_LIGHT) != 0};
    uint32_t pi, pj;
    float pspill;
    if (lo == 0) {
        pi = 0;
        pj = 0;
        pspill = 0.0f;
    } else {
        wrso_split(c->prefix, c->prefix_lo, c->N, c->hc, c->mean, c->mean64,
                   (uint32_t)lo * c->split_size, c->flags, &pi, &pj, &pspill);
    }
    for (uint64_t k = lo + 1; k <= hi; ++k) {
        uint32_t ni, nj;
        float nspill;
        if (k == c->K) {
            ni = c->N - c->hc;
            nj = c->hc;
            nspill = 0.0f;
        } else {
            wrso_split(c->prefix, c->prefix_lo, c->N, c->hc, c->mean, c->mean64,
                       (uint32_t)k * c->split_size, c->flags, &ni, &nj, &nspill);
        }
        uint32_t i1 = ni > pi ? ni : pi;
        uint32_t j1 = nj > pj ? nj : pj;
        wrso_pack(&pc, pi, i1, pj, j1, pspill);
        pi = ni;
        pj = nj;
        pspill = nspill;
    }
}

void wrso_psa_build(const float* w, uint32_t N, uint32_t split_size, int flags, int nthreads,
                    wrso_entry* table, float* mean_out, uint32_t* heavy_count_out) {
    if (nthreads < 1) nthreads = 1;
    wrso_psa_ctx c;
    memset(&c, 0, sizeof(c));
    c.w = w;
    c.N = N;
    c.split_size = split_size;
    c.flags = flags;
    c.table = table;
    c.part_sum = (double*)calloc((size_t)nthreads, sizeof(double));
    c.part_heavy = (uint32_t*)calloc((size_t)nthreads, sizeof(uint32_t));
    c.part_hsum = (double*)calloc((size_t)nthreads, sizeof(double));
    c.part_lsum = (double*)calloc((size_t)nthreads, sizeof(double));
    wrso_parallel(psa_sum_task, &c, nthreads);
    double total = 0.0;
    for (int t = 0; t < nthreads; ++t) total += c.part_sum[t];
    c.mean64 = N ? total / (double)N : 0.0;
    c.mean = (float)c.mean64;
    c.idx = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)N);
    c.elems = (float*)malloc(sizeof(float) * (size_t)N);
    c.prefix = (float*)malloc(sizeof(float) * (size_t)N);
    c.prefix_lo = (float*)malloc(sizeof(float) * (size_t)N);
    wrso_parallel(psa_count_task, &c, nthreads);
    uint32_t hc = 0;
    for (int t = 0; t < nthreads; ++t) hc += c.part_heavy[t];
    c.hc = hc;
    wrso_parallel(psa_scatter_task, &c, nthreads);
    if (!(flags & WRSO_SPLIT_FLOAT_FLOAT)) {
        free(c.prefix_lo);
        c.prefix_lo = NULL;
    }
    if (hc == 0 || hc == N) {
        for (uint32_t i = 0; i < N; ++i) {
            table[i].p = 1.0f;
            table[i].a = i;
        }
    } else {
        c.K = N / split_size;
        if (c.K == 0) c.K = 1;
        wrso_parallel(psa_splitpack_task, &c, nthreads);
    }
    if (mean_out) *mean_out = c.mean;
    if (heavy_count_out) *heavy_count_out = hc;
    free(c.idx);
    free(c.elems);
    free(c.prefix);
    free(c.prefix_lo);
    free(c.part_sum);
    free(c.part_heavy);
    free(c.part_hsum);
    free(c.part_lsum);
}

/* ------------------------------------------------------------------------- */
/* sampling                                                                  */
/* ------------------------------------------------------------------------- */

/* mix(x, y, a) restated as x*(1-a) + y*a with one rounding per operation. */
static inline float wrso_mix(float x, float y, float a) {
    volatile float oma = 1.0f - a;
    volatile float t0 = x * oma;
    volatile float t1 = y * a;
    return t0 + t1;
}

static inline uint32_t wrso_alias_one_ref(const wrso_entry* table, uint32_t N, uint32_t seed,
                                          uint32_t gid, int coop, int32_t sx, int32_t sy) {
    uint32_t r[2];
    wrso_philox2x32_7(0u, gid, seed, r);
    float ux = wrso_unit_ref(r[0]), uy = wrso_unit_ref(r[1]);
    float f = coop ? wrso_mix((float)sx, (float)sy, ux) : (float)N * ux;
    int32_t ix = (int32_t)f; /* int() truncates toward zero */
    if (ix < 0) ix = 0;
    if (ix > (int32_t)(N - 1)) ix = (int32_t)(N - 1);
    float p = table[ix].p;
    return uy >= p ? table[ix].a : (uint32_t)ix;
}

typedef struct {
    const wrso_entry* table;
    const float* cmf;
    uint32_t N;
    uint64_t S, seed, offset;
    uint32_t rng, coop;
    int parray;
    uint32_t* out;
} wrso_sample_ctx;

static void alias_task(void* p, int t, int nt) {
    wrso_sample_ctx* c = (wrso_sample_ctx*)p;
    /* chunks are multiples of 32 so that subgroups (warps) stay whole */
    uint64_t warps = (c->S + 31) / 32, lo, hi;
    wrso_range(warps, t, nt, &lo, &hi);
    const uint32_t N = c->N;
    const wrso_entry* table = c->table;
    for (uint64_t wi = lo; wi < hi; ++wi) {
        uint64_t s0 = wi * 32, s1 = s0 + 32;
        if (s1 > c->S) s1 = c->S;
        if (c->rng == WRSO_RNG_REFERENCE) {
            const uint32_t seed = (uint32_t)c->seed;
            int32_t sx = 0, sy = (int32_t)N;
            if (c->coop) {
                /* narrowSection (shader.comp:68-76): the elected lane is the warp's first
                 * sample; section = ix -/+ coop/2 */
                uint32_t g0 = (uint32_t)(c->offset + s0);
                uint32_t r[2];
                wrso_philox2x32_7(0u, g0, seed, r);
                float ux = wrso_unit_ref(r[0]);
                int32_t ix = (int32_t)((float)N * ux);
                sx = ix - (int32_t)c->coop / 2;
                sy = ix + (int32_t)c->coop / 2;
            }
            for (uint64_t s = s0; s < s1; ++s)
                c->out[s] = wrso_alias_one_ref(table, N, seed, (uint32_t)(c->offset + s),
                                               c->coop != 0, sx, sy);
        } else {
            const uint32_t key[2] = {(uint32_t)c->seed, (uint32_t)(c->seed >> 32)};
            for (uint64_t s = s0; s < s1; ++s) {
                uint64_t g = c->offset + s;
                uint32_t ctr[4] = {(uint32_t)g, (uint32_t)(g >> 32), 0u, 0u}, r[4];
                wrso_philox4x32_10(ctr, key, r);
                uint32_t ix = (uint32_t)(((uint64_t)r[0] * (uint64_t)N) >> 32);
                /* keep ix when p >= 1 or x1 < ceil(p * 2^32) (32-bit coin) */
                float p = table[ix].p;
                int keep = p >= 1.0f;
                if (!keep && p > 0.0f) keep = (double)r[1] < ceil((double)p * 4294967296.0);
                c->out[s] = keep ? ix : table[ix].a;
            }
        }
    }
}

void wrso_alias_sample(const wrso_entry* table, uint32_t N, uint64_t S, uint64_t seed,
                       uint64_t offset, uint32_t rng, uint32_t coop, int nthreads, uint32_t* out) {
    wrso_sample_ctx c = {table, NULL, N, S, seed, offset, rng, coop, 0, out};
    wrso_parallel(alias_task, &c, nthreads < 1 ? 1 : nthreads);
}

/* its/sampling/shader.comp:80-94: lowCmf + (highCmf - lowCmf) * u, one rounding per op */
static inline float wrso_search_range_u(const float* cmf, uint32_t x, uint32_t y, float u) {
    float lowCmf = x > 0 ? cmf[x - 1] : 0.0f;
    float highCmf = cmf[y];
    volatile float d = highCmf - lowCmf;
    volatile float m = d * u;
    return lowCmf + m;
}

/* its/sampling/shader.comp:131-140: lower bound with the shader's probe sequence */
static inline uint32_t wrso_bisect(const float* cmf, uint32_t x, uint32_t y, float u) {
    while (x < y) {
        uint32_t mid = (uint32_t)(((uint64_t)x + y) / 2);
        if (u > cmf[mid])
            x = mid + 1;
        else
            y = mid;
    }
    return x;
}

/* Philox ITS: first index with cmf >= T for the exact target T = (2 x0 + 1) * total * 2^-33,
 * bisecting like its/sampling/shader.comp:131-140.  T has at most 57 significant bits and
 * is held exactly in long double (64-bit significand on x86-64, 113-bit on aarch64). */
_Static_assert(LDBL_MANT_DIG >= 57, "the exact ITS target needs a >= 57-bit long double");
static uint32_t wrso_bisect_exact(const float* cmf, uint32_t last, long double T) {
    uint32_t x = 0, y = last;
    while (x < y) {
        uint32_t mid = (uint32_t)(((uint64_t)x + y) / 2);
        if (T > (long double)cmf[mid])
            x = mid + 1;
        else
            y = mid;
    }
    return x;
}

static void its_task(void* p, int t, int nt) {
    wrso_sample_ctx* c = (wrso_sample_ctx*)p;
    uint64_t warps = (c->S + 31) / 32, lo, hi;
    wrso_range(warps, t, nt, &lo, &hi);
    const uint32_t N = c->N;
    const float* cmf = c->cmf;
    for (uint64_t wi = lo; wi < hi; ++wi) {
        uint64_t s0 = wi * 32, s1 = s0 + 32;
        if (s1 > c->S) s1 = c->S;
        if (c->rng == WRSO_RNG_REFERENCE) {
            const uint32_t seed = (uint32_t)c->seed;
            uint32_t x = 0, y = N - 1;
            if (c->coop) {
                /* the elected lane (warp's first sample) draws u1 with the plain seed */
                uint32_t g0 = (uint32_t)(c->offset + s0);
                float u1 = wrso_search_range_u(cmf, 0, N - 1, wrso_unit_ref(wrso_wang_hash(seed + g0)));
                if (c->parray) {
                    /* pArrayNarrow (shader.comp:111-129); when no lane's partition end
                     * exceeds u1 (the shader's ballot is empty, undefined there) the
                     * remainder past the 32 partitions is kept, at least the last item */
                    uint32_t range = y - x + 1;
                    while (range > c->coop) {
                        uint32_t base = range / 32;
                        int found = 0;
                        for (uint32_t lane = 0; lane < 32; ++lane) {
                            uint32_t start = x + lane * base;
                            uint32_t end = start + base - 1;
                            if (end > y) end = y;
                            if (u1 < cmf[end]) {
                                x = start;
                                y = end;
                                found = 1;
                                break;
                            }
                        }
                        if (!found) x = (x + 32 * base < y) ? x + 32 * base : y;
                        range = y - x + 1;
                    }
                } else {
                    /* binaryNarrow (shader.comp:100-109) */
                    while (y - x + 1 > c->coop) {
                        uint32_t mid = (uint32_t)(((uint64_t)x + y) / 2);
                        if (u1 > cmf[mid])
                            x = mid + 1;
                        else
                            y = mid;
                    }
                }
            }
            const uint32_t seed2 = seed ^ 0xA9EC5C80u;
            for (uint64_t s = s0; s < s1; ++s) {
                uint32_t g = (uint32_t)(c->offset + s);
                float u2 = wrso_search_range_u(cmf, x, y, wrso_unit_ref(wrso_wang_hash(seed2 + g)));
                c->out[s] = wrso_bisect(cmf, x, y, u2);
            }
        } else {
            const uint32_t key[2] = {(uint32_t)c->seed, (uint32_t)(c->seed >> 32)};
            const float total = cmf[N - 1];
            for (uint64_t s = s0; s < s1; ++s) {
                uint64_t g = c->offset + s;
                uint32_t ctr[4] = {(uint32_t)g, (uint32_t)(g >> 32), 0u, 0u}, r[4];
                wrso_philox4x32_10(ctr, key, r);
                c->out[s] = wrso_bisect_exact(cmf, N - 1, (2.0L * r[0] + 1.0L) * total / 8589934592.0L);
            }
        }
    }
}

void wrso_its_sample(const float* cmf, uint32_t N, uint64_t S, uint64_t seed, uint64_t offset,
                     uint32_t rng, uint32_t coop, int parray, int nthreads, uint32_t* out) {
    wrso_sample_ctx c = {NULL, cmf, N, S, seed, offset, rng, coop, parray, out};
    wrso_parallel(its_task, &c, nthreads < 1 ? 1 : nthreads);
}

/* ------------------------------------------------------------------------- */
/* Cutpoint                                                                  */
/* ------------------------------------------------------------------------- */

/* cutpoint/guiding_table/shader.comp:40-55: guide[k] = lower bound of u_k = step * k with
 * step = cmf[N-1] / G, over the whole CMF with the shader's probe sequence. */
void wrso_cutpoint_guide(const float* cmf, uint32_t N, uint32_t G, uint32_t* guide) {
    const float total = cmf[N - 1];
    volatile float step = total / (float)G;
    for (uint32_t k = 0; k < G; ++k) {
        volatile float u = step * (float)k;
        guide[k] = wrso_bisect(cmf, 0, N - 1, u);
    }
}

typedef struct {
    const float* cmf;
    const uint32_t* guide;
    uint32_t N, G;
    uint64_t S, seed, offset;
    uint32_t rng;
    uint32_t* out;
} wrso_cutpoint_ctx;

/* cutpoint/sampling/shader.comp:100-140: the subgroup's elected lane (first sample of the
 * aligned group of 32) draws u1 = wang_hash(seed + g0) and picks cell min(u1 * G, G - 1);
 * each sample draws u2 = wang_hash((seed ^ 0x079145147) + g) inside the cell's CMF range
 * [cmf[guide[k] - 1], cmf[guide[k+1]]] and bisects [guide[k], guide[k+1]] (N - 1 for the last
 * cell).  Philox4x32-10 mode: u1 = x0 of the group's first sample, u2 = x1 of the sample. */
static void cutpoint_task(void* p, int t, int nt) {
    wrso_cutpoint_ctx* c = (wrso_cutpoint_ctx*)p;
    uint64_t warps = (c->S + 31) / 32, lo, hi;
    wrso_range(warps, t, nt, &lo, &hi);
    const uint32_t seed32 = (uint32_t)c->seed;
    const uint32_t key[2] = {(uint32_t)c->seed, (uint32_t)(c->seed >> 32)};
    for (uint64_t wi = lo; wi < hi; ++wi) {
        uint64_t s0 = wi * 32, s1 = s0 + 32;
        if (s1 > c->S) s1 = c->S;
        const uint64_t g0 = c->offset + s0;
        float u1;
        if (c->rng == WRSO_RNG_REFERENCE) {
            u1 = wrso_unit_ref(wrso_wang_hash(seed32 + (uint32_t)g0));
        } else {
            uint32_t ctr[4] = {(uint32_t)g0, (uint32_t)(g0 >> 32), 0u, 0u}, r[4];
            wrso_philox4x32_10(ctr, key, r);
            u1 = wrso_unit_ref(r[0]);
        }
        volatile float prod = u1 * (float)c->G;
        uint32_t k = (uint32_t)prod;
        if (k > c->G - 1) k = c->G - 1;
        const uint32_t x = c->guide[k];
        const uint32_t y = k != c->G - 1 ? c->guide[k + 1] : c->N - 1;
        for (uint64_t s = s0; s < s1; ++s) {
            const uint64_t g = c->offset + s;
            float uu;
            if (c->rng == WRSO_RNG_REFERENCE) {
                uu = wrso_unit_ref(wrso_wang_hash((seed32 ^ 0x79145147u) + (uint32_t)g));
            } else {
                uint32_t ctr[4] = {(uint32_t)g, (uint32_t)(g >> 32), 0u, 0u}, r[4];
                wrso_philox4x32_10(ctr, key, r);
                uu = wrso_unit_ref(r[1]);
            }
            c->out[s] = wrso_bisect(c->cmf, x, y, wrso_search_range_u(c->cmf, x, y, uu));
        }
    }
}

void wrso_cutpoint_sample(const float* cmf, uint32_t N, const uint32_t* guide, uint32_t G,
                          uint64_t S, uint64_t seed, uint64_t offset, uint32_t rng, int nthreads,
                          uint32_t* out) {
    wrso_cutpoint_ctx c = {cmf, guide, N, G, S, seed, offset, rng, out};
    wrso_parallel(cutpoint_task, &c, nthreads < 1 ? 1 : nthreads);
}

/* ------------------------------------------------------------------------- */
/* statistics                                                                */
/* ------------------------------------------------------------------------- */

void wrso_histogram(const uint32_t* samples, uint64_t S, uint32_t N, uint64_t* hist) {
    memset(hist, 0, sizeof(uint64_t) * (size_t)N);
    for (uint64_t s = 0; s < S; ++s)
        if (samples[s] < N) hist[samples[s]] += 1;
}

/* chi_square.hpp:17-37, evaluated in FP64 with Kahan summation.  Zero-weight bins
 * contribute nothing when empty (their expected count is 0). */
double wrso_chi_square(const uint64_t* hist, const float* w, uint32_t N, uint64_t S) {
    double W = wrso_total_mass(w, N);
    double sum = 0.0, c = 0.0;
    for (uint32_t i = 0; i < N; ++i) {
        double e = ((double)w[i] * (double)S) / W;
        if (e <= 0.0) continue;
        double o = (double)hist[i];
        double el = ((o - e) * (o - e)) / e;
        double y = el - c;
        double t = sum + y;
        c = (t - sum) - y;
        sum = t;
    }
    return sum;
}

/* Adjacent bins (in index order) are merged until each expected count reaches
 * min_expected, so that the chi-square approximation holds for large N. */
double wrso_chi_square_binned(const uint64_t* hist, const float* w, uint32_t N, uint64_t S,
                              double min_expected, uint64_t* bins_out) {
    double W = wrso_total_mass(w, N);
    double sum = 0.0, eacc = 0.0, oacc = 0.0;
    uint64_t bins = 0;
    for (uint32_t i = 0; i < N; ++i) {
        eacc += ((double)w[i] * (double)S) / W;
        oacc += (double)hist[i];
        if (eacc >= min_expected) {
            sum += (oacc - eacc) * (oacc - eacc) / eacc;
            ++bins;
            eacc = 0.0;
            oacc = 0.0;
        }
    }
    if (eacc > 0.0) {
        sum += (oacc - eacc) * (oacc - eacc) / eacc;
        ++bins;
    }
    if (bins_out) *bins_out = bins;
    return sum;
}

/* Regularised upper incomplete gamma Q(a, x): power series for x < a + 1,
 * Lentz continued fraction otherwise (Press et al., Numerical Recipes 6.2). */
static double wrso_gamma_q(double a, double x) {
    if (x <= 0.0) return 1.0;
    const double lpre = -x + a * log(x) - lgamma(a);
    if (x < a + 1.0) {
        double ap = a, del = 1.0 / a, sum = del;
        for (int n = 0; n < 10000000; ++n) {
            ap += 1.0;
            del *= x / ap;
            sum += del;
            if (fabs(del) < fabs(sum) * 1e-16) break;
        }
        double P = sum * exp(lpre);
        return P >= 1.0 ? 0.0 : 1.0 - P;
    }
    const double tiny = 1e-300;
    double b = x + 1.0 - a, cc = 1.0 / tiny, d = 1.0 / b, h = d;
    for (int i = 1; i < 10000000; ++i) {
        double an = -(double)i * ((double)i - a);
        b += 2.0;
        d = an * d + b;
        if (fabs(d) < tiny) d = tiny;
        cc = b + an / cc;
        if (fabs(cc) < tiny) cc = tiny;
        d = 1.0 / d;
        double del = d * cc;
        h *= del;
        if (fabs(del - 1.0) < 1e-16) break;
    }
    return exp(lpre) * h;
}

double wrso_chi2_sf(double x, double df) { return wrso_gamma_q(0.5 * df, 0.5 * x); }

/* src/dep/eval/rms.hpp:44-63: sqrt(mean_i (w_i/W - h_i/S)^2) with Kahan summation */
double wrso_rmse(const uint64_t* hist, const float* w, uint32_t N, uint64_t S) {
    double W = wrso_total_mass(w, N);
    double sum = 0.0, c = 0.0;
    for (uint32_t i = 0; i < N; ++i) {
        double d = (double)w[i] / W - (double)hist[i] / (double)S;
        double y = d * d - c;
        double t = sum + y;
        c = (t - sum) - y;
        sum = t;
    }
    return sqrt(sum / (double)N);
}

/* js_divergence.hpp:48-92 in FP64 */
double wrso_js_divergence(const uint64_t* hist, const float* w, uint32_t N, uint64_t S) {
    double W = wrso_total_mass(w, N);
    double kl1 = 0.0, kl2 = 0.0;
    for (uint32_t i = 0; i < N; ++i) {
        double o = (double)hist[i] / (double)S, e = (double)w[i] / W, m = 0.5 * (o + e);
        if (o > 0.0 && m > 0.0) kl1 += o * log(o / m);
        if (e > 0.0 && m > 0.0) kl2 += e * log(e / m);
    }
    return 0.5 * (kl1 + kl2);
}

/* inverse_alias_table.hpp:15-30: p clamped to [0,1]; entry i keeps p, its alias gets 1-p */
void wrso_alias_to_weights(const wrso_entry* table, uint32_t N, double* out) {
    memset(out, 0, sizeof(double) * (size_t)N);
    for (uint32_t i = 0; i < N; ++i) {
        double p = table[i].p;
        if (p < 0.0) p = 0.0;
        if (p > 1.0) p = 1.0;
        out[i] += p;
        if (table[i].a < N) out[table[i].a] += 1.0 - p;
    }
}

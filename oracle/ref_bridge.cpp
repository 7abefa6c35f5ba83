// ref_bridge.cpp -- exposes the reference's own CPU code through a C ABI.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the reference's
// header-only host code where it lies (REF=<reference checkout>), into
// oracle/_ref/libwrs_ref.so.  It pins the oracle restatement (wrs_oracle.c) and
// generates the golden fixtures under tests/golden/.  Nothing here is product
// code and the reference sources are not copied: this file only instantiates and
// calls the reference's templates:
//   host::generate_weights           src/host/gen/weight_generator.h:32-155
//   reference::psa_alias_table       src/host/reference/psa_alias_table.hpp:23-67
//   reference::prefix_sum            src/host/reference/prefix_sum.hpp:17-34
//   reference::kahan_reduction       src/host/reference/reduce.hpp:81-92
//   reference::stable_partition_indicies  src/host/reference/partition.hpp:37-52
//   reference::split / splitK        src/host/reference/split.hpp:15-85
//   reference::packSplits            src/host/reference/pack.hpp:183-200
//   reference::alias_table_to_normalized_weights  src/host/reference/inverse_alias_table.hpp:15
//   test::assert_is_alias_table      src/host/assert/is_alias_table.hpp:109-195
//   test::assert_is_inclusive_prefix src/host/assert/is_prefix.hpp:102-223
//   test::assert_is_split            src/host/assert/is_split.hpp:134-300
//   host::chi_square                 src/host/statistics/chi_square.hpp:17-37
//   host::js_divergence              src/host/statistics/js_divergence.hpp:48-92
//   alias_table_internals::sample_single  src/host/reference/sample_alias_table.hpp:16-25
// is_prefix.hpp uses std::setprecision without including <iomanip>
#include <iomanip>

#include "src/host/assert/is_alias_table.hpp"
#include "src/host/assert/is_prefix.hpp"
#include "src/host/assert/is_split.hpp"
#include "src/host/gen/weight_generator.h"
#include "src/host/reference/inverse_alias_table.hpp"
#include "src/host/reference/pack.hpp"
#include "src/host/reference/partition.hpp"
#include "src/host/reference/prefix_sum.hpp"
#include "src/host/reference/psa_alias_table.hpp"
#include "src/host/reference/reduce.hpp"
#include "src/host/reference/sample_alias_table.hpp"
#include "src/host/reference/split.hpp"
#include "src/host/statistics/chi_square.hpp"
#include "src/host/statistics/js_divergence.hpp"

#include <cstdint>
#include <cstring>
#include <span>
#include <vector>

using u32 = std::uint32_t;
using u64 = std::uint64_t;

extern "C" {

// dist: 0 = UNIFORM (all 1.0), 1 = PSEUDO_RANDOM_UNIFORM (fixed-seed mt19937, U[0.01,1))
int ref_generate_weights(int dist, u32 count, float* out) {
    host::Distribution d;
    if (dist == 0)
        d = host::Distribution::UNIFORM;
    else if (dist == 1)
        d = host::Distribution::PSEUDO_RANDOM_UNIFORM;
    else
        return 1;
    auto w = host::generate_weights<float>(d, count);
    std::memcpy(out, w.data(), sizeof(float) * count);
    return 0;
}

void ref_psa_alias_table(const float* w, u32 N, u32 K, float* p, u32* a) {
    auto table = host::reference::pmr::psa_alias_table<float, float, u32>(
        std::span<const float>(w, N), K);
    for (u32 i = 0; i < N; ++i) {
        p[i] = table[i].p;
        a[i] = table[i].a;
    }
}

void ref_prefix_sum(const float* w, u64 N, float* out) {
    auto pre = host::reference::prefix_sum<float>(std::span<const float>(w, N));
    std::memcpy(out, pre.data(), sizeof(float) * N);
}

float ref_kahan_reduction(const float* w, u64 N) {
    return host::reference::kahan_reduction<float>(std::span<const float>(w, N));
}

void ref_stable_partition_indices(const float* w, u32 N, float pivot, u32* out, u32* heavy_count) {
    auto part = host::reference::stable_partition_indicies<float, u32>(
        std::span<const float>(w, N), pivot);
    auto h = part.heavy();
    auto l = part.light();
    std::memcpy(out, h.data(), sizeof(u32) * h.size());
    std::memcpy(out + h.size(), l.data(), sizeof(u32) * l.size());
    *heavy_count = static_cast<u32>(h.size());
}

void ref_split(const float* heavy_prefix, u32 hc, const float* light_prefix, u32 lc, float mean,
               u32 n, u32* i, u32* j, float* spill) {
    auto s = host::reference::split<float, u32>(std::span<const float>(heavy_prefix, hc),
                                                std::span<const float>(light_prefix, lc), mean, n);
    *i = s.i;
    *j = s.j;
    *spill = s.spill;
}

void ref_splitK(const float* heavy_prefix, u32 hc, const float* light_prefix, u32 lc, float mean,
                u32 N, u32 K, u32* i, u32* j, float* spill) {
    auto s = host::reference::splitK<float, u32>(std::span<const float>(heavy_prefix, hc),
                                                 std::span<const float>(light_prefix, lc), mean, N,
                                                 K);
    for (u32 k = 0; k < K; ++k) {
        i[k] = s[k].i;
        j[k] = s[k].j;
        spill[k] = s[k].spill;
    }
}

void ref_pack_splits(const u32* heavy_idx, u32 hc, const u32* light_idx, u32 lc, const float* w,
                     u32 N, float mean, const u32* si, const u32* sj, const float* sspill, u32 K,
                     float* p, u32* a) {
    std::vector<host::Split<float, u32>> splits(K);
    for (u32 k = 0; k < K; ++k) splits[k] = host::Split<float, u32>(si[k], sj[k], sspill[k]);
    auto table = host::reference::packSplits<float, float, u32,
                                             std::allocator<host::AliasTableEntry<float, u32>>>(
        std::span<const u32>(heavy_idx, hc), std::span<const u32>(light_idx, lc),
        std::span<const float>(w, N), mean, std::span<const host::Split<float, u32>>(splits));
    for (u32 x = 0; x < N; ++x) {
        p[x] = table[x].p;
        a[x] = table[x].a;
    }
}

void ref_alias_to_normalized_weights(const float* p, const u32* a, u32 N, float* out) {
    std::vector<host::AliasTableEntry<float, u32>> table(N);
    for (u32 i = 0; i < N; ++i) table[i] = host::AliasTableEntry<float, u32>(p[i], a[i]);
    auto wts = host::reference::alias_table_to_normalized_weights<float, u32>(table);
    std::memcpy(out, wts.data(), sizeof(float) * N);
}

// Returns the aggregated IsAliasTableErrorType bits; *error_count = number of bad entries.
int ref_assert_is_alias_table(const float* w, u32 N, const float* p, const u32* a,
                              float total_weight, float margin, u64* error_count) {
    std::vector<host::AliasTableEntry<float, u32>> table(N);
    for (u32 i = 0; i < N; ++i) table[i] = host::AliasTableEntry<float, u32>(p[i], a[i]);
    auto err = host::test::pmr::assert_is_alias_table<float, float, u32>(
        std::span<const float>(w, N),
        std::span<const host::AliasTableEntry<float, u32>>(table.data(), N), total_weight,
        margin);
    *error_count = err.errors.size();
    return static_cast<int>(err.type);
}

int ref_assert_is_inclusive_prefix(const float* elements, const float* prefix, u64 N,
                                   u64* error_count) {
    auto err = host::test::pmr::assert_is_inclusive_prefix<float>(std::span<const float>(elements, N),
                                                             std::span<const float>(prefix, N));
    *error_count = err.errors.size();
    return static_cast<int>(err.errorTypes);
}

int ref_assert_is_split(const u32* si, const u32* sj, const float* sspill, u32 K,
                        const float* heavy_prefix, u32 hc, const float* light_prefix, u32 lc,
                        float mean, float margin, u64* error_count) {
    std::vector<host::Split<float, u32>> splits(K);
    for (u32 k = 0; k < K; ++k) splits[k] = host::Split<float, u32>(si[k], sj[k], sspill[k]);
    auto err = host::test::pmr::assert_is_split<float, u32>(
        std::span<const host::Split<float, u32>>(splits), K,
        std::span<const float>(heavy_prefix, hc), std::span<const float>(light_prefix, lc), mean,
        margin);
    *error_count = err.errors.size();
    return static_cast<int>(err.type);
}

float ref_chi_square(const u32* samples, u64 S, const float* w, u32 N) {
    return host::chi_square<u32, float>(std::span<const u32>(samples, S),
                                        std::span<const float>(w, N));
}

float ref_js_divergence(const u32* samples, u64 S, const float* w, u32 N) {
    return host::js_divergence<u32, float>(std::span<const u32>(samples, S),
                                           std::span<const float>(w, N));
}

u32 ref_sample_single(const float* p, const u32* a, u32 N, u32 u1, float u2) {
    std::vector<host::AliasTableEntry<float, u32>> table(N);
    for (u32 i = 0; i < N; ++i) table[i] = host::AliasTableEntry<float, u32>(p[i], a[i]);
    return host::reference::alias_table_internals::sample_single<float, u32>(
        std::span<const host::AliasTableEntry<float, u32>>(table.data(), N), u1, u2);
}

} // extern "C"

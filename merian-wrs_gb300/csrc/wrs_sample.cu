// wrs_sample.cu -- sampling kernels of the WRS hot path for sm_103a.
//
//   k_alias_sample  alias-table sampling      (reference: src/device/wrs/alias/sampling/shader.comp:68-111)
//   k_its_sample    inverse transform sampling by bisection over the CMF
//                                             (reference: src/device/wrs/its/sampling/shader.comp:80-177)
//
// Two generator modes:
//   RNG_REF      the shaders' own streams: Philox2x32-7 variant with counter (0, gid) and
//                key = seed for the alias method; wang_hash(seed + gid) for ITS.  Indices
//                are bit-exact with the shaders' arithmetic.
//   RNG_PHILOX   Random123 Philox4x32-10, key = (seed lo, seed hi), counter = (sample
//                index lo, hi, 0, 0).  Alias: ix = mulhi(x0, N); the bucket keeps ix when
//                p >= 1 or x1 < ceil(p * 2^32), else returns its alias (32-bit coin).
//                ITS: target T = (2*x0 + 1) * cmf[N-1] * 2^-33 in (0, total), formed
//                exactly in 64-bit integers and kept as its FP32 rounding plus the sign of
//                the rounding residual, so every probe "T > cmf[mid]" is decided exactly
//                with one FP32 compare; result = first index with cmf >= T.  Zero-weight
//                items can never be drawn.
#include "wrs_device.cuh"
#include "wrs_internal.cuh"

namespace wrs {

constexpr uint32_t RNG_REF = 0, RNG_PHILOX = 1;

// mix(x, y, a) evaluated as x*(1-a) + y*a, one rounding per operation
__device__ __forceinline__ float mix_rn(float x, float y, float a) {
    return __fadd_rn(__fmul_rn(x, __fsub_rn(1.0f, a)), __fmul_rn(y, a));
}

// The coin filter of a table: per bucket one byte q = floor(256 p) (255 for p >= 1, 0 for
// p <= 0 or NaN), a lower bound of the bucket's keep threshold in both generator modes: a
// coin below it (x1 < q * 2^24, or u < q / 256 for the shader's float coin) keeps the bucket
// whatever its entry holds.  The sampler then reads the 8-byte entry only for the other
// samples -- 1 - mean(q) / 256 of them: 0.42 for uniform weights, whose PSA buckets keep 58 %
// of their draws -- while the filter (N bytes: 64 MB at N = 2^26) stays in L2 and the table
// does not.
// Every decision is the unfiltered one, so the samples are identical.
__device__ __forceinline__ uint32_t coin_code(uint32_t pbits) {
    const float p = __uint_as_float(pbits);
    if (!(p > 0.0f)) return 0u;
    if (p >= 1.0f) return 255u;
    return static_cast<uint32_t>(__fmul_rn(p, 256.0f));  // exact product; truncation = floor
}

// Samples [block * 1024 + 4t, +4) of one distribution (thread t of the CTA).  FILTER: coins is
// the table's coin filter, read where `use` holds.
template <uint32_t RNG, bool COOP, bool FILTER>
__device__ __forceinline__ void alias_block(const uint2* __restrict__ table,
                                            const uint8_t* __restrict__ coins, bool use,
                                            uint32_t n, uint64_t S, uint64_t seed,
                                            uint64_t offset, uint32_t coop,
                                            uint32_t* __restrict__ out, uint64_t block) {
    const uint64_t t = block * kSampleThreads + threadIdx.x;
    const uint64_t s0 = t * kAliasPerThread;
    if (s0 >= S) return;
    uint32_t r[kAliasPerThread];
    uint64_t pol = 0;
    if constexpr (FILTER) pol = l2_policy_evict_first();  // table entries: keep the filter in L2
    if constexpr (RNG == RNG_REF) {
        const uint32_t key = static_cast<uint32_t>(seed);
        const float fn = __uint2float_rn(n);
        float sx = 0.f, sy = 0.f;
        if constexpr (COOP) {
            // narrowSection (shader.comp:68-76): the subgroup's elected lane is the first
            // sample of its aligned group of 32; section = ix -/+ coop/2
            const uint32_t g0 = static_cast<uint32_t>(offset + (s0 & ~31ull));
            const uint2 u = philox2x32_7(0u, g0, key);
            const int ix = __float2int_rz(__fmul_rn(fn, unit_ref(u.x)));
            sx = __int2float_rn(ix - static_cast<int>(coop) / 2);
            sy = __int2float_rn(ix + static_cast<int>(coop) / 2);
        }
        uint2 ent[kAliasPerThread];
        int ixs[kAliasPerThread];
        float uys[kAliasPerThread];
#pragma unroll
        for (int v = 0; v < kAliasPerThread; ++v) {
            const uint32_t g = static_cast<uint32_t>(offset + s0 + v);
            const uint2 u = philox2x32_7(0u, g, key);
            const float ux = unit_ref(u.x);
            uys[v] = unit_ref(u.y);
            const float f = COOP ? mix_rn(sx, sy, ux) : __fmul_rn(fn, ux);
            int ix = __float2int_rz(f);
            ix = ix < 0 ? 0 : ix;
            ix = ix > static_cast<int>(n - 1u) ? static_cast<int>(n - 1u) : ix;
            ixs[v] = ix;
        }
        if constexpr (FILTER) {
            bool need[kAliasPerThread];
#pragma unroll
            for (int v = 0; v < kAliasPerThread; ++v) need[v] = true;
            if (use) {
#pragma unroll
                for (int v = 0; v < kAliasPerThread; ++v)
                    need[v] = !(uys[v] <
                                __fmul_rn(__uint2float_rn(__ldg(coins + ixs[v])), 0.00390625f));
            }
#pragma unroll
            for (int v = 0; v < kAliasPerThread; ++v)
                ent[v] = need[v] ? ld_entry_policy(table + ixs[v], pol) : make_uint2(0u, 0u);
#pragma unroll
            for (int v = 0; v < kAliasPerThread; ++v)
                r[v] = need[v] && uys[v] >= __uint_as_float(ent[v].x) ? ent[v].y
                                                                      : static_cast<uint32_t>(ixs[v]);
        } else {
#pragma unroll
            for (int v = 0; v < kAliasPerThread; ++v) ent[v] = ld_entry(table + ixs[v]);
#pragma unroll
            for (int v = 0; v < kAliasPerThread; ++v)
                r[v] = uys[v] >= __uint_as_float(ent[v].x) ? ent[v].y : static_cast<uint32_t>(ixs[v]);
        }
    } else {
        uint2 ks[10];
        philox4x32_10_keys(seed, ks);
        uint2 ent[kAliasPerThread];
        uint32_t ixs[kAliasPerThread];
        uint32_t coin[kAliasPerThread];
#pragma unroll
        for (int v = 0; v < kAliasPerThread; ++v) {
            const uint64_t g = offset + s0 + v;
            const uint4 x = philox4x32_10(
                make_uint4(static_cast<uint32_t>(g), static_cast<uint32_t>(g >> 32), 0u, 0u), ks);
            ixs[v] = __umulhi(x.x, n);
            coin[v] = x.y;
        }
        bool need[kAliasPerThread];
#pragma unroll
        for (int v = 0; v < kAliasPerThread; ++v) need[v] = true;
        if (FILTER && use) {
#pragma unroll
            for (int v = 0; v < kAliasPerThread; ++v)
                need[v] = coin[v] >= (static_cast<uint32_t>(__ldg(coins + ixs[v])) << 24);
        }
#pragma unroll
        for (int v = 0; v < kAliasPerThread; ++v) {
            if constexpr (FILTER)
                ent[v] = need[v] ? ld_entry_policy(table + ixs[v], pol) : make_uint2(0u, 0u);
            else
                ent[v] = ld_entry(table + ixs[v]);
        }
#pragma unroll
        for (int v = 0; v < kAliasPerThread; ++v) {
            const float p = __uint_as_float(ent[v].x);
            const bool keep = !need[v] || p >= 1.0f ||
                              coin[v] < __float2uint_ru(__fmul_rn(p, 4294967296.0f));
            r[v] = keep ? ixs[v] : ent[v].y;
        }
    }
    if (s0 + kAliasPerThread <= S && (reinterpret_cast<uintptr_t>(out) & 15u) == 0) {
        __stcs(reinterpret_cast<uint4*>(out + s0), make_uint4(r[0], r[1], r[2], r[3]));
    } else {
#pragma unroll
        for (int v = 0; v < kAliasPerThread; ++v)
            if (s0 + v < S) out[s0 + v] = r[v];
    }
}

template <uint32_t RNG, bool COOP, bool FILTER>
__global__ __launch_bounds__(kSampleThreads) void k_alias_sample(
    const uint2* __restrict__ table, const uint8_t* __restrict__ coins,
    const unsigned long long* __restrict__ coin_sum, uint32_t n, uint64_t S, uint64_t seed,
    uint64_t offset, uint32_t coop, uint32_t* __restrict__ out) {
    pdl_entry();
    bool use = false;
    if constexpr (FILTER) use = __ldg(coin_sum) >= kCoinMinMean * n;
    alias_block<RNG, COOP, FILTER>(table, coins, use, n, S, seed, offset, coop, out, blockIdx.x);
}

// All distributions of a batch in one launch: CTA b samples block b - sample0 of the
// distribution the map names, with that distribution's seed and counter = sample index,
// so each distribution draws exactly the samples a per-call wrs_sample would.
template <uint32_t RNG, bool COOP>
__global__ __launch_bounds__(kSampleThreads) void k_alias_sample_batch(BatchView bv,
                                                                       uint32_t coop) {
    pdl_entry();
    const uint32_t d = __ldg(bv.sample_map + blockIdx.x);
    const DistDesc* D = bv.dist + d;
    alias_block<RNG, COOP, false>(D->table, nullptr, false, D->n, D->s, D->seed, 0ull, coop,
                                  D->out, blockIdx.x - D->sample0);
}

// The coin filter of table[0, n) (coin_code per entry, four entries per thread per step of a
// grid-striding loop) and the sum of its codes, added into *coin_sum once per CTA.
__global__ __launch_bounds__(kSampleThreads) void k_coin_filter(const uint2* __restrict__ table,
                                                                uint32_t n,
                                                                uint8_t* __restrict__ coins,
                                                                unsigned long long* coin_sum) {
    pdl_entry();
    __shared__ unsigned long long s_sum[kSampleThreads / 32];
    const uint64_t groups = (static_cast<uint64_t>(n) + 3u) / 4u;
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kSampleThreads;
    unsigned long long sum = 0;
    for (uint64_t t = static_cast<uint64_t>(blockIdx.x) * kSampleThreads + threadIdx.x;
         t < groups; t += stride) {
        const uint64_t e0 = 4ull * t;
        if (e0 + 4u <= n) {
            const uint4 a = __ldcs(reinterpret_cast<const uint4*>(table + e0));
            const uint4 b = __ldcs(reinterpret_cast<const uint4*>(table + e0 + 2u));
            const uint32_t c0 = coin_code(a.x), c1 = coin_code(a.z), c2 = coin_code(b.x),
                           c3 = coin_code(b.z);
            reinterpret_cast<uint32_t*>(coins)[t] = c0 | c1 << 8 | c2 << 16 | c3 << 24;
            sum += c0 + c1 + c2 + c3;
        } else {
            for (uint64_t e = e0; e < n; ++e) {
                const uint32_t c = coin_code(table[e].x);
                coins[e] = static_cast<uint8_t>(c);
                sum += c;
            }
        }
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, m);
    if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long tot = 0;
        for (int w = 0; w < kSampleThreads / 32; ++w) tot += s_sum[w];
        atomicAdd(coin_sum, tot);
    }
}

// its/sampling/shader.comp:80-94
__device__ __forceinline__ float search_range_u(const float* __restrict__ cmf, uint32_t x,
                                                uint32_t y, float u) {
    const float lo = x > 0 ? __ldg(cmf + x - 1) : 0.0f;
    const float hi = __ldg(cmf + y);
    return __fadd_rn(lo, __fmul_rn(__fsub_rn(hi, lo), u));
}

// its/sampling/shader.comp:131-140: lower bound with the shader's probe sequence
__device__ __forceinline__ uint32_t bisect(const float* __restrict__ cmf, uint32_t x, uint32_t y,
                                           float u) {
    while (x < y) {
        const uint32_t mid = x + ((y - x) >> 1);
        if (u > __ldg(cmf + mid))
            x = mid + 1;
        else
            y = mid;
    }
    return x;
}

// T = (2x + 1) * total * 2^-33 as (t_hi = T rounded to nearest FP32, t_sgn = sign(T - t_hi)).
// total = Mt * 2^Et with a 24-bit integer Mt; P = (2x + 1) * Mt < 2^57 is exact in 64 bits.
__device__ __forceinline__ void exact_target(uint32_t x, float total, float& t_hi, int& t_sgn) {
    const uint32_t tb = __float_as_uint(total);
    const int e = static_cast<int>((tb >> 23) & 0xffu);
    const uint64_t mt = e ? ((tb & 0x7fffffu) | 0x800000u) : (tb & 0x7fffffu);
    const int et = (e ? e : 1) - 150;
    const uint64_t P = (2ull * x + 1ull) * mt;
    if (P == 0) {
        t_hi = 0.0f;
        t_sgn = 0;
        return;
    }
    const int bits = 64 - __clzll(static_cast<long long>(P));
    int sh = bits > 24 ? bits - 24 : 0;
    uint64_t mant = P >> sh;
    int sgn = 0;
    if (sh > 0) {
        const uint64_t rem = P & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (mant & 1ull))) {
            ++mant;
            sgn = -1;
        } else {
            sgn = rem ? 1 : 0;
        }
        if (mant == (1ull << 24)) {
            mant >>= 1;
            ++sh;
        }
    }
    t_hi = ldexpf(static_cast<float>(mant), et - 33 + sh);
    t_sgn = sgn;
}

// first index in [0, last] with cmf >= T, bisecting like its/sampling/shader.comp:131-140
__device__ __forceinline__ uint32_t bisect_exact(const float* __restrict__ cmf, uint32_t last,
                                                 float t_hi, int t_sgn) {
    uint32_t x = 0, y = last;
    while (x < y) {
        const uint32_t mid = x + ((y - x) >> 1);
        const float c = __ldg(cmf + mid);
        if (t_hi > c || (t_hi == c && t_sgn > 0))
            x = mid + 1;
        else
            y = mid;
    }
    return x;
}

// COOP: 0 = none, 1 = binary narrowing, 2 = p-array narrowing.  One sample per thread so a
// warp is the shader's subgroup of 32 consecutive samples; every lane of the warp takes
// part in the narrowing (also lanes past S in the last warp, which then store nothing).
template <uint32_t RNG, int COOP>
__global__ __launch_bounds__(kSampleThreads) void k_its_sample(const float* __restrict__ cmf,
                                                               uint32_t n, uint64_t S,
                                                               uint64_t seed, uint64_t offset,
                                                               uint32_t coop,
                                                               uint32_t* __restrict__ out) {
    pdl_entry();
    const uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if constexpr (COOP == 0) {
        if (s >= S) return;
    } else {
        if ((s & ~31ull) >= S) return;  // whole warps only
    }
    uint32_t res;
    if constexpr (RNG == RNG_REF) {
        const uint32_t seed32 = static_cast<uint32_t>(seed);
        const uint32_t g = static_cast<uint32_t>(offset + s);
        uint32_t x = 0, y = n - 1u;
        if constexpr (COOP != 0) {
            const int lane = threadIdx.x & 31;
            const uint32_t g0 = __shfl_sync(0xffffffffu, g, 0);
            const float u1 =
                __shfl_sync(0xffffffffu, search_range_u(cmf, 0, n - 1u, unit_ref(wang_hash(seed32 + g0))), 0);
            if constexpr (COOP == 2) {
                uint32_t range = y - x + 1u;
                while (range > coop) {
                    const uint32_t base = range / 32u;
                    const uint32_t start = x + lane * base;
                    uint32_t end = start + base - 1u;
                    end = end > y ? y : end;
                    const unsigned b = __ballot_sync(0xffffffffu, u1 < __ldg(cmf + end));
                    if (b) {
                        const int id = __ffs(b) - 1;
                        x = __shfl_sync(0xffffffffu, start, id);
                        y = __shfl_sync(0xffffffffu, end, id);
                    } else {
                        // u1 beyond every partition end (the shader's ballot is empty there):
                        // keep the remainder, at least the last item
                        x = min(x + 32u * base, y);
                    }
                    range = y - x + 1u;
                }
            } else {
                while (y - x + 1u > coop) {
                    const uint32_t mid = x + ((y - x) >> 1);
                    if (u1 > __ldg(cmf + mid))
                        x = mid + 1;
                    else
                        y = mid;
                }
            }
        }
        const float u2 = search_range_u(cmf, x, y, unit_ref(wang_hash((seed32 ^ 0xA9EC5C80u) + g)));
        res = bisect(cmf, x, y, u2);
    } else {
        uint2 ks[10];
        philox4x32_10_keys(seed, ks);
        const uint64_t g = offset + s;
        const uint4 r = philox4x32_10(
            make_uint4(static_cast<uint32_t>(g), static_cast<uint32_t>(g >> 32), 0u, 0u), ks);
        float t_hi;
        int t_sgn;
        exact_target(r.x, __ldg(cmf + n - 1u), t_hi, t_sgn);
        res = bisect_exact(cmf, n - 1u, t_hi, t_sgn);
    }
    if (s < S) __stcs(out + s, res);
}

// ---- ITS without cooperative narrowing: the bisection's probe tree, top cached ----------
//
// Every non-cooperative search starts with x = 0, y = N - 1 and probes mid = x + (y - x) / 2,
// so its first probes walk one implicit binary tree: node k (root 1; children 2k for
// "T <= cmf[mid]" and 2k + 1 for "T > cmf[mid]") holds the range left by the branch
// decisions spelled by the bits of k below its leading one.  Each CTA copies the probe
// values of the top kItsTreeLevels levels into shared memory once, then runs the searches
// -- unchanged probe sequence, so results are bit-identical to the plain bisection -- with
// kItsPerThread searches interleaved per thread to keep several loads in flight.
constexpr int kItsTreeLevels = 12;
constexpr int kItsTreeNodes = 1 << kItsTreeLevels;  // nodes 1 .. 4095 (index 0 unused)
constexpr int kItsPerThread = 4;
constexpr int kItsGroup = kSampleThreads * kItsPerThread;
constexpr int kItsMaxBlocks = 152 * 16;

__device__ __forceinline__ void tree_range(uint32_t k, uint32_t last, uint32_t& x, uint32_t& y) {
    x = 0;
    y = last;
    const int d = 31 - __clz(k);
    for (int b = d - 1; b >= 0; --b) {
        if (x >= y) return;
        const uint32_t mid = x + ((y - x) >> 1);
        if ((k >> b) & 1u)
            x = mid + 1;
        else
            y = mid;
    }
}

static_assert(kItsTreeLevels == static_cast<int>(kTreeTop), "shared levels above the blocks");

// One thread per stored block (TreeBlock): the range of its root node, then the ranges of the
// root's 6 descendants and the probe values of the 7 nodes (0 for a node whose range is one
// index: no search reaches it with a probe).  Slot 7 holds the root's range [x, x + len - 1]
// as x | (len - floor(n / 2^level)) << 31: the ranges of one tree level are floor(n / 2^level)
// or one more long (the left half of a range takes the odd index), and x < 2^31.
__global__ __launch_bounds__(kSampleThreads) void k_its_tree(const float* __restrict__ cmf,
                                                             uint32_t n, uint32_t L,
                                                             TreeBlock* __restrict__ blocks) {
    pdl_entry();
    static_assert(its_tree_blocks(kTopBlockLevels) == kTopBlocks, "top block count");
    const size_t gb = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gb >= its_tree_blocks(L)) return;
    uint32_t level = 0;
    size_t off = 0;
    while (gb >= off + (size_t(1) << level)) {
        off += size_t(1) << level;
        level += kTreeBlockLevels;
    }
    uint32_t xs[8], ys[8];
    tree_range((1u << level) + static_cast<uint32_t>(gb - off), n - 1u, xs[1], ys[1]);
    float v[8];
#pragma unroll
    for (int j = 1; j < 8; ++j) {
        const bool live = xs[j] < ys[j];
        const uint32_t mid = xs[j] + ((ys[j] - xs[j]) >> 1);
        v[j - 1] = live ? __ldg(cmf + mid) : 0.0f;
        if (j < 4) {
            // children: a finished range leaves finished ones
            xs[2 * j] = xs[j];
            ys[2 * j] = live ? mid : xs[j];
            xs[2 * j + 1] = live ? mid + 1 : xs[j];
            ys[2 * j + 1] = live ? ys[j] : xs[j];
        }
    }
    v[7] = __uint_as_float(xs[1] | ((ys[1] - xs[1] + 1u - (n >> level)) << 31));
    float4* dst = reinterpret_cast<float4*>(blocks + gb);
    dst[0] = make_float4(v[0], v[1], v[2], v[3]);
    dst[1] = make_float4(v[4], v[5], v[6], v[7]);
}

// With stored blocks (B > 0, so n > 2^16) no range ends above the tail: the ranges of tree
// level l hold at least floor(n / 2^l) >= 4 indices for every l below the last block level's
// bottom.  The shared and all but the last block levels then only follow the node (its probe
// value is the tree's); the last block's slot 7 gives the range of its root, and the searches
// track their ranges from there.  A decision is one comparison: "T > c" (the exact target's
// tie rule folded into the FP32 target: T_hi + a positive remainder is > c exactly when the
// next float above T_hi is > c).
template <uint32_t RNG>
__global__ __launch_bounds__(kSampleThreads) void k_its_sample_tree(const float* __restrict__ cmf,
                                                                    uint32_t n, uint64_t S,
                                                                    uint64_t seed, uint64_t offset,
                                                                    uint32_t* __restrict__ out,
                                                                    const TreeBlock* __restrict__ blocks,
                                                                    uint32_t B) {
    pdl_entry();
    __shared__ float s_tree[kItsTreeNodes];
    const uint32_t last = n - 1u;
    for (uint32_t k = threadIdx.x + 1; k < kItsTreeNodes; k += blockDim.x) {
        uint32_t x, y;
        tree_range(k, last, x, y);
        s_tree[k] = x < y ? __ldg(cmf + x + ((y - x) >> 1)) : 0.0f;
    }
    __syncthreads();
    const float total = __ldg(cmf + last);
    for (uint64_t grp = blockIdx.x; grp * kItsGroup < S; grp += gridDim.x) {
        const uint64_t s0 = grp * kItsGroup + threadIdx.x;
        float t[kItsPerThread];  // a search goes right at probe c exactly when t > c
        uint32_t x[kItsPerThread], y[kItsPerThread], node[kItsPerThread];
        if constexpr (RNG == RNG_REF) {
            const uint32_t seed32 = static_cast<uint32_t>(seed);
#pragma unroll
            for (int v = 0; v < kItsPerThread; ++v) {
                const uint32_t g = static_cast<uint32_t>(offset + s0 + v * kSampleThreads);
                t[v] = search_range_u(cmf, 0, last, unit_ref(wang_hash((seed32 ^ 0xA9EC5C80u) + g)));
            }
        } else {
            uint2 ks[10];
            philox4x32_10_keys(seed, ks);
#pragma unroll
            for (int v = 0; v < kItsPerThread; ++v) {
                const uint64_t g = offset + s0 + v * kSampleThreads;
                const uint4 r = philox4x32_10(
                    make_uint4(static_cast<uint32_t>(g), static_cast<uint32_t>(g >> 32), 0u, 0u), ks);
                float t_hi;
                int t_sgn;
                exact_target(r.x, total, t_hi, t_sgn);
                // t_hi >= 0: the next float above is one bit pattern up (+inf above the largest)
                t[v] = t_sgn > 0 ? __uint_as_float(__float_as_uint(t_hi) + 1u) : t_hi;
            }
        }
        if (B > 0) {
#pragma unroll
            for (int v = 0; v < kItsPerThread; ++v) node[v] = 1;
#pragma unroll
            for (int l = 0; l < kItsTreeLevels; ++l)
#pragma unroll
                for (int v = 0; v < kItsPerThread; ++v)
                    node[v] = 2 * node[v] + (t[v] > s_tree[node[v]] ? 1u : 0u);
            const TreeBlock* level_blocks = blocks;
            uint32_t level = kTreeTop;
#pragma unroll 1
            for (uint32_t bl = 0; bl < B; ++bl, level += kTreeBlockLevels) {
                const uint32_t first = 1u << level;  // the level's first node
                uint4 lo[kItsPerThread], hi[kItsPerThread];
#pragma unroll
                for (int v = 0; v < kItsPerThread; ++v)
                    ld_u32x8(reinterpret_cast<const uint32_t*>(level_blocks + (node[v] - first)),
                             lo[v], hi[v]);
                level_blocks += first;
                if (bl + 1 < B) {
#pragma unroll
                    for (int v = 0; v < kItsPerThread; ++v) {
                        const uint32_t r0 = t[v] > __uint_as_float(lo[v].x) ? 1u : 0u;
                        const uint32_t r1 =
                            t[v] > __uint_as_float(r0 ? lo[v].z : lo[v].y) ? 1u : 0u;
                        const uint32_t c2 = r0 ? (r1 ? hi[v].z : hi[v].y) : (r1 ? hi[v].x : lo[v].w);
                        const uint32_t r2 = t[v] > __uint_as_float(c2) ? 1u : 0u;
                        node[v] = 8 * node[v] + 4 * r0 + 2 * r1 + r2;
                    }
                } else {
                    const uint32_t floor_len = n >> level;
#pragma unroll
                    for (int v = 0; v < kItsPerThread; ++v) {
                        x[v] = hi[v].w & 0x7fffffffu;
                        y[v] = x[v] + floor_len + (hi[v].w >> 31) - 1u;
                        uint32_t mid = x[v] + ((y[v] - x[v]) >> 1);
                        const uint32_t r0 = t[v] > __uint_as_float(lo[v].x) ? 1u : 0u;
                        x[v] = r0 ? mid + 1 : x[v];
                        y[v] = r0 ? y[v] : mid;
                        mid = x[v] + ((y[v] - x[v]) >> 1);
                        const uint32_t r1 =
                            t[v] > __uint_as_float(r0 ? lo[v].z : lo[v].y) ? 1u : 0u;
                        x[v] = r1 ? mid + 1 : x[v];
                        y[v] = r1 ? y[v] : mid;
                        mid = x[v] + ((y[v] - x[v]) >> 1);
                        const uint32_t c2 = r0 ? (r1 ? hi[v].z : hi[v].y) : (r1 ? hi[v].x : lo[v].w);
                        const uint32_t r2 = t[v] > __uint_as_float(c2) ? 1u : 0u;
                        x[v] = r2 ? mid + 1 : x[v];
                        y[v] = r2 ? y[v] : mid;
                        // the tail reads stay inside the CMF whatever the block holds
                        y[v] = min(y[v], last);
                        x[v] = min(x[v], y[v]);
                    }
                }
            }
#pragma unroll
            for (int v = 0; v < kItsPerThread; ++v)
                if (s0 + v * kSampleThreads >= S) y[v] = x[v];  // past the end: no tail loads
        } else {
            // the shared levels with ranges (short CMFs end inside them)
#pragma unroll
            for (int v = 0; v < kItsPerThread; ++v) {
                x[v] = 0;
                y[v] = s0 + v * kSampleThreads < S ? last : 0u;
                node[v] = 1;
            }
#pragma unroll 1
            for (int l = 0; l < kItsTreeLevels; ++l) {
#pragma unroll
                for (int v = 0; v < kItsPerThread; ++v) {
                    if (x[v] < y[v]) {
                        const uint32_t mid = x[v] + ((y[v] - x[v]) >> 1);
                        if (t[v] > s_tree[node[v]]) {
                            x[v] = mid + 1;
                            node[v] = 2 * node[v] + 1;
                        } else {
                            y[v] = mid;
                            node[v] = 2 * node[v];
                        }
                    }
                }
            }
        }
        // remaining levels from global memory, the searches' loads issued together
        for (;;) {
            float c[kItsPerThread];
            bool any = false;
#pragma unroll
            for (int v = 0; v < kItsPerThread; ++v) {
                any = any || x[v] < y[v];
                c[v] = x[v] < y[v] ? __ldg(cmf + x[v] + ((y[v] - x[v]) >> 1)) : 0.0f;
            }
            if (!any) break;
#pragma unroll
            for (int v = 0; v < kItsPerThread; ++v) {
                if (x[v] < y[v]) {
                    const uint32_t mid = x[v] + ((y[v] - x[v]) >> 1);
                    if (t[v] > c[v])
                        x[v] = mid + 1;
                    else
                        y[v] = mid;
                }
            }
        }
#pragma unroll
        for (int v = 0; v < kItsPerThread; ++v)
            if (s0 + v * kSampleThreads < S) __stcs(out + s0 + v * kSampleThreads, x[v]);
    }
}

// ---- ITS on an exactly non-decreasing CMF: cell blocks ----------------------------------
//
// On a non-decreasing CMF every lower-bound search returns the same index, so the search can
// start anywhere that brackets the answer (the compensated scan's CMF is non-decreasing by
// construction).  The CMF's range is cut into G = ceil(N / entry) cells of equal mass, the
// Cutpoint guiding table's: cell k starts at x_k = lower bound of c_k = fl(fl(total / G) * k),
// and a target T with c_k < T <= c_{k+1} has its lower bound in [x_k, y_k], y_k = x_{k+1}
// (N - 1 for the last cell).  Cell k is stored as one 32-byte block (ItsCell): x_k, y_k and,
// for the range cut into kCellParts parts of d = ceil((y - x + 1) / kCellParts) indices, the
// CMF at the last index of each part (min(x + (j + 1) d - 1, y)).  A sample finds its cell (an
// FP32 estimate moved by exact comparisons against c_k), reads the block with one 32-byte
// load -- one random sector, what an alias-table entry costs (a random 64-byte read costs
// about twice that on GB300) -- and the first part whose last value is >= T holds the lower
// bound: with d = 1 (cells of at most kCellParts candidates) that is the answer, otherwise a
// bisection of the part's d indices of the CMF finds it.  A target above the block's last
// value (a cell estimate that did not settle) falls back to the bisection of [0, N - 1].
// Results equal the bisection's (k_its_sample_tree's).

// Starts x_k = lower bound of c_k = fl(step * k) (clamped to N - 1) of the equal-mass cells of
// a non-decreasing CMF, in three passes, each bracketing the next (c_k is non-decreasing in k,
// so x_k is too).  k_cell_coarse bisects the whole CMF for every kCoarseStride-th start;
// k_cell_groups bisects, inside those brackets, for the first start of every group of 32
// cells; then one warp per group finds its 32 starts in the group's bracket [x_{32g},
// x_{32(g+1)}]: where that holds at most 128 values, the lanes load them with one coalesced
// pass and each start is the bracket's start plus the number of values below its threshold,
// found by a bisection over the values held in the warp's registers (shuffles, no dependent
// loads); wider brackets are bisected in memory.
__device__ __forceinline__ float cell_step(const float* __restrict__ cmf, uint32_t n, uint32_t G) {
    return __fdiv_rn(__ldg(cmf + n - 1u), __uint2float_rn(G));
}

__global__ __launch_bounds__(kSampleThreads) void k_cell_coarse(const float* __restrict__ cmf,
                                                                uint32_t n, uint32_t G,
                                                                uint32_t* __restrict__ coarse) {
    pdl_entry();
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= coarse_entries(G)) return;
    const uint64_t k = static_cast<uint64_t>(j) * kCoarseStride;
    coarse[j] = k < G ? bisect(cmf, 0, n - 1u,
                               __fmul_rn(cell_step(cmf, n, G), __uint2float_rn(static_cast<uint32_t>(k))))
                      : n - 1u;
}

__device__ __forceinline__ uint32_t cell_start(const float* __restrict__ cmf, uint32_t n,
                                               uint32_t G, const uint32_t* __restrict__ coarse,
                                               uint32_t k) {
    const uint32_t j = k / kCoarseStride;
    const uint32_t lo = __ldg(coarse + j);
    if (k % kCoarseStride == 0u) return lo;
    return bisect(cmf, lo, __ldg(coarse + j + 1u),
                  __fmul_rn(cell_step(cmf, n, G), __uint2float_rn(k)));
}

// group[g] = x_{32 g} (N - 1 past the last cell), g <= ceil(G / 32)
__global__ __launch_bounds__(kSampleThreads) void k_cell_groups(const float* __restrict__ cmf,
                                                                uint32_t n, uint32_t G,
                                                                const uint32_t* __restrict__ coarse,
                                                                uint32_t* __restrict__ group) {
    pdl_entry();
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= group_entries(G)) return;
    const uint64_t k = static_cast<uint64_t>(g) * 32u;
    group[g] = k < G ? cell_start(cmf, n, G, coarse, static_cast<uint32_t>(k)) : n - 1u;
}

// The start of cell k = 32 g + lane (all lanes of the warp call it; k >= G returns N - 1), and
// the end of the group's bracket in hi.
__device__ __forceinline__ uint32_t cell_start_warp(const float* __restrict__ cmf, uint32_t n,
                                                    uint32_t G, const uint32_t* __restrict__ group,
                                                    uint32_t g, uint32_t& hi) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lo = __ldg(group + g);
    hi = __ldg(group + g + 1u);
    const uint32_t k = g * 32u + lane;
    const float t = k < G ? __fmul_rn(cell_step(cmf, n, G), __uint2float_rn(k))
                          : __int_as_float(0x7f800000);
    uint32_t x;
    if (hi >= lo && hi - lo < 128u) {
        // values lo .. lo + 127, 4 consecutive per lane (past hi or N: +inf, never below t)
        float v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t pos = lo + 4u * lane + q;
            v[q] = pos <= hi && pos < n ? __ldg(cmf + pos) : __int_as_float(0x7f800000);
        }
        // the values are non-decreasing across the lanes: find the first lane whose last
        // value is >= t (a bisection over the lanes' maxima, fixed trip count so that every
        // lane takes part in every shuffle), then count inside its 4 values
        uint32_t a = 0, b = 32;
#pragma unroll
        for (int it = 0; it < 6; ++it) {
            const uint32_t mid = (a + b) >> 1;
            const float m = __shfl_sync(0xffffffffu, v[3], min(mid, 31u));
            if (a < b) {
                if (m < t)
                    a = mid + 1u;
                else
                    b = mid;
            }
        }
        const uint32_t c = min(a, 31u);
        uint32_t in = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) in += __shfl_sync(0xffffffffu, v[q], c) < t ? 1u : 0u;
        const uint32_t cnt = a < 32u ? 4u * a + in : 128u;
        x = min(lo + cnt, hi);
    } else {
        x = k < G ? bisect(cmf, lo, hi > lo ? hi : lo, t) : n - 1u;
    }
    return k < G ? x : n - 1u;
}

// bit 31 of a cell's y: an FP32 CMF's cell the search cannot serve (the search bisects it)
constexpr uint32_t kCellUnsafe = 0x80000000u;

__device__ __forceinline__ uint32_t cell_part(uint32_t x, uint32_t y) {
    return (y - x + kCellParts) / kCellParts;  // ceil((y - x + 1) / kCellParts)
}

// CHECK (an FP32 CMF, which need not be monotone): a cell whose start x > 0 does not have
// cmf[x - 1] < c_k is marked for the bisection as it is written
template <bool CHECK>
__global__ __launch_bounds__(kSampleThreads) void k_its_cells(const float* __restrict__ cmf,
                                                              uint32_t n, uint32_t G,
                                                              const uint32_t* __restrict__ group,
                                                              ItsCell* __restrict__ cells) {
    pdl_entry();
    const uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // whole warps
    if (g * 32u >= G) return;
    uint32_t hi;
    const uint32_t x = cell_start_warp(cmf, n, G, group, g, hi);
    const uint32_t k = g * 32u + (threadIdx.x & 31u);
    // the end of a cell is the next cell's start: the next lane's, or the next group's
    uint32_t y = __shfl_down_sync(0xffffffffu, x, 1);
    if ((threadIdx.x & 31u) == 31u) y = hi;
    if (k >= G) return;
    if (k + 1u >= G) y = n - 1u;
    const uint32_t d = cell_part(x, y);
    float v[kCellParts];
#pragma unroll
    for (int j = 0; j < kCellParts; ++j)
        v[j] = __ldg(cmf + min(x + (j + 1) * d - 1u, y));
    uint32_t ym = y;
    if (CHECK && x > 0u) {
        const float ck = __fmul_rn(cell_step(cmf, n, G), __uint2float_rn(k));
        if (!(x <= n - 1u && __ldg(cmf + x - 1u) < ck)) ym |= kCellUnsafe;
    }
    uint4* dst = reinterpret_cast<uint4*>(cells + k);
    dst[0] = make_uint4(x, ym, __float_as_uint(v[0]), __float_as_uint(v[1]));
    dst[1] = make_uint4(__float_as_uint(v[2]), __float_as_uint(v[3]), __float_as_uint(v[4]),
                        __float_as_uint(v[5]));
}

// ---- cells on an FP32 CMF: cells whose targets can meet an inversion ------------------
//
// On a CMF that is not monotone every lower-bound search still returns the bisection's index
// for a target t that lies in no inversion interval (cmf[j], cmf[i]] (i < j, cmf[j] < cmf[i]):
// then every value below t comes before every value >= t.  For each i the union of its
// intervals is (S(i + 1), cmf[i]] with S the suffix minimum, so a pass over the CMF marks the
// cells whose target range meets one (bit 31 of the cell's y; n < 2^31), and the cells whose
// start x does not have cmf[x - 1] < c_k; a CMF with a value that is not finite or is negative
// marks every cell.  The cell search serves the unmarked cells and the bisection the others.
constexpr uint32_t kMarkSpan = 64;  // an interval over more cells marks the whole CMF unsafe

// the largest k < G with c_k = fl(step * k) < t (0 if none): the cell of targets just above t
__device__ __forceinline__ uint32_t cell_below(float t, float step, uint32_t G) {
    uint32_t lo = 0, hi = G - 1u;  // c_0 = 0
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo + 1u) >> 1);
        if (__fmul_rn(step, __uint2float_rn(mid)) < t)
            lo = mid;
        else
            hi = mid - 1u;
    }
    return lo;
}

// per 4096-value tile of the CMF: its minimum; any value that is NaN, infinite or negative
// raises `bad`
__global__ __launch_bounds__(kSampleThreads) void k_cmf_tile_min(const float* __restrict__ cmf,
                                                                 uint32_t n,
                                                                 float* __restrict__ tile_min,
                                                                 uint32_t* __restrict__ bad) {
    pdl_entry();
    __shared__ float s_m[kSampleThreads / 32];
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTileItems;
    float m = INFINITY;
    bool b = false;
    for (uint32_t e = threadIdx.x; e < kTileItems; e += blockDim.x) {
        if (base + e < n) {
            const float v = __ldg(cmf + base + e);
            b = b || !(v >= 0.0f && v <= 3.402823466e38f);
            m = fminf(m, v);
        }
    }
    if (__syncthreads_or(b) && threadIdx.x == 0) atomicOr(bad, 1u);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, d));
    if ((threadIdx.x & 31u) == 0) s_m[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < static_cast<int>(kSampleThreads / 32); ++w) m = fminf(m, s_m[w]);
        tile_min[blockIdx.x] = fminf(m, s_m[0]);
    }
}

// suffix minima of the tile minima (one CTA, chunks of 1024 from the end)
__global__ __launch_bounds__(1024) void k_tile_suffix_min(const float* __restrict__ tile_min,
                                                          uint32_t tiles,
                                                          float* __restrict__ suf) {
    pdl_entry();
    __shared__ float s_w[32];
    __shared__ float s_carry;
    if (threadIdx.x == 0) s_carry = INFINITY;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t end = tiles; end > 0; end -= 1024) {
        // thread j holds tile end - 1 - j (reversed, so an inclusive prefix min is a suffix min)
        const int64_t t = end - 1 - static_cast<int64_t>(threadIdx.x);
        float v = t >= 0 ? tile_min[t] : INFINITY;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const float o = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= d) v = fminf(v, o);
        }
        if (lane == 31) s_w[warp] = v;
        __syncthreads();
        if (warp == 0) {
            float u = s_w[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const float o = __shfl_up_sync(0xffffffffu, u, d);
                if (lane >= d) u = fminf(u, o);
            }
            s_w[lane] = u;  // inclusive over warps 0 .. lane
        }
        __syncthreads();
        const float carry = s_carry;
        const float r = fminf(fminf(v, warp ? s_w[warp - 1] : INFINITY), carry);
        if (t >= 0) suf[t] = r;
        __syncthreads();
        if (threadIdx.x == 1023) s_carry = r;
        __syncthreads();
    }
}

// marks the cells k in [cell_below(lo+), cell_below(hi)] for the interval (lo, hi]; an interval
// over more than kMarkSpan cells raises `bad` instead
__device__ __forceinline__ void mark_interval(float lo, float hi, float step, uint32_t G,
                                              ItsCell* __restrict__ cells,
                                              uint32_t* __restrict__ bad) {
    const uint32_t a = cell_below(__uint_as_float(__float_as_uint(lo) + 1u), step, G);
    const uint32_t b = cell_below(hi, step, G);
    if (b >= a && b - a >= kMarkSpan) {
        atomicOr(bad, 1u);
        return;
    }
    for (uint32_t k = a; k <= b; ++k) atomicOr(&cells[k].y, kCellUnsafe);
}

// one CTA per 4096-value tile, 16 consecutive values per thread: S(i + 1) from the thread's own
// later values, the later threads' and the later tiles' minima; every i with S(i + 1) < cmf[i]
// marks the cells of (S(i + 1), cmf[i]].  Skipped when `bad` is set (every cell is marked then).
__global__ __launch_bounds__(kSampleThreads) void k_cmf_mark(const float* __restrict__ cmf,
                                                             uint32_t n, uint32_t G,
                                                             const float* __restrict__ suf,
                                                             uint32_t tiles,
                                                             ItsCell* __restrict__ cells,
                                                             uint32_t* __restrict__ bad) {
    pdl_entry();
    __shared__ float s_w[kSampleThreads / 32];
    // one decision for the whole CTA (other CTAs may raise `bad` meanwhile)
    if (__syncthreads_or(*reinterpret_cast<volatile uint32_t*>(bad) != 0u)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kTileItems + threadIdx.x * 16u;
    float v[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) v[c] = base + c < n ? __ldg(cmf + base + c) : INFINITY;
    float tmin = v[15];
#pragma unroll
    for (int c = 14; c >= 0; --c) tmin = fminf(tmin, v[c]);
    // minimum over the later threads of the tile (exclusive), then over the later tiles
    float inc = tmin;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float o = __shfl_down_sync(0xffffffffu, inc, d);
        if (lane + d < 32) inc = fminf(inc, o);
    }
    if (lane == 0) s_w[warp] = inc;  // warp's minimum
    __syncthreads();
    float after = __shfl_down_sync(0xffffffffu, inc, 1);
    if (lane == 31) after = INFINITY;
    for (int w = warp + 1; w < static_cast<int>(kSampleThreads / 32); ++w) after = fminf(after, s_w[w]);
    if (blockIdx.x + 1u < tiles) after = fminf(after, suf[blockIdx.x + 1u]);
    const float step = __fdiv_rn(__ldg(cmf + n - 1u), __uint2float_rn(G));
    float s = after;  // S(i + 1) for the thread's last value
#pragma unroll
    for (int c = 15; c >= 0; --c) {
        if (base + c < n && s < v[c]) mark_interval(s, v[c], step, G, cells, bad);
        s = fminf(s, v[c]);
    }
}

// with `bad` raised (a value that is not finite or is negative, or an interval over too many
// cells) every cell is marked
__global__ __launch_bounds__(kSampleThreads) void k_cells_mark_all(uint32_t G,
                                                                   ItsCell* __restrict__ cells,
                                                                   const uint32_t* __restrict__ bad) {
    pdl_entry();
    if (*reinterpret_cast<const volatile uint32_t*>(bad) == 0u) return;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < G; k += gridDim.x * blockDim.x)
        cells[k].y |= kCellUnsafe;
}

// The bisection of [0, n - 1] for target t (a probe c sends it right when t > c) through the
// stored probe-tree blocks (L = its_tree_stored_levels(n) > 0 levels: the node alone above the
// last one, whose slot 7 gives the range), then the CMF for the tail: the same probe sequence.
__device__ uint32_t bisect_blocks(const float* __restrict__ cmf, uint32_t n,
                                  const TreeBlock* __restrict__ blocks, uint32_t L, float t) {
    uint32_t node = 1, level = 0, x = 0, y = 0;
    const TreeBlock* lb = blocks;
    for (uint32_t bl = 0; bl < L; ++bl, level += kTreeBlockLevels) {
        const uint32_t first = 1u << level;
        uint4 lo, hi;
        ld_u32x8(reinterpret_cast<const uint32_t*>(lb + (node - first)), lo, hi);
        lb += first;
        const uint32_t r0 = t > __uint_as_float(lo.x) ? 1u : 0u;
        const uint32_t c1 = r0 ? lo.z : lo.y;
        const uint32_t r1 = t > __uint_as_float(c1) ? 1u : 0u;
        const uint32_t c2 = r0 ? (r1 ? hi.z : hi.y) : (r1 ? hi.x : lo.w);
        const uint32_t r2 = t > __uint_as_float(c2) ? 1u : 0u;
        if (bl + 1u < L) {
            node = 8u * node + 4u * r0 + 2u * r1 + r2;
        } else {
            x = hi.w & 0x7fffffffu;
            y = x + (n >> level) + (hi.w >> 31) - 1u;
            const uint32_t r[3] = {r0, r1, r2};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const uint32_t mid = x + ((y - x) >> 1);
                x = r[d] ? mid + 1u : x;
                y = r[d] ? y : mid;
            }
            y = min(y, n - 1u);
            x = min(x, y);
        }
    }
    while (x < y) {
        const uint32_t mid = x + ((y - x) >> 1);
        if (t > __ldg(cmf + mid))
            x = mid + 1u;
        else
            y = mid;
    }
    return x;
}

// steps of the cell correction (beyond them the bracket check sends the sample to the
// bisection, so the bound only caps the work)
constexpr int kCellFix = 8;

template <uint32_t RNG>
__global__ __launch_bounds__(kSampleThreads) void k_its_sample_cells(
    const float* __restrict__ cmf, uint32_t n, const ItsCell* __restrict__ cells, uint32_t G,
    uint64_t S, uint64_t seed, uint64_t offset, uint32_t* __restrict__ out,
    const TreeBlock* __restrict__ blocks, uint32_t L) {
    pdl_entry();
    const uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const uint32_t last = n - 1u;
    const float total = __ldg(cmf + last);
    const uint64_t g = offset + s;
    float t_hi;
    int t_sgn = 0;
    if constexpr (RNG == RNG_REF) {
        const uint32_t seed32 = static_cast<uint32_t>(seed);
        t_hi = search_range_u(cmf, 0, last,
                              unit_ref(wang_hash((seed32 ^ 0xA9EC5C80u) + static_cast<uint32_t>(g))));
    } else {
        uint2 ks[10];
        philox4x32_10_keys(seed, ks);
        const uint4 r = philox4x32_10(
            make_uint4(static_cast<uint32_t>(g), static_cast<uint32_t>(g >> 32), 0u, 0u), ks);
        exact_target(r.x, total, t_hi, t_sgn);
    }
    // "T > c" for the target T = (t_hi, t_sgn) (RNG_REF: t_sgn = 0, the shader's u > cmf[mid])
    auto above = [&](float c) { return t_hi > c || (t_hi == c && t_sgn > 0); };
    // the cell holding T: c_k < T <= c_{k+1} with the build's c_k = fl(step * k), from an FP32
    // estimate (off by a few cells at most) moved by exact comparisons
    const float step = __fdiv_rn(total, __uint2float_rn(G));
    const float scale = __fdiv_rn(__uint2float_rn(G), total);
    uint32_t k = __float2uint_rz(__fmul_rn(t_hi, scale));
    k = k < G - 1u ? k : G - 1u;
    for (int it = 0; it < kCellFix && k > 0u && !above(__fmul_rn(step, __uint2float_rn(k))); ++it)
        --k;
    for (int it = 0; it < kCellFix && k + 1u < G && above(__fmul_rn(step, __uint2float_rn(k + 1u)));
         ++it)
        ++k;
    // c_k < T <= c_{k+1} (then cmf[x_k - 1] < c_k < T, and T is in the range the cell's
    // inversion mark covers); cmf[y_k] >= T is checked on the block
    const bool settled = (k == 0u || above(__fmul_rn(step, __uint2float_rn(k)))) &&
                         (k + 1u >= G || !above(__fmul_rn(step, __uint2float_rn(k + 1u))));
    const uint64_t once = l2_policy_evict_first();
    uint4 q0, q1;
    ld_u32x8_policy(reinterpret_cast<const uint32_t*>(cells + k), once, q0, q1);
    // an FP32 CMF's cell may be marked (its targets can meet an inversion, or its start is not
    // below c_k): bisect those (the compensated CMF's cells are never marked)
    const bool unsafe = (q0.y & kCellUnsafe) != 0u;
    // (a cell block holds indices < n for the n it was built for; the clamp keeps any other
    // block's search inside the CMF)
    uint32_t x = q0.x, y = min(q0.y & ~kCellUnsafe, last);
    const float v[kCellParts] = {__uint_as_float(q0.z), __uint_as_float(q0.w),
                                 __uint_as_float(q1.x), __uint_as_float(q1.y),
                                 __uint_as_float(q1.z), __uint_as_float(q1.w)};
    // (y >= x holds for every non-decreasing CMF; the test keeps weights outside the
    // contract -- NaN, negative -- from producing an index outside [0, N))
    if (!unsafe && settled && y >= x && !above(v[kCellParts - 1])) {
        // the first part whose last value is >= T (the values are non-decreasing)
        uint32_t part = 0;
#pragma unroll
        for (int j = 0; j < kCellParts; ++j) part += above(v[j]) ? 1u : 0u;
        const uint32_t d = cell_part(x, y);
        const uint32_t lo = x + part * d;
        if (d == 1u) {
            __stcs(out + s, lo);
            return;
        }
        y = min(lo + d - 1u, y);  // cmf[y] >= T and cmf[lo - 1] < T
        x = lo;
    } else if (blocks) {
        // the bisection through the stored probe tree (t_hi with the tie folded in: T > c
        // exactly when the next float above t_hi is > c, for t_sgn > 0)
        const float t = t_sgn > 0 ? __uint_as_float(__float_as_uint(t_hi) + 1u) : t_hi;
        __stcs(out + s, bisect_blocks(cmf, n, blocks, L, t));
        return;
    } else {
        x = 0;
        y = last;
    }
    while (x < y) {
        const uint32_t mid = x + ((y - x) >> 1);
        if (above(ld_f32_policy(cmf + mid, once)))
            x = mid + 1;
        else
            y = mid;
    }
    __stcs(out + s, x);
}

// Guiding table of an exactly non-decreasing CMF: the same entries as k_cutpoint_guide
// (guide[k] = lower bound of fl(fl(total / G) * k), clamped to N - 1), where every lower-bound
// search gives the same index, so the bracketed searches of cell_start apply.
__global__ __launch_bounds__(kSampleThreads) void k_guide_monotone(const float* __restrict__ cmf,
                                                                   uint32_t n, uint32_t G,
                                                                   const uint32_t* __restrict__ group,
                                                                   uint32_t* __restrict__ guide) {
    pdl_entry();
    const uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // whole warps
    if (g * 32u >= G) return;
    uint32_t hi;
    const uint32_t x = cell_start_warp(cmf, n, G, group, g, hi);
    const uint32_t k = g * 32u + (threadIdx.x & 31u);
    if (k < G) guide[k] = x;
}

// the first two passes: coarse starts, then group starts (scratch: coarse_entries(G) +
// group_entries(G) words); returns the group array
static uint32_t* launch_cell_brackets(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                                      uint32_t* scratch) {
    const uint32_t m = coarse_entries(G), ng = group_entries(G);
    uint32_t* group = scratch + m;
    launch_pdl(k_cell_coarse, (m + kSampleThreads - 1) / kSampleThreads, kSampleThreads, 0, st, cmf, n, G,
                                                                                        scratch);
    launch_pdl(k_cell_groups, (ng + kSampleThreads - 1) / kSampleThreads, kSampleThreads, 0, st, 
        cmf, n, G, scratch, group);
    return group;
}

static uint32_t warp_blocks(uint32_t G) {
    const uint64_t threads = (static_cast<uint64_t>(G) + 31u) / 32u * 32u;
    return static_cast<uint32_t>((threads + kSampleThreads - 1) / kSampleThreads);
}

cudaError_t launch_its_cells(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                             uint32_t* coarse, ItsCell* cells, bool check) {
    uint32_t* group = launch_cell_brackets(st, cmf, n, G, coarse);
    if (check)
        launch_pdl(k_its_cells<true>, warp_blocks(G), kSampleThreads, 0, st, cmf, n, G, group, cells);
    else
        launch_pdl(k_its_cells<false>, warp_blocks(G), kSampleThreads, 0, st, cmf, n, G, group, cells);
    return cudaGetLastError();
}

cudaError_t launch_its_marks(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                             ItsCell* cells, float* tile_scratch, uint32_t* bad) {
    const uint32_t tiles = tiles_for(n);
    float* tile_min = tile_scratch;
    float* suf = tile_scratch + tiles;
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    launch_pdl(k_cmf_tile_min, tiles, kSampleThreads, 0, st, cmf, n, tile_min, bad);
    launch_pdl(k_tile_suffix_min, 1, 1024, 0, st, tile_min, tiles, suf);
    launch_pdl(k_cmf_mark, tiles, kSampleThreads, 0, st, cmf, n, G, suf, tiles, cells, bad);
    // (a grid-stride loop: any grid covers the cells; most launches return at once)
    const uint32_t mark_grid = min((G + kSampleThreads - 1) / kSampleThreads, 1024u);
    launch_pdl(k_cells_mark_all, mark_grid, kSampleThreads, 0, st, G, cells, bad);
    return cudaGetLastError();
}

cudaError_t launch_its_sample_cells(cudaStream_t st, uint32_t rng, const float* cmf, uint32_t n,
                                    const ItsCell* cells, uint32_t G, uint64_t S, uint64_t seed,
                                    uint64_t offset, uint32_t* out, const TreeBlock* blocks,
                                    uint32_t L) {
    const uint64_t grid = (S + kSampleThreads - 1) / kSampleThreads;
    if (grid == 0) return cudaSuccess;
    if (grid > 0x7fffffffull) return cudaErrorInvalidValue;
    if (rng == RNG_REF)
        launch_pdl(k_its_sample_cells<RNG_REF>, static_cast<unsigned>(grid), kSampleThreads, 0, st, 
            cmf, n, cells, G, S, seed, offset, out, blocks, L);
    else
        launch_pdl(k_its_sample_cells<RNG_PHILOX>, static_cast<unsigned>(grid), kSampleThreads, 0, st, 
            cmf, n, cells, G, S, seed, offset, out, blocks, L);
    return cudaGetLastError();
}

// ---- Cutpoint (guiding table) -----------------------------------------------------------

// cutpoint/guiding_table/shader.comp:40-55: entry k = lower bound of (total / G) * k over the
// whole CMF, with the shader's FP32 step and probe sequence.
__global__ __launch_bounds__(kSampleThreads) void k_cutpoint_guide(const float* __restrict__ cmf,
                                                                   uint32_t n, uint32_t G,
                                                                   uint32_t* __restrict__ guide) {
    pdl_entry();
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= G) return;
    const float total = __ldg(cmf + n - 1u);
    const float step = __fdiv_rn(total, __uint2float_rn(G));
    guide[k] = bisect(cmf, 0, n - 1u, __fmul_rn(step, __uint2float_rn(k)));
}

// cutpoint/sampling/shader.comp:100-140.  The subgroup's elected lane (the first sample of the
// aligned group of 32) draws u1, which picks guiding cell k = min(u1 * G, G - 1); the search
// range is [guide[k], guide[k + 1]] (up to N - 1 for the last cell), and every sample bisects
// it for u2 drawn inside the cell's CMF range.  RNG_REF: u1 = wang_hash(seed + g0), u2 =
// wang_hash((seed ^ 0x79145147) + g) as the shader; RNG_PHILOX: u1 = x0 of the group's first
// sample, u2 = x1 of the sample (Philox4x32-10, counter = sample index).
template <uint32_t RNG>
__global__ __launch_bounds__(kSampleThreads) void k_cutpoint_sample(
    const float* __restrict__ cmf, uint32_t n, const uint32_t* __restrict__ guide, uint32_t G,
    uint64_t S, uint64_t seed, uint64_t offset, uint32_t* __restrict__ out) {
    pdl_entry();
    const uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const uint64_t g = offset + s, g0 = offset + (s & ~31ull);
    float u1, uu;
    if constexpr (RNG == RNG_REF) {
        const uint32_t seed32 = static_cast<uint32_t>(seed);
        u1 = unit_ref(wang_hash(seed32 + static_cast<uint32_t>(g0)));
        uu = unit_ref(wang_hash((seed32 ^ 0x79145147u) + static_cast<uint32_t>(g)));
    } else {
        uint2 ks[10];
        philox4x32_10_keys(seed, ks);
        const uint4 r0 = philox4x32_10(
            make_uint4(static_cast<uint32_t>(g0), static_cast<uint32_t>(g0 >> 32), 0u, 0u), ks);
        const uint4 r = philox4x32_10(
            make_uint4(static_cast<uint32_t>(g), static_cast<uint32_t>(g >> 32), 0u, 0u), ks);
        u1 = unit_ref(r0.x);
        uu = unit_ref(r.y);
    }
    uint32_t k = __float2uint_rz(__fmul_rn(u1, __uint2float_rn(G)));
    k = k < G - 1u ? k : G - 1u;
    // (entries are < n for the CMF the table was built from; the clamps keep a table built
    // for another n from reading outside the CMF)
    const uint32_t x = min(__ldg(guide + k), n - 1u);
    const uint32_t y = k != G - 1u ? max(min(__ldg(guide + k + 1u), n - 1u), x) : n - 1u;
    const float u2 = search_range_u(cmf, x, y, uu);
    __stcs(out + s, bisect(cmf, x, y, u2));
}

cudaError_t launch_cutpoint_guide(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                                  uint32_t* guide) {
    const uint32_t blocks = (G + kSampleThreads - 1) / kSampleThreads;
    launch_pdl(k_cutpoint_guide, blocks, kSampleThreads, 0, st, cmf, n, G, guide);
    return cudaGetLastError();
}

cudaError_t launch_guide_monotone(cudaStream_t st, const float* cmf, uint32_t n, uint32_t G,
                                  uint32_t* coarse, uint32_t* guide) {
    uint32_t* group = launch_cell_brackets(st, cmf, n, G, coarse);
    launch_pdl(k_guide_monotone, warp_blocks(G), kSampleThreads, 0, st, cmf, n, G, group, guide);
    return cudaGetLastError();
}

cudaError_t launch_cutpoint_sample(cudaStream_t st, uint32_t rng, const float* cmf, uint32_t n,
                                   const uint32_t* guide, uint32_t G, uint64_t S, uint64_t seed,
                                   uint64_t offset, uint32_t* out) {
    const uint64_t blocks = (S + kSampleThreads - 1) / kSampleThreads;
    if (blocks == 0) return cudaSuccess;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    if (rng == RNG_REF)
        launch_pdl(k_cutpoint_sample<RNG_REF>, static_cast<unsigned>(blocks), kSampleThreads, 0, st, 
            cmf, n, guide, G, S, seed, offset, out);
    else
        launch_pdl(k_cutpoint_sample<RNG_PHILOX>, static_cast<unsigned>(blocks), kSampleThreads, 0, st, 
            cmf, n, guide, G, S, seed, offset, out);
    return cudaGetLastError();
}

cudaError_t launch_alias_sample(cudaStream_t st, uint32_t rng, uint32_t coop, const uint2* table,
                                const uint8_t* coins, const unsigned long long* coin_sum,
                                uint32_t n, uint64_t S, uint64_t seed, uint64_t offset,
                                uint32_t* out) {
    const uint64_t threads = (S + kAliasPerThread - 1) / kAliasPerThread;
    const uint64_t blocks = (threads + kSampleThreads - 1) / kSampleThreads;
    if (blocks == 0) return cudaSuccess;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    const dim3 grid(static_cast<unsigned>(blocks));
    const uint8_t* c = coop || !coin_sum ? nullptr : coins;  // cooperative: the table alone
    if (rng == RNG_REF) {
        if (coop)
            launch_pdl(k_alias_sample<RNG_REF, true, false>, grid, kSampleThreads, 0, st, table, c, coin_sum, n, S, seed, offset, coop, out);
        else if (c)
            launch_pdl(k_alias_sample<RNG_REF, false, true>, grid, kSampleThreads, 0, st, table, c, coin_sum, n, S, seed, offset, coop, out);
        else
            launch_pdl(k_alias_sample<RNG_REF, false, false>, grid, kSampleThreads, 0, st, table, c, coin_sum, n, S, seed, offset, coop, out);
    } else if (c) {
        launch_pdl(k_alias_sample<RNG_PHILOX, false, true>, grid, kSampleThreads, 0, st, table, c, coin_sum, n, S, seed, offset, coop, out);
    } else {
        launch_pdl(k_alias_sample<RNG_PHILOX, false, false>, grid, kSampleThreads, 0, st, table, c, coin_sum, n, S, seed, offset, coop, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_coin_filter(cudaStream_t st, const uint2* table, uint32_t n, uint8_t* coins,
                               unsigned long long* coin_sum) {
    const uint64_t groups = (static_cast<uint64_t>(n) + 3u) / 4u;
    const uint64_t blocks = (groups + kSampleThreads - 1) / kSampleThreads;
    if (blocks == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(coin_sum, 0, sizeof(*coin_sum), st);
    if (e != cudaSuccess) return e;
    // a few CTAs per SM, striding over the table: one atomic per CTA
    const unsigned grid = static_cast<unsigned>(blocks < 8u * 152u ? blocks : 8u * 152u);
    launch_pdl(k_coin_filter, grid, kSampleThreads, 0, st, table, n, coins, coin_sum);
    return cudaGetLastError();
}

cudaError_t launch_batch_alias_sample(cudaStream_t st, uint32_t rng, uint32_t coop,
                                      const BatchView& b) {
    if (b.sample_blocks == 0) return cudaSuccess;
    if (rng == RNG_REF) {
        if (coop)
            launch_pdl(k_alias_sample_batch<RNG_REF, true>, b.sample_blocks, kSampleThreads, 0, st, b, coop);
        else
            launch_pdl(k_alias_sample_batch<RNG_REF, false>, b.sample_blocks, kSampleThreads, 0, st, b, 0u);
    } else {
        launch_pdl(k_alias_sample_batch<RNG_PHILOX, false>, b.sample_blocks, kSampleThreads, 0, st, b, 0u);
    }
    return cudaGetLastError();
}

cudaError_t launch_its_tree(cudaStream_t st, const float* cmf, uint32_t n, uint32_t L,
                            TreeBlock* blocks) {
    const size_t count = its_tree_blocks(L);
    if (count == 0) return cudaSuccess;
    const size_t grid = (count + kSampleThreads - 1) / kSampleThreads;
    if (grid > 0x7fffffffull) return cudaErrorInvalidValue;
    launch_pdl(k_its_tree, static_cast<unsigned>(grid), kSampleThreads, 0, st, cmf, n, L, blocks);
    return cudaGetLastError();
}

cudaError_t launch_its_sample(cudaStream_t st, uint32_t rng, uint32_t coop, bool parray,
                              const float* cmf, uint32_t n, uint64_t S, uint64_t seed,
                              uint64_t offset, uint32_t* out, const TreeBlock* tree,
                              uint32_t B) {
    const uint64_t blocks = (S + kSampleThreads - 1) / kSampleThreads;
    if (blocks == 0) return cudaSuccess;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    const dim3 grid(static_cast<unsigned>(blocks));
    if (coop == 0) {
        const uint64_t groups = (S + kItsGroup - 1) / kItsGroup;
        const unsigned tb = static_cast<unsigned>(groups < kItsMaxBlocks ? groups : kItsMaxBlocks);
        if (rng == RNG_REF)
            launch_pdl(k_its_sample_tree<RNG_REF>, tb, kSampleThreads, 0, st, cmf, n, S, seed, offset, out,
                                                                      tree, B);
        else
            launch_pdl(k_its_sample_tree<RNG_PHILOX>, tb, kSampleThreads, 0, st, cmf, n, S, seed, offset,
                                                                         out, tree, B);
    } else if (parray) {
        launch_pdl(k_its_sample<RNG_REF, 2>, grid, kSampleThreads, 0, st, cmf, n, S, seed, offset, coop, out);
    } else {
        launch_pdl(k_its_sample<RNG_REF, 1>, grid, kSampleThreads, 0, st, cmf, n, S, seed, offset, coop, out);
    }
    return cudaGetLastError();
}

}  // namespace wrs

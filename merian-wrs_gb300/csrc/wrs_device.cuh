// wrs_device.cuh -- device-side building blocks shared by the WRS kernels (sm_103a).
//
//  * float-float ("compensated") arithmetic for the carries of the decoupled lookback;
//  * self-validating 64-bit lookback words (every word carries its own ready bit, so
//    readers never see a torn state and writers need no fences);
//  * the counter-based generators: the reference shaders' Philox2x32-7 variant and
//    wang_hash (bit-exact restatements), and Random123 Philox4x32-10;
//  * bounded spin helpers: every wait in this library gives up after a fixed budget
//    and raises a status bit instead of hanging the GPU.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace wrs {

// bits of the per-build device status word
constexpr uint32_t kStatusTimeout = 1u;      // a lookback spin exhausted its budget
constexpr uint32_t kStatusNonMonotone = 2u;  // split k+1 < split k (overlapping subproblems)

constexpr uint32_t kSpinLimit = 1u << 21;  // lookback polls before giving up (>= ~1 s)
// mbarrier tries a CTA spends on its own bulk copy after the first kSpinLimit ran out: the copy's
// completion depends on no other CTA, so this only bounds a wait that ends in practice; the CTA
// leaves before the copy lands only after both budgets
constexpr uint32_t kCopyDrainLimit = 1u << 25;

// Programmatic dependent launch.  A kernel launched with programmatic stream serialization
// (launch_pdl) may be scheduled while the kernel before it in the stream still runs: its CTAs
// wait here until that kernel has completed and its memory is visible, so the launch and the
// CTAs' start overlap the predecessor's tail instead of following it.  The kernel then lets its
// own dependent be scheduled.  For an ordinary launch both instructions do nothing.
__device__ __forceinline__ void pdl_entry() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---------------------------------------------------------------------------
// float-float arithmetic (Knuth two-sum); every operation rounds once.
// ---------------------------------------------------------------------------
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bp = __fsub_rn(s, a);
    float ap = __fsub_rn(s, bp);
    float e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
    return {s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

template <bool COMP>
__device__ __forceinline__ ff carry_add(ff a, ff b) {
    if constexpr (COMP) {
        ff s = two_sum(a.hi, b.hi);
        float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
        return fast_two_sum(s.hi, e);
    } else {
        return {__fadd_rn(a.hi, b.hi), 0.0f};
    }
}

// round(carry + x) to FP32
template <bool COMP>
__device__ __forceinline__ float carry_apply(ff c, float x) {
    if constexpr (COMP) {
        ff s = two_sum(c.hi, x);
        return __fadd_rn(s.hi, __fadd_rn(s.lo, c.lo));
    } else {
        return __fadd_rn(c.hi, x);
    }
}

__device__ __forceinline__ ff shfl_xor_ff(ff v, int m) {
    return {__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
}

// float-float accumulation of one FP32 value
__device__ __forceinline__ ff ff_add_f(ff a, float x) {
    ff s = two_sum(a.hi, x);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ __forceinline__ ff ff_shfl(ff v, int src) {
    return {__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

// inclusive float-float scan over the lanes of a warp
__device__ __forceinline__ ff ff_warp_incl(ff v, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const ff o{__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d)};
        if (lane >= d) v = carry_add<true>(o, v);
    }
    return v;
}

// exclusive value from an inclusive scan (lane 0 gets zero)
__device__ __forceinline__ ff ff_shfl_up_excl(ff incl, int lane) {
    const ff o{__shfl_up_sync(0xffffffffu, incl.hi, 1), __shfl_up_sync(0xffffffffu, incl.lo, 1)};
    return lane ? o : ff{0.f, 0.f};
}

// float-float sum over the warp (butterfly; every lane gets the same value)
__device__ __forceinline__ ff ff_warp_total(ff v) {
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) v = carry_add<true>(v, shfl_xor_ff(v, m));
    return v;
}

// ---------------------------------------------------------------------------
// Exact fixed-point carries.  A distribution's heavy/light sums are carried through
// the lookback as unsigned integers k on the grid 2^g, g = E - 123 where the FP64
// total mass lies in [2^(E-1), 2^E): every weight is at most 2^123 grid units and
// every sum stays below 2^125.  Integer addition is associative, so a tile's carry
// does not depend on which predecessors the lookback happened to see (the FP32 and
// float-float carries do): builds are bit-for-bit reproducible, alone or batched.
// A weight converts to the grid by truncation (exact for weights above 2^(E-100)).
// ---------------------------------------------------------------------------
typedef unsigned __int128 u128;

__device__ __forceinline__ int fx_grid(double total) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(total));
    const int e = static_cast<int>((b >> 52) & 0x7ffu);
    if (e == 0) return -149 - 24;    // zero total: every weight is zero
    if (e == 0x7ff) return 0;        // not finite: results are meaningless, stay defined
    return (e - 1022) - 123;
}

__device__ __forceinline__ u128 fx_from_float(float x, int g) {
    const uint32_t b = __float_as_uint(x);
    const int e = static_cast<int>((b >> 23) & 0xffu);
    uint32_t m = b & 0x7fffffu;
    int ex = -149;
    if (e) {
        m |= 0x800000u;
        ex = e - 150;
    }
    int sh = ex - g;
    if (sh >= 0) return static_cast<u128>(m) << (sh < 103 ? sh : 103);
    sh = -sh;
    return sh >= 24 ? static_cast<u128>(0) : static_cast<u128>(m >> sh);
}

// A float-float value hi + lo (hi >= 0, |lo| <= ulp(hi) / 2) on the grid; lo may be negative,
// so its part enters in two's complement and the sum is again non-negative.
__device__ __forceinline__ u128 fx_from_ff(ff v, int g) {
    const u128 lo = fx_from_float(v.lo, g);  // magnitude (the sign bit is ignored)
    return fx_from_float(v.hi, g) + (v.lo < 0.0f ? static_cast<u128>(0) - lo : lo);
}

__device__ __forceinline__ u128 shfl_xor_u128(u128 v, int m) {
    const unsigned long long lo = __shfl_xor_sync(0xffffffffu, static_cast<unsigned long long>(v), m);
    const unsigned long long hi =
        __shfl_xor_sync(0xffffffffu, static_cast<unsigned long long>(v >> 64), m);
    return (static_cast<u128>(hi) << 64) | lo;
}

// k > 0 rounded to nearest FP32, as the float f = RN(top) with top the leading 64 bits of
// k (a sticky bit folded into bit 0) and the bit length nb of k: value = f * 2^(nb - 64).
__device__ __forceinline__ float fx_lead(u128 k, int& nb) {
    const unsigned long long hi = static_cast<unsigned long long>(k >> 64);
    const unsigned long long lo = static_cast<unsigned long long>(k);
    const int lz = hi ? __clzll(static_cast<long long>(hi)) : 64 + __clzll(static_cast<long long>(lo));
    nb = 128 - lz;
    const u128 norm = k << lz;
    const unsigned long long top = static_cast<unsigned long long>(norm >> 64) |
                                   (static_cast<unsigned long long>(norm) != 0ull ? 1ull : 0ull);
    return __ull2float_rn(top);
}

// The grid value f * 2^(nb - 64) of fx_lead as an integer (f has at most 24 significant
// bits, and is a multiple of 2^40 when nb > 24, so the shifts below are exact).
__device__ __forceinline__ u128 fx_lead_int(float f, int nb) {
    if (f >= 18446744073709551616.0f) return static_cast<u128>(1) << nb;  // rounded up to 2^64
    const unsigned long long fi = __float2ull_rn(f);
    return nb >= 64 ? static_cast<u128>(fi) << (nb - 64) : static_cast<u128>(fi >> (64 - nb));
}

// f * 2^e for the f of fx_lead (2^63 <= f <= 2^64): an exact power-of-two product where the
// result is normal, ldexpf otherwise.
__device__ __forceinline__ float fx_scale(float f, int e) {
    return (e >= -126 && e <= 127) ? __fmul_rn(f, __int_as_float((e + 127) << 23)) : ldexpf(f, e);
}

// k * 2^g rounded to nearest FP32.
__device__ __forceinline__ float fx_round(u128 k, int g) {
    if (k == 0) return 0.0f;
    int nb;
    const float f = fx_lead(k, nb);
    return fx_scale(f, nb - 64 + g);
}

// k * 2^g as a float-float pair: hi = RN(k * 2^g), lo = RN((k - hi) * 2^g).  Deterministic
// (a function of k and g only).
__device__ __forceinline__ ff fx_to_ff(u128 k, int g) {
    if (k == 0) return {0.0f, 0.0f};
    int nb;
    const float f = fx_lead(k, nb);
    const u128 kh = fx_lead_int(f, nb);
    const float hi = fx_scale(f, nb - 64 + g);
    float lo = 0.0f;
    if (kh != k) {
        const bool neg = kh > k;
        const u128 r = neg ? kh - k : k - kh;
        int nr;
        const float fr = fx_lead(r, nr);
        lo = fx_scale(neg ? -fr : fr, nr - 64 + g);
    }
    return {hi, lo};
}

// Lookback words of a fixed-point value (k < 2^126): two 63-bit limbs, bit 63 of each word
// is its ready bit.
constexpr unsigned long long kLimbMask = 0x7fffffffffffffffull;
constexpr unsigned long long kLimbReady = 0x8000000000000000ull;
__device__ __forceinline__ unsigned long long fx_word_lo(u128 k) {
    return (static_cast<unsigned long long>(k) & kLimbMask) | kLimbReady;
}
__device__ __forceinline__ unsigned long long fx_word_hi(u128 k) {
    return (static_cast<unsigned long long>(k >> 63) & kLimbMask) | kLimbReady;
}
__device__ __forceinline__ bool fx_ready(unsigned long long lo, unsigned long long hi) {
    return (lo & hi & kLimbReady) != 0ull;
}
__device__ __forceinline__ u128 fx_unpack(unsigned long long lo, unsigned long long hi) {
    return (static_cast<u128>(hi & kLimbMask) << 63) | (lo & kLimbMask);
}

// ---------------------------------------------------------------------------
// lookback words.  An ff word is {hi bits, lo bits | 1}: the LSB of lo's
// mantissa is the ready bit (the value loses at most one ulp of lo).  A count
// word is {count, 1}.  State buffers are zero when a build starts.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long pack_ff(ff v) {
    uint32_t hi = __float_as_uint(v.hi);
    uint32_t lo = __float_as_uint(v.lo) | 1u;
    return (static_cast<unsigned long long>(lo) << 32) | hi;
}
__device__ __forceinline__ bool ff_ready(unsigned long long w) { return (w >> 32) & 1ull; }
__device__ __forceinline__ ff unpack_ff(unsigned long long w) {
    return {__uint_as_float(static_cast<uint32_t>(w)),
            __uint_as_float(static_cast<uint32_t>(w >> 32) & ~1u)};
}
__device__ __forceinline__ unsigned long long pack_cnt(uint32_t c) {
    return (1ull << 32) | c;
}
__device__ __forceinline__ bool cnt_ready(unsigned long long w) { return (w >> 32) != 0; }

__device__ __forceinline__ void st_relaxed_v2(unsigned long long* p, unsigned long long a,
                                              unsigned long long b) {
    asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b)
                 : "memory");
}
__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long a) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(a) : "memory");
}
__device__ __forceinline__ void ld_relaxed_v2(const unsigned long long* p, unsigned long long& a,
                                              unsigned long long& b) {
    asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];"
                 : "=l"(a), "=l"(b)
                 : "l"(p)
                 : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// exponential back-off for spin loops (bounded: 32 ns .. 1 us)
__device__ __forceinline__ void backoff(uint32_t spins) {
    uint32_t ns = 32u << (spins < 5 ? spins : 5);
    __nanosleep(ns);
}

// ---------------------------------------------------------------------------
// generators
// ---------------------------------------------------------------------------

// src/device/wrs/alias/sampling/shader.comp:39-54 -- 7 rounds of
//   (hi,lo) = mulExtended(x0, 0xD256D193); x0 = x1 ^ hi; x1 = lo + k; k += 0x9E3779B9
__device__ __forceinline__ uint2 philox2x32_7(uint32_t x0, uint32_t x1, uint32_t key) {
    uint32_t k = key;
#pragma unroll
    for (int r = 0; r < 7; ++r) {
        uint32_t hi = __umulhi(x0, 0xD256D193u);
        uint32_t lo = x0 * 0xD256D193u;
        x0 = x1 ^ hi;
        x1 = lo + k;
        k += 0x9E3779B9u;
    }
    return make_uint2(x0, x1);
}

// Random123 Philox4x32-10 (Salmon et al., SC'11).  The key schedule is hoisted by
// the caller: ks[r] = key + r * (0x9E3779B9, 0xBB67AE85).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, const uint2* ks) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ ks[r].x, lo1, hi0 ^ c.w ^ ks[r].y, lo0);
    }
    return c;
}

__device__ __forceinline__ void philox4x32_10_keys(uint64_t seed, uint2* ks) {
    uint32_t k0 = static_cast<uint32_t>(seed), k1 = static_cast<uint32_t>(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        ks[r] = make_uint2(k0, k1);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// src/device/wrs/its/sampling/shader.comp:70-78 (bits before the division by 2^32)
__device__ __forceinline__ uint32_t wang_hash(uint32_t seed) {
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    return seed;
}

// float(x) / 4294967296.0 with a round-to-nearest conversion (the division is exact)
__device__ __forceinline__ float unit_ref(uint32_t x) {
    return __fmul_rn(__uint2float_rn(x), 2.3283064365386963e-10f);
}

// ---------------------------------------------------------------------------
// memory helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint2 ld_entry(const uint2* p) {
    uint2 v;
    asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];"
                 : "=r"(v.x), "=r"(v.y)
                 : "l"(p));
    return v;
}
// ld_entry carrying an L2 eviction policy (createpolicy)
__device__ __forceinline__ uint2 ld_entry_policy(const uint2* p, uint64_t pol) {
    uint2 v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
                 : "=r"(v.x), "=r"(v.y)
                 : "l"(p), "l"(pol));
    return v;
}

// An L2 eviction policy (createpolicy) and read-only loads that carry it: data read once at
// random (a large CMF, the ITS cell blocks) is marked evict-first.
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ float ld_f32_policy(const float* p, uint64_t pol) {
    float v;
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}
// 32 bytes in one request (256-bit load, sm_100 and later); p 32-byte aligned
__device__ __forceinline__ void ld_u32x8_policy(const uint32_t* p, uint64_t pol, uint4& a,
                                                uint4& b) {
    asm volatile("ld.global.nc.L2::cache_hint.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8], %9;"
                 : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z),
                   "=r"(b.w)
                 : "l"(p), "l"(pol));
}
// ---- bulk copies global -> shared (the TMA unit's cp.async.bulk) completing on mbarriers ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}
// makes initialised mbarriers visible to the async proxy (the bulk copies)
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// bytes (a multiple of 16) from src to dst (both 16-byte aligned); the mbarrier's transaction
// count drops by bytes when they have landed
__device__ __forceinline__ void bulk_load_smem(void* dst, const void* src, uint32_t bytes,
                                               uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}
// waits for the phase of `parity` to complete, at most `limit` tries (each try suspends the
// thread for a bounded, implementation-defined time); false if it gave up
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t k = 0; k < limit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 32 bytes in one request without an L2 policy; p 32-byte aligned
__device__ __forceinline__ void ld_u32x8(const uint32_t* p, uint4& a, uint4& b) {
    asm volatile("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z),
                   "=r"(b.w)
                 : "l"(p));
}

}  // namespace wrs

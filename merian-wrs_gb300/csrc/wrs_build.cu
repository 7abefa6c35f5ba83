// wrs_build.cu -- build kernels of the WRS hot path for sm_103a.
//
//   k_total_mass        total mass / mean                 (reference: src/device/mean/atomic/shader.comp)
//   k_prefix_partition  fused heavy/light stable partition + heavy and light inclusive
//                       prefix sums + heavyCount, single pass with decoupled lookback
//                                                          (src/device/prefix_partition/decoupled/shader.comp)
//   k_scan_bulk         inclusive FP32 scan, single pass, tiles brought in by bulk copies
//                                                          (src/device/prefix_sum/decoupled/shader.comp)
//   k_scan_exact        the compensated form: exact fixed-point carries, correctly rounded
//                       outputs (after k_total_mass, which sets the grid)
//   k_split_pack        PSA split search + pack, one thread per split
//                                                          (src/device/wrs/alias/psa/splitpack/inline/shader.comp)
//
// The total-mass, partition and split+pack kernels come in two forms from one body: a
// single distribution (BATCH = false; CTA b works on tile / split block b), and a batch
// of distributions of any sizes in one launch (BATCH = true; a per-CTA map names the
// distribution, whose tiles and split blocks are numbered from its first one).  A
// distribution's results do not depend on the form or on the other distributions.
//
// All lookback kernels take their tile index from an atomic ticket (a tile only ever
// waits for tiles whose CTAs already run; a batch's distributions occupy consecutive
// ticket ranges), bound every spin (kSpinLimit polls, then raise kStatusTimeout and
// continue), and clean up after themselves: the state buffer is double-buffered by an
// epoch; each launch clears the half the next launch will use, and its last CTA resets
// the ticket and advances the epoch.
#include "wrs_device.cuh"
#include "wrs_internal.cuh"

namespace wrs {

// ---------------------------------------------------------------------------------
// tile loads
// ---------------------------------------------------------------------------------

// Items of local tile `lt` held by this thread: x[v][c] = item lt*4096 + warp*512 + v*128 +
// lane*4 + c (16-byte loads, fully coalesced, where the tile is whole and aligned); items
// past n read as 0.
__device__ __forceinline__ void load_tile(const float* __restrict__ w, uint32_t n, uint32_t lt,
                                          float (&x)[4][4]) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tbase = lt * kTileItems;
    const uint32_t wbase = tbase + warp * kWarpItems;
    const bool full = (static_cast<uint64_t>(tbase) + kTileItems <= n) &&
                      ((reinterpret_cast<uintptr_t>(w) & 15u) == 0);
    if (full) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            float4 q = __ldcs(reinterpret_cast<const float4*>(w + wbase + v * 128 + lane * 4));
            x[v][0] = q.x;
            x[v][1] = q.y;
            x[v][2] = q.z;
            x[v][3] = q.w;
        }
    } else {
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                uint32_t e = wbase + v * 128 + lane * 4 + c;
                x[v][c] = e < n ? __ldg(w + e) : 0.0f;
            }
    }
}

// Resident partition CTAs per SM the register allocation is sized for (5 x 256 threads:
// at most 51 registers per thread).
#ifndef WRS_PART_MIN_BLOCKS
#define WRS_PART_MIN_BLOCKS 5
#endif
constexpr int kPartMinBlocks = WRS_PART_MIN_BLOCKS;

// staged-output array index of output slot q: one padding word per 32 spreads the scattered
// stores of a warp over the banks; consecutive slots stay conflict-free for the write-out
constexpr int kStageWords = kTileItems + kTileItems / 32;
__device__ __forceinline__ uint32_t stage_idx(uint32_t q) { return q + (q >> 5); }

// float4 slot of chunk q (items 4q..4q+3) of a tile parked in shared memory: the XOR
// swizzle spreads both the coalesced order (q = 32v + lane per warp) and the transposed order
// (q = 4 lane + j) over all eight 16-byte bank groups (4 wavefronts per warp access).
__device__ __forceinline__ uint32_t park_slot(uint32_t q) { return q ^ ((q >> 3) & 7u); }

// ---------------------------------------------------------------------------------
// total mass
// ---------------------------------------------------------------------------------

// One CTA per 4096-item tile.  Each thread sums its 16 items in a fixed order with a
// compensated FP32 accumulator (two-sum), the CTA combines its threads in float-float in a
// fixed tree (FP32 arithmetic: GB300's FP64 pipe is narrow), the tile partial hi + lo is
// stored in FP64, and the last tile of the distribution to finish sums the partials in FP64
// in a fixed order.  The total is therefore a function of the weights alone (not of the
// launch geometry, of the buffer's alignment or of other distributions in a batch).
template <bool BATCH>
__global__ __launch_bounds__(kTileThreads) void k_total_mass(const float* __restrict__ w_in,
                                                             uint32_t n_in,
                                                             double* __restrict__ partials,
                                                             BuildCtrl* __restrict__ ctrl_in,
                                                             BatchView bv) {
    pdl_entry();
    __shared__ double s_red[kTileWarps];
    __shared__ ff s_part[kTileWarps];
    __shared__ bool s_last;
    const uint32_t tile = blockIdx.x;
    const float* w = w_in;
    uint32_t n = n_in, first = 0;
    BuildCtrl* ctrl = ctrl_in;
    if constexpr (BATCH) {
        const uint32_t d = __ldg(bv.tile_map + tile);
        const DistDesc* D = bv.dist + d;
        w = D->w;
        n = D->n;
        first = D->tile0;
        ctrl = bv.dctrl + d;
    }
    const uint32_t lt = tile - first, ntiles = tiles_for(n);
    float x[4][4];
    load_tile(w, n, lt, x);
    ff acc = {0.0f, 0.0f};
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc = carry_add<true>(acc, ff{x[v][c], 0.0f});

    acc = ff_warp_total(acc);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) s_part[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        ff b = s_part[0];
        for (int k = 1; k < kTileWarps; ++k) b = carry_add<true>(b, s_part[k]);
        partials[tile] = __dadd_rn(static_cast<double>(b.hi), static_cast<double>(b.lo));
        __threadfence();
        const uint32_t prev = atomicAdd(&ctrl->mass_done, 1u);
        s_last = (prev == ntiles - 1u);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double t = 0.0;
    for (uint32_t k = threadIdx.x; k < ntiles; k += blockDim.x)
        t = __dadd_rn(t, __ldcg(partials + first + k));
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) t = __dadd_rn(t, __shfl_xor_sync(0xffffffffu, t, m));
    __syncthreads();
    if (lane == 0) s_red[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0.0;
        for (int k = 0; k < kTileWarps; ++k) total = __dadd_rn(total, s_red[k]);
        ctrl->total = total;
        const double m64 = n ? __ddiv_rn(total, static_cast<double>(n)) : 0.0;
        const float m = __double2float_rn(m64);
        ctrl->mean64 = m64;
        ctrl->mean = m;
        ctrl->mean_lo = __double2float_rn(__dsub_rn(m64, static_cast<double>(m)));
        ctrl->mass_done = 0u;
    }
}

cudaError_t launch_total_mass(cudaStream_t st, const float* w, uint32_t n, double* partials,
                              BuildCtrl* ctrl) {
    launch_pdl(k_total_mass<false>, tiles_for(n), kTileThreads, 0, st, w, n, partials, ctrl, BatchView{});
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// shared pieces of the lookback kernels
// ---------------------------------------------------------------------------------

__device__ __forceinline__ float warp_incl_f(float v, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        float o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v = __fadd_rn(v, o);
    }
    return v;
}
__device__ __forceinline__ uint32_t warp_incl_u(uint32_t v, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    return v;
}

// Ticket, epoch and clearing of the other state half.  Returns the tile index.
template <class State>
__device__ __forceinline__ uint32_t lookback_begin(LbCtrl* ctrl, State* states,
                                                   uint32_t cap_tiles, State*& cur) {
    __shared__ uint32_t s_tile, s_epoch;
    if (threadIdx.x == 0) {
        s_tile = atomicAdd(&ctrl->ticket, 1u);
        s_epoch = ld_relaxed_u32(&ctrl->epoch);
    }
    __syncthreads();
    const uint32_t tile = s_tile, epoch = s_epoch;
    cur = states + static_cast<size_t>(epoch & 1u) * cap_tiles;
    State* other = states + static_cast<size_t>((epoch + 1u) & 1u) * cap_tiles;
    // the other half was last used by the previous launch (finished, stream order) and is
    // next used by the following launch: clear the entries this launch is responsible for
    constexpr int kWords = sizeof(State) / 16;
    for (uint32_t t = tile; t < cap_tiles; t += gridDim.x) {
        if (threadIdx.x < kWords)
            reinterpret_cast<ulonglong2*>(other + t)[threadIdx.x] = make_ulonglong2(0ull, 0ull);
    }
    return tile;
}

__device__ __forceinline__ void lookback_end(LbCtrl* ctrl) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        uint32_t prev = atomicAdd(&ctrl->done, 1u);
        if (prev == gridDim.x - 1) {
            ctrl->ticket = 0u;
            ctrl->done = 0u;
            ctrl->epoch = ctrl->epoch + 1u;
            __threadfence();
        }
    }
}

// Decoupled-lookback window walk shared by the partition and scan lookbacks.  `probe(pos,
// v)` reads tile pos's state into v and returns 2 (inclusive prefix), 1 (aggregate only) or
// 0 (not yet published); `sum(v, take)` returns the warp total of v over lanes < take;
// `acc(ex, v)` adds.  Tiles before `first` count as published zeros.  Runs on one warp; the
// result is valid in every lane.
template <class V, class Probe, class Sum, class Acc>
__device__ __forceinline__ V lookback_walk(uint32_t tile, uint32_t first, uint32_t* status,
                                           uint32_t spin_limit, V zero, Probe probe, Sum sum,
                                           Acc acc) {
    const int lane = threadIdx.x & 31;
    V ex = zero;
    int64_t base = static_cast<int64_t>(tile) - 1;
    uint32_t spins = 0;
    for (;;) {
        const int64_t pos = base - lane;
        int s = 2;
        V v = zero;
        if (pos >= static_cast<int64_t>(first)) s = probe(static_cast<uint32_t>(pos), v);
        const unsigned nr = __ballot_sync(0xffffffffu, s == 0);
        const unsigned dn = __ballot_sync(0xffffffffu, s == 2);
        const int first_nr = nr ? __ffs(nr) - 1 : 32;
        const int first_dn = dn ? __ffs(dn) - 1 : 32;
        const bool finish = first_dn < first_nr;
        const int take = finish ? first_dn + 1 : first_nr;
        if (take > 0) {
            ex = acc(ex, sum(lane < take ? v : zero));
            base -= take;
            spins = 0;
        }
        if (finish) break;
        if (take == 0) {
            if (++spins >= spin_limit) {
                if (lane == 0) atomicOr(status, kStatusTimeout);
                break;
            }
            backoff(spins);
        }
    }
    return ex;
}

// ---------------------------------------------------------------------------------
// fused prefix-partition
// ---------------------------------------------------------------------------------

// FP32-mode carry (reference arithmetic; association depends on lookback timing)
struct PartCarry {
    float h, l;
    uint32_t c;
};
// exact carry of the compensated modes
struct PartX {
    u128 h, l;
    uint32_t c;
};

__device__ __forceinline__ PartCarry part_sum_f(PartCarry v) {
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
        v.h = __fadd_rn(v.h, __shfl_xor_sync(0xffffffffu, v.h, m));
        v.l = __fadd_rn(v.l, __shfl_xor_sync(0xffffffffu, v.l, m));
        v.c += __shfl_xor_sync(0xffffffffu, v.c, m);
    }
    return v;
}
__device__ __forceinline__ PartX part_sum_x(PartX v) {
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
        v.h += shfl_xor_u128(v.h, m);
        v.l += shfl_xor_u128(v.l, m);
        v.c += __shfl_xor_sync(0xffffffffu, v.c, m);
    }
    return v;
}

__device__ PartX part_lookback_x(const PartState* st, uint32_t tile, uint32_t first,
                                 uint32_t* status, uint32_t spin_limit) {
    const PartX zero{0, 0, 0u};
    return lookback_walk(
        tile, first, status, spin_limit, zero,
        [st](uint32_t pos, PartX& v) -> int {
            // inclusive words first; the aggregate only where those are not yet published
            const unsigned long long* q = st[pos].q;
            unsigned long long h0, h1, l0, l1, c, pad;
            ld_relaxed_v2(q + 8, h0, h1);
            ld_relaxed_v2(q + 10, l0, l1);
            ld_relaxed_v2(q + 6, c, pad);
            int s = 2;
            if (!(fx_ready(h0, h1) && fx_ready(l0, l1) && cnt_ready(c))) {
                ld_relaxed_v2(q + 0, h0, h1);
                ld_relaxed_v2(q + 2, l0, l1);
                ld_relaxed_v2(q + 4, c, pad);
                s = fx_ready(h0, h1) && fx_ready(l0, l1) && cnt_ready(c) ? 1 : 0;
            }
            if (s) v = {fx_unpack(h0, h1), fx_unpack(l0, l1), static_cast<uint32_t>(c)};
            return s;
        },
        [](PartX v) { return part_sum_x(v); },
        [](PartX a, PartX b) { return PartX{a.h + b.h, a.l + b.l, a.c + b.c}; });
}

__device__ PartCarry part_lookback_f(const PartState* st, uint32_t tile, uint32_t first,
                                     uint32_t* status, uint32_t spin_limit) {
    const PartCarry zero{0.f, 0.f, 0u};
    return lookback_walk(
        tile, first, status, spin_limit, zero,
        [st](uint32_t pos, PartCarry& v) -> int {
            const unsigned long long* q = st[pos].q;
            unsigned long long h, l, c, pad;
            ld_relaxed_v2(q + 8, h, l);
            ld_relaxed_v2(q + 6, c, pad);
            int s = 2;
            if (!(ff_ready(h) && ff_ready(l) && cnt_ready(c))) {
                ld_relaxed_v2(q + 0, h, l);
                ld_relaxed_v2(q + 4, c, pad);
                s = ff_ready(h) && ff_ready(l) && cnt_ready(c) ? 1 : 0;
            }
            if (s) v = {unpack_ff(h).hi, unpack_ff(l).hi, static_cast<uint32_t>(c)};
            return s;
        },
        [](PartCarry v) { return part_sum_f(v); },
        [](PartCarry a, PartCarry b) {
            return PartCarry{__fadd_rn(a.h, b.h), __fadd_rn(a.l, b.l), a.c + b.c};
        });
}

__device__ __forceinline__ void part_publish_x(PartState* s, const PartX& a, bool incl) {
    unsigned long long* q = s->q + (incl ? 8 : 0);
    st_relaxed_v2(q + 0, fx_word_lo(a.h), fx_word_hi(a.h));
    st_relaxed_v2(q + 2, fx_word_lo(a.l), fx_word_hi(a.l));
    st_relaxed(s->q + (incl ? 6 : 4), pack_cnt(a.c));
}
__device__ __forceinline__ void part_publish_f(PartState* s, const PartCarry& a, bool incl) {
    st_relaxed_v2(s->q + (incl ? 8 : 0), pack_ff(ff{a.h, 0.f}), pack_ff(ff{a.l, 0.f}));
    st_relaxed(s->q + (incl ? 6 : 4), pack_cnt(a.c));
}

struct PartArgs {
    const float* w;  // single distribution: weights, n, control block
    uint32_t n;
    BuildCtrl* ctrl;
    LbCtrl* lb;
    PartState* states;
    uint32_t cap_tiles;
    uint32_t spin_limit;
    uint32_t* status;
    uint32_t* idx;  // outputs (a batch adds each distribution's base)
    float* prefix;
    float* elems;
    float* prefix_lo;
    // block-wise baseline: exclusive per-tile offsets (heavy count, heavy sum, light sum)
    // precomputed by k_bw_part_reduce + k_bw_tiles instead of the lookback
    const uint32_t* bw_c;
    const float* bw_h;
    const float* bw_l;
};

// One CTA = one tile of 4096 weights.  The tile is loaded with 16-byte coalesced loads and
// parked in shared memory; thread t of warp w then works on the 16 consecutive items
// [w*512 + 16t, +16), so a single warp scan per class gives every thread its offsets.
// Heavy (w > mean) items go to idx[heavyRank], light items to idx[N-1-lightRank]; prefix[]
// holds the inclusive heavy resp. light prefix sum, elems[] the weight
// (shader.comp:329-361).
//
// COMP (compensated modes): the tile aggregates (FP32, or float-float with FFOUT) are summed
// along the lookback exactly in fixed point (fx_*) and the carry is rounded once to a
// float-float pair per tile; sums within a tile run in a fixed order.  Every prefix is then a
// deterministic function of the weights.  FFOUT also writes prefix_lo[], the low word of the
// prefix as a float-float pair (prefix[] is its high word): float-float local sums give the
// carried prefix before each thread's first item, and the thread adds its items to that in
// float-float.
template <bool COMP, bool FFOUT, bool BATCH, bool BW = false>
__global__ __launch_bounds__(kTileThreads, kPartMinBlocks) void k_prefix_partition(PartArgs a,
                                                                                   BatchView bv) {
    pdl_entry();
    // warp totals (phase A), turned into warp-exclusive offsets by warp 0 (phase B)
    __shared__ uint32_t s_wc[kTileWarps];
    __shared__ float s_wh[kTileWarps], s_wl[kTileWarps];  // local FP32 sums (!FFOUT)
    __shared__ ff s_fh[kTileWarps], s_fl[kTileWarps];     // local float-float sums (FFOUT)
    __shared__ ff s_exh, s_exl;
    __shared__ uint32_t s_exc, s_aggc;
    // the parked tile (swizzled, park_slot), then the staged outputs by output slot: the tile's
    // heavy items take slots [0, heavy) in order, its light items slots 4095, 4094, ... in order,
    // so both runs are written out as contiguous, coalesced segments (stage_idx pads 1 word per
    // 32).  Until phase C the staging area holds the lane-exclusive offsets of phase A.
    __shared__ __align__(16) unsigned char s_raw[kTileItems * 4 + kStageWords * 2 + kStageWords * 4];
    float4* const s_x = reinterpret_cast<float4*>(s_raw);
    uint16_t* const s_key = reinterpret_cast<uint16_t*>(s_raw + kTileItems * 4);
    float* const s_val = reinterpret_cast<float*>(s_raw + kTileItems * 4 + kStageWords * 2);
    uint32_t* const s_lc = reinterpret_cast<uint32_t*>(s_val);                 // lane-exclusive counts
    float2* const s_lh = reinterpret_cast<float2*>(s_val + kTileThreads);      // lane-exclusive sums
    float2* const s_ll = reinterpret_cast<float2*>(s_val + 3 * kTileThreads);

    PartState* cur = nullptr;
    const uint32_t tile = BW ? blockIdx.x : lookback_begin(a.lb, a.states, a.cap_tiles, cur);
    const float* w = a.w;
    uint32_t n = a.n, first = 0;
    BuildCtrl* ctrl = a.ctrl;
    const DistDesc* D = nullptr;
    if constexpr (BATCH) {
        D = bv.dist + __ldg(bv.tile_map + tile);
        w = D->w;
        n = D->n;
        first = D->tile0;
        ctrl = bv.dctrl + (D - bv.dist);
    }
    const uint32_t lt = tile - first;
    const float pivot = ctrl->mean;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    {
        float x[4][4];
        load_tile(w, n, lt, x);
#pragma unroll
        for (int v = 0; v < 4; ++v)
            s_x[park_slot(warp * 128 + v * 32 + lane)] = make_float4(x[v][0], x[v][1], x[v][2], x[v][3]);
    }
    __syncwarp();

    // ---- phase A: thread totals over 16 consecutive items, warp scans; the lane-exclusive
    // values wait in shared memory until phase C (registers stay free for the lookback)
    {
        float y[16];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 q = s_x[park_slot(warp * 128 + lane * 4 + j)];
            y[4 * j] = q.x;
            y[4 * j + 1] = q.y;
            y[4 * j + 2] = q.z;
            y[4 * j + 3] = q.w;
        }
        uint32_t tc = 0;
        float th = 0.f, tl = 0.f;
        ff fh{0.f, 0.f}, fl{0.f, 0.f};
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            if constexpr (FFOUT) {
                // one float-float add on the selected accumulator (the operations of adding to
                // it in a branch, without the two predicated paths)
                const bool hv = y[i] > pivot;
                tc += hv ? 1u : 0u;
                const ff acc = ff_add_f(hv ? fh : fl, y[i]);
                fh = hv ? acc : fh;
                fl = hv ? fl : acc;
            } else if (y[i] > pivot) {
                ++tc;
                th = __fadd_rn(th, y[i]);
            } else {
                tl = __fadd_rn(tl, y[i]);
            }
        }
        const uint32_t ic = warp_incl_u(tc, lane);
        s_lc[threadIdx.x] = ic - tc;
        uint32_t wtot_c = __shfl_sync(0xffffffffu, ic, 31);
        float wtot_h = 0.f, wtot_l = 0.f;
        ff wf_h{0.f, 0.f}, wf_l{0.f, 0.f};
        if constexpr (FFOUT) {
            const ff ih = ff_warp_incl(fh, lane), il = ff_warp_incl(fl, lane);
            const ff lh = ff_shfl_up_excl(ih, lane), ll = ff_shfl_up_excl(il, lane);
            s_lh[threadIdx.x] = make_float2(lh.hi, lh.lo);
            s_ll[threadIdx.x] = make_float2(ll.hi, ll.lo);
            wf_h = ff_shfl(ih, 31);
            wf_l = ff_shfl(il, 31);
        } else {
            const float ih = warp_incl_f(th, lane), il = warp_incl_f(tl, lane);
            const float eh = __shfl_up_sync(0xffffffffu, ih, 1);
            const float el = __shfl_up_sync(0xffffffffu, il, 1);
            s_lh[threadIdx.x] = make_float2(lane ? eh : 0.f, 0.f);
            s_ll[threadIdx.x] = make_float2(lane ? el : 0.f, 0.f);
            wtot_h = __shfl_sync(0xffffffffu, ih, 31);
            wtot_l = __shfl_sync(0xffffffffu, il, 31);
        }
        if (lane == 0) {
            s_wc[warp] = wtot_c;
            if constexpr (FFOUT) {
                s_fh[warp] = wf_h;
                s_fl[warp] = wf_l;
            } else {
                s_wh[warp] = wtot_h;
                s_wl[warp] = wtot_l;
            }
        }
    }
    __syncthreads();

    // ---- phase B (warp 0): warp-exclusive offsets, tile aggregate, lookback
    if (warp == 0) {
        const uint32_t ic = warp_incl_u(lane < kTileWarps ? s_wc[lane] : 0u, lane);
        const uint32_t ec = __shfl_up_sync(0xffffffffu, ic, 1);
        const uint32_t agg_c = __shfl_sync(0xffffffffu, ic, kTileWarps - 1);
        float eh = 0.f, el = 0.f;
        ff agg_h{0.f, 0.f}, agg_l{0.f, 0.f}, fxh{0.f, 0.f}, fxl{0.f, 0.f};
        if constexpr (FFOUT) {
            const ff ith = ff_warp_incl(lane < kTileWarps ? s_fh[lane] : ff{0.f, 0.f}, lane);
            const ff itl = ff_warp_incl(lane < kTileWarps ? s_fl[lane] : ff{0.f, 0.f}, lane);
            fxh = ff_shfl_up_excl(ith, lane);
            fxl = ff_shfl_up_excl(itl, lane);
            agg_h = ff_shfl(ith, kTileWarps - 1);
            agg_l = ff_shfl(itl, kTileWarps - 1);
        } else {
            const float ih = warp_incl_f(lane < kTileWarps ? s_wh[lane] : 0.f, lane);
            const float il = warp_incl_f(lane < kTileWarps ? s_wl[lane] : 0.f, lane);
            eh = __shfl_up_sync(0xffffffffu, ih, 1);
            el = __shfl_up_sync(0xffffffffu, il, 1);
            agg_h = {__shfl_sync(0xffffffffu, ih, kTileWarps - 1), 0.f};
            agg_l = {__shfl_sync(0xffffffffu, il, kTileWarps - 1), 0.f};
        }
        __syncwarp();
        if (lane < kTileWarps) {
            s_wc[lane] = lane ? ec : 0u;
            if constexpr (FFOUT) {
                s_fh[lane] = fxh;
                s_fl[lane] = fxl;
            } else {
                s_wh[lane] = lane ? eh : 0.f;
                s_wl[lane] = lane ? el : 0.f;
            }
        }
        ff exh{0.f, 0.f}, exl{0.f, 0.f};
        uint32_t exc = 0;
        if constexpr (BW) {
            exh = {__ldg(a.bw_h + tile), 0.f};
            exl = {__ldg(a.bw_l + tile), 0.f};
            exc = __ldg(a.bw_c + tile);
        } else if constexpr (COMP) {
            const int grid = fx_grid(ctrl->total);
            const PartX agg{fx_from_ff(agg_h, grid), fx_from_ff(agg_l, grid), agg_c};
            PartX ex{0, 0, 0u};
            if (tile == first) {
                if (lane == 0) {
                    part_publish_x(cur + tile, agg, false);
                    part_publish_x(cur + tile, agg, true);
                }
            } else {
                if (lane == 0) part_publish_x(cur + tile, agg, false);
                ex = part_lookback_x(cur, tile, first, a.status, a.spin_limit);
                if (lane == 0)
                    part_publish_x(cur + tile, PartX{ex.h + agg.h, ex.l + agg.l, ex.c + agg.c}, true);
            }
            if (lane == 0) {
                exh = fx_to_ff(ex.h, grid);
                exl = fx_to_ff(ex.l, grid);
            }
            exc = ex.c;
        } else {
            const PartCarry agg{agg_h.hi, agg_l.hi, agg_c};
            PartCarry ex{0.f, 0.f, 0u};
            if (tile == first) {
                if (lane == 0) {
                    part_publish_f(cur + tile, agg, false);
                    part_publish_f(cur + tile, agg, true);
                }
            } else {
                if (lane == 0) part_publish_f(cur + tile, agg, false);
                ex = part_lookback_f(cur, tile, first, a.status, a.spin_limit);
                if (lane == 0)
                    part_publish_f(cur + tile,
                                   PartCarry{__fadd_rn(ex.h, agg.h), __fadd_rn(ex.l, agg.l),
                                             ex.c + agg.c},
                                   true);
            }
            exh = {ex.h, 0.f};
            exl = {ex.l, 0.f};
            exc = ex.c;
        }
        if (lane == 0) {
            s_exh = exh;
            s_exl = exl;
            s_exc = exc;
            s_aggc = agg_c;
        }
    }
    __syncthreads();

    // ---- phase C: running sums over the thread's items, staged by output slot, written out
    const uint32_t tbase = lt * kTileItems;
    const uint32_t tloc = warp * kWarpItems + lane * 16;  // this thread's first item in the tile
    const ff ex_h = s_exh, ex_l = s_exl;
    const uint32_t ex_c = s_exc, agg_c = s_aggc;
    const uint32_t m = n - tbase < static_cast<uint32_t>(kTileItems) ? n - tbase : kTileItems;
    const uint32_t hc0 = s_wc[warp] + s_lc[threadIdx.x];  // heavy items of the tile before ours
    float rh32 = 0.f, rl32 = 0.f;
    ff rh0{0.f, 0.f}, rl0{0.f, 0.f};
    {
        const float2 lh = s_lh[threadIdx.x], ll = s_ll[threadIdx.x];
        if constexpr (FFOUT) {
            // the carried prefix before the thread's first item; the items are then added
            // to it one by one in float-float
            rh0 = carry_add<true>(ex_h, carry_add<true>(s_fh[warp], ff{lh.x, lh.y}));
            rl0 = carry_add<true>(ex_l, carry_add<true>(s_fl[warp], ff{ll.x, ll.y}));
        } else {
            rh32 = __fadd_rn(s_wh[warp], lh.x);
            rl32 = __fadd_rn(s_wl[warp], ll.x);
        }
    }
    __syncthreads();  // the lane offsets are read; the staging area is free
    // float-float: the low words of the first round's sums wait here for the second round
    float lo_keep[16];
    {
        uint32_t hc = hc0;
        ff rh = rh0, rl = rl0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 q = s_x[park_slot(warp * 128 + lane * 4 + j)];
            const float yv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint32_t local = tloc + 4 * j + c;
                lo_keep[4 * j + c] = 0.f;
                if (local < m) {
                    const float xv = yv[c];
                    uint32_t slot;
                    float hi;
                    if constexpr (FFOUT) {
                        // branch-free, as in phase A
                        const bool hv = xv > pivot;
                        slot = hv ? hc : kTileItems - 1u - (local - hc);
                        hc += hv ? 1u : 0u;
                        const ff acc = ff_add_f(hv ? rh : rl, xv);
                        rh = hv ? acc : rh;
                        rl = hv ? rl : acc;
                        hi = acc.hi;
                        lo_keep[4 * j + c] = acc.lo;
                    } else if (xv > pivot) {
                        slot = hc++;
                        rh32 = __fadd_rn(rh32, xv);
                        hi = carry_apply<COMP>(ex_h, rh32);
                    } else {
                        slot = kTileItems - 1u - (local - hc);
                        rl32 = __fadd_rn(rl32, xv);
                        hi = carry_apply<COMP>(ex_l, rl32);
                    }
                    s_key[stage_idx(slot)] = static_cast<uint16_t>(local);
                    s_val[stage_idx(slot)] = hi;
                }
            }
        }
    }
    __syncthreads();
    // write-out: slot q < agg_c -> heavy position ex_c + q; slot q >= 4096 - light -> light
    // rank 4095 - q at position n - 1 - (light items before the tile) - rank
    uint32_t* idx_out = a.idx;
    float* prefix_out = a.prefix;
    float* elems_out = a.elems;
    float* prefix_lo_out = a.prefix_lo;
    if constexpr (BATCH) {
        const uint64_t base = D->base;
        idx_out += base;
        prefix_out += base;
        if (elems_out) elems_out += base;
        if (prefix_lo_out) prefix_lo_out += base;
    }
    const uint32_t light_top = kTileItems - (m - agg_c);      // first light slot
    const uint32_t light_base = n - 1u - (tbase - ex_c) - (kTileItems - 1u);  // position of slot 0
    const float* s_xf = reinterpret_cast<const float*>(s_x);
    for (uint32_t q = threadIdx.x; q < static_cast<uint32_t>(kTileItems); q += kTileThreads) {
        const bool heavy = q < agg_c;
        if (!heavy && q < light_top) continue;
        const uint32_t pos = heavy ? ex_c + q : light_base + q;
        if (pos >= n) continue;  // only after a lookback wait gave up
        const uint32_t local = s_key[stage_idx(q)];
        idx_out[pos] = tbase + local;
        prefix_out[pos] = s_val[stage_idx(q)];
        if (elems_out) elems_out[pos] = s_xf[park_slot(local >> 2) * 4 + (local & 3)];
    }
    if constexpr (FFOUT) {
        // second round for the low words, kept in registers by the first round
        __syncthreads();
        uint32_t hc = hc0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 q = s_x[park_slot(warp * 128 + lane * 4 + j)];
            const float yv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint32_t local = tloc + 4 * j + c;
                if (local < m) {
                    const uint32_t slot = yv[c] > pivot ? hc++ : kTileItems - 1u - (local - hc);
                    s_val[stage_idx(slot)] = lo_keep[4 * j + c];
                }
            }
        }
        __syncthreads();
        for (uint32_t q = threadIdx.x; q < static_cast<uint32_t>(kTileItems); q += kTileThreads) {
            const bool heavy = q < agg_c;
            if (!heavy && q < light_top) continue;
            const uint32_t pos = heavy ? ex_c + q : light_base + q;
            if (pos >= n) continue;
            prefix_lo_out[pos] = s_val[stage_idx(q)];
        }
    }
    if (threadIdx.x == 0 && lt == tiles_for(n) - 1u) ctrl->heavy_count = ex_c + s_aggc;
    if constexpr (!BW) lookback_end(a.lb);
}

template <bool BATCH>
static void part_dispatch(cudaStream_t st, uint32_t precision, uint32_t grid, const PartArgs& a,
                          const BatchView& bv) {
    if (precision == 2)
        launch_pdl(k_prefix_partition<true, true, BATCH>, grid, kTileThreads, 0, st, a, bv);
    else if (precision == 1)
        launch_pdl(k_prefix_partition<true, false, BATCH>, grid, kTileThreads, 0, st, a, bv);
    else
        launch_pdl(k_prefix_partition<false, false, BATCH>, grid, kTileThreads, 0, st, a, bv);
}

cudaError_t launch_prefix_partition(cudaStream_t st, bool comp, const float* w, uint32_t n,
                                    BuildCtrl* ctrl, PartState* states, uint32_t cap_tiles,
                                    uint32_t* idx_out, float* prefix_out, float* elems_out,
                                    float* prefix_lo_out) {
    const PartArgs a{w,         n,           ctrl,          &ctrl->part, states,   cap_tiles,
                     kSpinLimit, &ctrl->status, idx_out,  prefix_out, elems_out, prefix_lo_out};
    const uint32_t precision = prefix_lo_out ? 2u : (comp ? 1u : 0u);
    part_dispatch<false>(st, precision, tiles_for(n), a, BatchView{});
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// inclusive scan (ITS build)
// ---------------------------------------------------------------------------------

template <bool COMP>
__device__ __forceinline__ ff ff_warp_sum(ff v) {
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) v = carry_add<COMP>(v, shfl_xor_ff(v, m));
    return v;
}

template <bool COMP>
__device__ ff scan_lookback(const ScanState* st, uint32_t tile, uint32_t* status,
                            uint32_t spin_limit) {
    return lookback_walk(
        tile, 0u, status, spin_limit, ff{0.f, 0.f},
        [st](uint32_t pos, ff& v) -> int {
            unsigned long long a, p;
            ld_relaxed_v2(reinterpret_cast<const unsigned long long*>(st + pos), a, p);
            if (ff_ready(p)) {
                v = unpack_ff(p);
                return 2;
            }
            if (ff_ready(a)) {
                v = unpack_ff(a);
                return 1;
            }
            return 0;
        },
        [](ff v) { return ff_warp_sum<COMP>(v); },
        [](ff a, ff b) { return carry_add<COMP>(a, b); });
}

// The FP32-carry scan with its tile brought in by one bulk copy.  Thread 0 takes the tile's
// ticket and at once issues a cp.async.bulk (the TMA unit) of the whole tile, kScanBulkV * 4 KB,
// into shared memory, completing on an mbarrier; the threads then read it from there.  With
// no registers held by loads in flight, a CTA covers kScanBulkV * 1024 items and more CTAs fit
// on an SM than with register tiles, so more of HBM's latency is covered while tiles wait in
// the lookback.  Per tile: each thread sums its float4s, warp scans give lane and warp offsets,
// warp 0 publishes the tile aggregate and runs the lookback, and every element is the FP32
// carry plus its running sum (thread (warp w, lane l) holds the items w*V*128 + v*128 + 4l + c,
// v < V, c < 4).  A tile that is not whole, or an input
// that is not 16-byte aligned, is read with plain loads.  The scan states are indexed by these
// tiles (fewer than the 4096-item tiles the state buffer is sized for).
template <bool COMP, int V>
__global__ __launch_bounds__(kTileThreads) void k_scan_bulk(const float* __restrict__ in,
                                                            uint32_t n, float* __restrict__ out,
                                                            BuildCtrl* __restrict__ ctrl,
                                                            ScanState* __restrict__ states,
                                                            uint32_t cap_tiles,
                                                            uint32_t spin_limit) {
    pdl_entry();
    constexpr uint32_t kItems = kTileThreads * 4u * V;  // per tile
    constexpr uint32_t kWarpSpan = 128u * V;             // per warp
    extern __shared__ __align__(128) float s_tile[];     // kItems floats
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_tile_id, s_epoch;
    __shared__ float s_w[kTileWarps];
    __shared__ ff s_ex;
    LbCtrl* lb = &ctrl->scan;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool aligned_in = (reinterpret_cast<uintptr_t>(in) & 15u) == 0;
    if (threadIdx.x == 0) {
        const uint32_t t = atomicAdd(&lb->ticket, 1u);
        s_tile_id = t;
        s_epoch = ld_relaxed_u32(&lb->epoch);
        if (aligned_in && static_cast<uint64_t>(t) * kItems + kItems <= n) {
            mbar_init(&s_bar, 1u);
            mbar_init_fence();
            mbar_arrive_expect_tx(&s_bar, kItems * 4u);
            bulk_load_smem(s_tile, in + static_cast<size_t>(t) * kItems, kItems * 4u, &s_bar);
        }
    }
    __syncthreads();
    const uint32_t tile = s_tile_id, epoch = s_epoch;
    ScanState* cur = states + static_cast<size_t>(epoch & 1u) * cap_tiles;
    {
        // the other half of the states is the next launch's: clear this launch's share
        ScanState* other = states + static_cast<size_t>((epoch + 1u) & 1u) * cap_tiles;
        constexpr int kWords = sizeof(ScanState) / 16;
        for (uint32_t t = tile; t < cap_tiles; t += gridDim.x)
            if (threadIdx.x < kWords)
                reinterpret_cast<ulonglong2*>(other + t)[threadIdx.x] = make_ulonglong2(0ull, 0ull);
    }
    const uint64_t tbase = static_cast<uint64_t>(tile) * kItems;
    const bool whole = aligned_in && tbase + kItems <= n;
    bool landed = true;
    if (whole) {
        // the copy's own budget, not the caller's lookback budget: whether it lands depends
        // on no other CTA
        landed = mbar_wait_bounded(&s_bar, 0u, kSpinLimit);
    } else {
        for (uint32_t e = threadIdx.x; e < kItems; e += kTileThreads)
            s_tile[e] = tbase + e < n ? __ldg(in + tbase + e) : 0.0f;
    }
    if (__syncthreads_or(!landed)) {
        // the copy did not land in time: report it, keep waiting (kCopyDrainLimit more tries)
        // for it to end before the CTA's shared memory goes, and leave the tile unpublished
        // (its successors' lookbacks give up in turn)
        if (threadIdx.x == 0) atomicOr(&ctrl->status, kStatusTimeout);
        if (whole) mbar_wait_bounded(&s_bar, 0u, kCopyDrainLimit);
        lookback_end(lb);
        return;
    }
    const float4* q = reinterpret_cast<const float4*>(s_tile + warp * kWarpSpan);
    float lex[V], voff[V], run = 0.f;
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const float4 e4 = q[v * 32 + lane];
        float t = __fadd_rn(__fadd_rn(__fadd_rn(e4.x, e4.y), e4.z), e4.w);
        float inc = warp_incl_f(t, lane);
        float e = __shfl_up_sync(0xffffffffu, inc, 1);
        lex[v] = lane ? e : 0.f;
        voff[v] = run;
        run = __fadd_rn(run, __shfl_sync(0xffffffffu, inc, 31));
    }
    if (lane == 0) s_w[warp] = run;
    __syncthreads();
    if (warp == 0) {
        float t = lane < kTileWarps ? s_w[lane] : 0.f;
        float inc = warp_incl_f(t, lane);
        float e = __shfl_up_sync(0xffffffffu, inc, 1);
        ff agg{__shfl_sync(0xffffffffu, inc, kTileWarps - 1), 0.f};
        __syncwarp();
        if (lane < kTileWarps) s_w[lane] = lane ? e : 0.f;
        ff ex{0.f, 0.f};
        unsigned long long* st = reinterpret_cast<unsigned long long*>(cur + tile);
        if (tile == 0) {
            if (lane == 0) st_relaxed_v2(st, pack_ff(agg), pack_ff(agg));
        } else {
            if (lane == 0) st_relaxed(st, pack_ff(agg));
            ex = scan_lookback<COMP>(cur, tile, &ctrl->status, spin_limit);
            if (lane == 0) st_relaxed(st + 1, pack_ff(carry_add<COMP>(ex, agg)));
        }
        if (lane == 0) s_ex = ex;
    }
    __syncthreads();
    const ff ex = s_ex;
    const float wex = s_w[warp];
    const uint64_t wbase = tbase + warp * kWarpSpan;
    const bool full = whole && (reinterpret_cast<uintptr_t>(out) & 15u) == 0;
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const float4 e4 = q[v * 32 + lane];
        const float xv[4] = {e4.x, e4.y, e4.z, e4.w};
        float r = __fadd_rn(__fadd_rn(wex, voff[v]), lex[v]);
        float y[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            r = __fadd_rn(r, xv[c]);
            y[c] = carry_apply<COMP>(ex, r);
        }
        const uint64_t e0 = wbase + v * 128 + lane * 4;
        if (full) {
            __stcs(reinterpret_cast<float4*>(out + e0), make_float4(y[0], y[1], y[2], y[3]));
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (e0 + c < n) out[e0 + c] = y[c];
        }
    }
    lookback_end(lb);
}
constexpr int kScanBulkV = 8;  // 8192 items (32 KB) per tile

// Compensated scan with exact carries (the ITS / Cutpoint CMF).  Thread t of warp w holds the
// 16 consecutive items [w*512 + 16t, +16) (re-read from the parked tile) and runs an FP32
// running sum r over them from zero; its total T is that sum's last value.  Every element's
// value is RN(C + E + fx(r)): C the exact carry of the tiles before, E the exact sum of
// fx(T) over the threads before it in the tile, all on the fixed-point grid of the
// distribution's total mass.  A thread's last element and the next thread's (or tile's) first
// element therefore differ by exactly that element's own FP32 increment: the CMF is
// non-decreasing, equal across zero weights (which can never be drawn), and independent of
// the lookback's timing.
__device__ u128 scan_lookback_x(const ScanState* st, uint32_t tile, uint32_t* status,
                                uint32_t spin_limit) {
    return lookback_walk(
        tile, 0u, status, spin_limit, static_cast<u128>(0),
        [st](uint32_t pos, u128& v) -> int {
            const unsigned long long* q = st[pos].q;
            unsigned long long lo, hi;
            ld_relaxed_v2(q + 2, lo, hi);
            int s = 2;
            if (!fx_ready(lo, hi)) {
                ld_relaxed_v2(q + 0, lo, hi);
                s = fx_ready(lo, hi) ? 1 : 0;
            }
            if (s) v = fx_unpack(lo, hi);
            return s;
        },
        [](u128 v) {
#pragma unroll
            for (int m = 1; m < 32; m <<= 1) v += shfl_xor_u128(v, m);
            return v;
        },
        [](u128 a, u128 b) { return a + b; });
}

// RN(k * 2^g + r), r the thread's FP32 running sum, decided from a float-float evaluation
// where that is safe (Ziv's rounding test).  With kf = fx_to_ff(k, g) (kf.hi + kf.lo within
// u^2 of k * 2^g, u = 2^-24 the unit roundoff), two_sum(kf.hi, r) exact, one rounding of u^2
// in the low words and fast_two_sum exact, v.hi + v.lo is within 3u^2 (1 + u) of the exact
// value X.  If it lies more than 2^-44 v.hi (> 5 times that) from the midpoints between v.hi
// and its neighbours, X rounds to v.hi; otherwise -- and for r < 0 or NaN, and values outside
// [2^-100, 2^100], where the spacing arithmetic below is not exact -- the fixed-point path
// rounds the exact sum, so the result is fx_round's in every case.
__device__ __forceinline__ float cmf_round(u128 k, ff kf, float r, int g) {
    const ff s = two_sum(kf.hi, r);
    const ff v = fast_two_sum(s.hi, __fadd_rn(s.lo, kf.lo));
    const uint32_t b = __float_as_uint(v.hi);
    const float up = __fsub_rn(__uint_as_float(b + 1u), v.hi);    // spacing above v.hi
    const float down = __fsub_rn(v.hi, __uint_as_float(b - 1u));  // spacing below v.hi
    const float margin = __fsub_rn(__fmul_rn(0.5f, v.lo >= 0.0f ? up : down), fabsf(v.lo));
    const bool ok = r >= 0.0f && v.hi >= 0x1p-100f && v.hi <= 0x1p100f &&
                    margin > __fmul_rn(v.hi, 0x1p-44f);
    return ok ? v.hi : fx_round(k + fx_from_float(r, g), g);
}

// 8 CTAs per SM (32 registers): while warp 0 of a CTA walks the lookback, the other CTAs'
// warps keep the SM busy (0.255 -> 0.234 ms for the compensated prefix sum at N = 2^26 against
// the default 6 CTAs of 40 registers)
__global__ __launch_bounds__(kTileThreads, 8) void k_scan_exact(const float* __restrict__ in,
                                                             uint32_t n, float* __restrict__ out,
                                                             BuildCtrl* __restrict__ ctrl,
                                                             ScanState* __restrict__ states,
                                                             uint32_t cap_tiles,
                                                             uint32_t spin_limit) {
    pdl_entry();
    __shared__ float4 s_x[kTileItems / 4];  // the tile (park_slot), later its outputs
    __shared__ u128 s_e[kTileThreads];       // exact thread-exclusive sums within the warp
    __shared__ u128 s_wt[kTileWarps];        // exact warp totals -> warp-exclusive sums
    __shared__ u128 s_c;                     // exact carry of the tiles before
    ScanState* cur;
    const uint32_t tile = lookback_begin(&ctrl->scan, states, cap_tiles, cur);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grid = fx_grid(ctrl->total);
    {
        float x[4][4];
        load_tile(in, n, tile, x);
#pragma unroll
        for (int v = 0; v < 4; ++v)
            s_x[park_slot(warp * 128 + v * 32 + lane)] = make_float4(x[v][0], x[v][1], x[v][2], x[v][3]);
    }
    __syncwarp();
    {
        float t = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 q = s_x[park_slot(warp * 128 + lane * 4 + j)];
            t = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(t, q.x), q.y), q.z), q.w);
        }
        const u128 X = fx_from_float(t, grid);
        u128 inc = X;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long lo =
                __shfl_up_sync(0xffffffffu, static_cast<unsigned long long>(inc), d);
            const unsigned long long hi =
                __shfl_up_sync(0xffffffffu, static_cast<unsigned long long>(inc >> 64), d);
            if (lane >= d) inc += (static_cast<u128>(hi) << 64) | lo;
        }
        s_e[threadIdx.x] = inc - X;
        if (lane == 31) s_wt[warp] = inc;
    }
    __syncthreads();
    if (warp == 0) {
        u128 agg = 0;
        if (lane == 0) {
            for (int k = 0; k < kTileWarps; ++k) {
                const u128 t = s_wt[k];
                s_wt[k] = agg;
                agg += t;
            }
        }
        __syncwarp();
        const unsigned long long alo = __shfl_sync(0xffffffffu, static_cast<unsigned long long>(agg), 0);
        const unsigned long long ahi =
            __shfl_sync(0xffffffffu, static_cast<unsigned long long>(agg >> 64), 0);
        agg = (static_cast<u128>(ahi) << 64) | alo;
        unsigned long long* q = cur[tile].q;
        u128 ex = 0;
        if (tile == 0) {
            if (lane == 0) {
                st_relaxed_v2(q + 0, fx_word_lo(agg), fx_word_hi(agg));
                st_relaxed_v2(q + 2, fx_word_lo(agg), fx_word_hi(agg));
            }
        } else {
            if (lane == 0) st_relaxed_v2(q + 0, fx_word_lo(agg), fx_word_hi(agg));
            ex = scan_lookback_x(cur, tile, &ctrl->status, spin_limit);
            if (lane == 0) st_relaxed_v2(q + 2, fx_word_lo(ex + agg), fx_word_hi(ex + agg));
        }
        if (lane == 0) s_c = ex;
    }
    __syncthreads();
    {
        const u128 K = s_c + s_wt[warp] + s_e[threadIdx.x];
        const ff kf = fx_to_ff(K, grid);
        float r = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float4& slot = s_x[park_slot(warp * 128 + lane * 4 + j)];
            float4 q = slot;
            r = __fadd_rn(r, q.x);
            q.x = cmf_round(K, kf, r, grid);
            r = __fadd_rn(r, q.y);
            q.y = cmf_round(K, kf, r, grid);
            r = __fadd_rn(r, q.z);
            q.z = cmf_round(K, kf, r, grid);
            r = __fadd_rn(r, q.w);
            q.w = cmf_round(K, kf, r, grid);
            slot = q;  // this thread's own chunks: no other thread touches them here
        }
    }
    __syncthreads();
    const uint32_t tbase = tile * kTileItems;
    const bool full = (static_cast<uint64_t>(tbase) + kTileItems <= n) &&
                      ((reinterpret_cast<uintptr_t>(out) & 15u) == 0);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const uint32_t chunk = warp * 128 + v * 32 + lane;
        const float4 y = s_x[park_slot(chunk)];
        const uint32_t e0 = tbase + chunk * 4;
        if (full) {
            __stcs(reinterpret_cast<float4*>(out + e0), y);
        } else {
            const float yv[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (e0 + c < n) out[e0 + c] = yv[c];
        }
    }
    lookback_end(&ctrl->scan);
}

cudaError_t launch_scan(cudaStream_t st, bool comp, const float* in, uint32_t n, float* out,
                        BuildCtrl* ctrl, ScanState* states, uint32_t cap_tiles, double* partials,
                        uint32_t spin_limit) {
    const uint32_t tiles = tiles_for(n);
    if (comp) {
        // the exact carries need the distribution's fixed-point grid: its total mass first
        cudaError_t e = launch_total_mass(st, in, n, partials, ctrl);
        if (e != cudaSuccess) return e;
        launch_pdl(k_scan_exact, tiles, kTileThreads, 0, st, in, n, out, ctrl, states, cap_tiles, spin_limit);
    } else {
        constexpr uint32_t items = kTileThreads * 4u * kScanBulkV;
        const uint32_t bulk_tiles = static_cast<uint32_t>((static_cast<uint64_t>(n) + items - 1) / items);
        launch_pdl(k_scan_bulk<false, kScanBulkV>, bulk_tiles, kTileThreads, items * sizeof(float), st, 
            in, n, out, ctrl, states, cap_tiles, spin_limit);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// PSA split + pack
// ---------------------------------------------------------------------------------

struct PackIn {
    const float* w;
    const uint32_t* idx;
    const float* elems;  // partition-ordered weights, or nullptr (then w[idx[pos]])
    const float* prefix;
    const float* prefix_lo;  // low words of a float-float prefix, or nullptr
    uint32_t n, hc, lc;
    uint32_t lcap;  // largest light count a split may take: lc - 1 (shader) or lc
    float mean;
    float mean_lo;  // (mean, mean_lo) = total / N as a float-float pair
};

// Float-float (FP32) evaluation of sigma - target with sigma = (h + hl) + (l + ll) and
// target = (t + tl): two_sum of the high words plus the low words, then the high parts of
// sigma and target are subtracted first (exact when within a factor of two of each other,
// decisive otherwise) and the low parts added.  Rounded once to FP32.
__device__ __forceinline__ float ff_sigma_minus(float h, float hl, float l, float ll, float t,
                                                float tl) {
    const ff s = two_sum(h, l);
    const float lo = __fadd_rn(__fadd_rn(s.lo, hl), ll);
    const float d = __fsub_rn(s.hi, t);
    return __fadd_rn(d, __fsub_rn(lo, tl));
}

// (mean + mean_lo) * n as a float-float pair in FP32: n = n1 + n2 with n1 = n & ~0xff and
// n2 = n & 0xff (both exact in FP32); the products of the high word are exact through FMA,
// the low word's product is rounded once.
__device__ __forceinline__ ff ff_target(float m, float ml, uint32_t n) {
    const float n1 = __uint2float_rn(n & ~0xffu), n2 = __uint2float_rn(n & 0xffu);
    const float p1 = __fmul_rn(m, n1), e1 = __fmaf_rn(m, n1, -p1);
    const float p2 = __fmul_rn(m, n2), e2 = __fmaf_rn(m, n2, -p2);
    const float p3 = __fmul_rn(ml, __uint2float_rn(n));
    const ff s = two_sum(p1, p2);
    const float lo = __fadd_rn(s.lo, __fadd_rn(__fadd_rn(e1, e2), p3));
    return fast_two_sum(s.hi, lo);
}


// splitpack/inline/shader.comp:81-114: bisection over the number of heavy items with the
// shader's probe sequence (a = 0, b = heavyCount - 1, j = (a + b) / 2) and its FP32
// comparisons, so split points match the shader's.  R64 evaluates the split-point
// residual (the spill) in FP64 and rounds it once.  The light count is capped at c.lcap:
// lightCount - 1 as in the shader, or lightCount (which keeps i + j = n at the end of the
// table).  If every probe exceeds the target (the shader's b would wrap), j = 0.
//
// FF (float-float prefix): each comparison sigma <= target and the final spill are
// evaluated on float-float values (ff_sigma_minus) -- sigma from the high and low words of
// the heavy and light prefixes, target = (total / N) * n as a float-float pair (ff_target) --
// instead of on FP32 high words and the FP32 mean, all in FP32 arithmetic (GB300 runs FP64
// at a small fraction of the FP32 rate).  Measuring targets against the exact mean keeps the
// FP32 rounding of the mean from piling up in the last heavy bucket.
template <bool R64, bool FF>
__device__ __forceinline__ void compute_split(const PackIn& c, uint32_t nsplit, uint32_t& io,
                                              uint32_t& jo, float& spill) {
    // indices fit in int32 (n < 2^31); b becomes -1 when every probe exceeds the target
    int a = 0, b = static_cast<int>(c.hc) - 1;
    const float target = __fmul_rn(c.mean, __uint2float_rn(nsplit));
    ff tff{0.f, 0.f};
    if constexpr (FF) tff = ff_target(c.mean, c.mean_lo, nsplit);
    const uint32_t lcm1 = c.lcap;
    while (a <= b) {
        const uint32_t j = static_cast<uint32_t>(a + ((b - a) >> 1));
        const uint32_t i = j > nsplit ? lcm1 : min(nsplit - j, lcm1);
        const float heavy = j == 0 ? 0.f : __ldg(c.prefix + j - 1);
        const float light = i == 0 ? 0.f : __ldg(c.prefix + c.n - i);
        bool le;
        if constexpr (FF) {
            const float hl = j == 0 ? 0.f : __ldg(c.prefix_lo + j - 1);
            const float ll = i == 0 ? 0.f : __ldg(c.prefix_lo + c.n - i);
            le = ff_sigma_minus(heavy, hl, light, ll, tff.hi, tff.lo) <= 0.0f;
        } else {
            le = __fadd_rn(light, heavy) <= target;
        }
        if (le)
            a = static_cast<int>(j) + 1;
        else
            b = static_cast<int>(j) - 1;
    }
    const uint32_t j = b < 0 ? 0u : static_cast<uint32_t>(b);
    const uint32_t i = j > nsplit ? lcm1 : min(nsplit - j, lcm1);
    const float light = i == 0 ? 0.f : __ldg(c.prefix + c.n - i);
    const float heavy2 = __ldg(c.prefix + j);
    if constexpr (FF) {
        const float hl2 = __ldg(c.prefix_lo + j);
        const float ll = i == 0 ? 0.f : __ldg(c.prefix_lo + c.n - i);
        spill = ff_sigma_minus(heavy2, hl2, light, ll, tff.hi, tff.lo);
    } else if constexpr (R64) {
        const double target64 =
            __dmul_rn(static_cast<double>(c.mean), static_cast<double>(nsplit));
        spill = __double2float_rn(
            __dsub_rn(__dadd_rn(static_cast<double>(heavy2), static_cast<double>(light)), target64));
    } else {
        spill = __fsub_rn(__fadd_rn(heavy2, light), target);
    }
    io = i;
    jo = j;
}

// compute_split's probe sequence and arithmetic for the split-pack's one split per thread,
// started from (a, b): the bisection state after the levels every split of the CTA decides
// alike (split_descent), or (0, hc - 1) from the top.
//
// FF: an FP32 pre-test decides most levels without the low words.  d = (h + l) - t differs
// from the float-float value (h + hl) + (l + ll) - (t + tl) by at most 3u(h + l) + 2u t
// (u = 2^-24, |lo| <= u |hi|), and the float-float evaluation is accurate to O(u^2); beyond
// 8u(h + l + t) both have d's sign, so the low words are only read near the split point and
// every decision is the float-float one.
template <bool R64, bool FF>
__device__ __forceinline__ void bisect_one(const PackIn& c, uint32_t nsplit, bool on, uint32_t& io,
                                           uint32_t& jo, float& spill, int a, int b) {
    if (!on) return;
    const float target = __fmul_rn(c.mean, __uint2float_rn(nsplit));
    ff tff{0.f, 0.f};
    if constexpr (FF) tff = ff_target(c.mean, c.mean_lo, nsplit);
    const uint32_t lcm1 = c.lcap;
    while (a <= b) {
        const uint32_t j = static_cast<uint32_t>(a + ((b - a) >> 1));
        const uint32_t i = j > nsplit ? lcm1 : min(nsplit - j, lcm1);
        const float heavy = j ? __ldg(c.prefix + j - 1) : 0.f;
        const float light = i ? __ldg(c.prefix + c.n - i) : 0.f;
        bool le;
        if constexpr (FF) {
            const float hs = __fadd_rn(heavy, light);
            const float d = __fsub_rn(hs, tff.hi);
            const float m = __fmul_rn(4.76837158203125e-07f, __fadd_rn(hs, tff.hi));
            if (d > m) {
                le = false;
            } else if (d < -m) {
                le = true;
            } else {
                const float hl = j ? __ldg(c.prefix_lo + j - 1) : 0.f;
                const float ll = i ? __ldg(c.prefix_lo + c.n - i) : 0.f;
                le = ff_sigma_minus(heavy, hl, light, ll, tff.hi, tff.lo) <= 0.0f;
            }
        } else {
            le = __fadd_rn(light, heavy) <= target;
        }
        if (le)
            a = static_cast<int>(j) + 1;
        else
            b = static_cast<int>(j) - 1;
    }
    const uint32_t j = b < 0 ? 0u : static_cast<uint32_t>(b);
    const uint32_t i = j > nsplit ? lcm1 : min(nsplit - j, lcm1);
    const float light = i == 0 ? 0.f : __ldg(c.prefix + c.n - i);
    const float heavy2 = __ldg(c.prefix + j);
    if constexpr (FF) {
        const float hl2 = __ldg(c.prefix_lo + j);
        const float l2 = i == 0 ? 0.f : __ldg(c.prefix_lo + c.n - i);
        spill = ff_sigma_minus(heavy2, hl2, light, l2, tff.hi, tff.lo);
    } else if constexpr (R64) {
        const double target64 =
            __dmul_rn(static_cast<double>(c.mean), static_cast<double>(nsplit));
        spill = __double2float_rn(
            __dsub_rn(__dadd_rn(static_cast<double>(heavy2), static_cast<double>(light)), target64));
    } else {
        spill = __fsub_rn(__fadd_rn(heavy2, light), target);
    }
    io = i;
    jo = j;
}

// The top of the bisections of one CTA's splits, shared.  Every split of a CTA starts from
// (a, b) = (0, hc - 1) and probes the same j while its decisions agree with the others'.  For a
// fixed j the probed difference f(n) = heavy(j) + light(n - j) - mean * n does not increase
// with n in exact arithmetic (one more light item adds at most the mean), and the stored
// prefixes are non-decreasing up to a few ulps; so where the CTA's first split n0 and last
// split n1 both evaluate f beyond a margin M of 64 ulps of the larger of their
// (heavy + light + target) on the same side, every split n0 <= n <= n1 has |f(n)| > M - (a
// few ulps) on that side, which its own FP32 evaluation (error below 2 ulps of its, smaller,
// heavy + light + target) and float-float evaluation decide alike.  split_descent walks the
// levels the two end splits decide alike with that margin and stops at the first other one;
// starting every split of the CTA from the state it returns skips those levels without
// changing any split (the probe sequence below it is the shader's).
template <bool FF>
__device__ void split_descent(const PackIn& c, uint32_t n0, uint32_t n1, int& a, int& b) {
    a = 0;
    b = static_cast<int>(c.hc) - 1;
    const uint32_t lcap = c.lcap;
    const uint32_t ns[2] = {n0, n1};
    float t[2];
#pragma unroll
    for (int e = 0; e < 2; ++e)
        t[e] = FF ? ff_target(c.mean, c.mean_lo, ns[e]).hi : __fmul_rn(c.mean, __uint2float_rn(ns[e]));
    while (a <= b) {
        const uint32_t j = static_cast<uint32_t>(a + ((b - a) >> 1));
        float d[2], mag[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const uint32_t i = j > ns[e] ? lcap : min(ns[e] - j, lcap);
            const float h = j == 0 ? 0.f : __ldg(c.prefix + j - 1);
            const float l = i == 0 ? 0.f : __ldg(c.prefix + c.n - i);
            const float sum = __fadd_rn(l, h);
            d[e] = __fsub_rn(sum, t[e]);
            mag[e] = __fadd_rn(sum, t[e]);
        }
        const float m = __fmul_rn(3.814697265625e-06f, fmaxf(mag[0], mag[1]));  // 64 * 2^-24
        int dec[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) dec[e] = d[e] < -m ? 1 : (d[e] > m ? -1 : 0);
        if (dec[0] == 0 || dec[0] != dec[1]) break;
        if (dec[0] > 0)
            a = static_cast<int>(j) + 1;
        else
            b = static_cast<int>(j) - 1;
    }
}

// splitpack/inline/shader.comp:130-211.  The shader's closing "last heavy -> (1, self)"
// write (:212-222) is not performed: in subproblem order it is always overwritten by the
// final subproblem, which packs the last heavy item itself (the oracle keeps the write and
// the parity tests confirm the tables agree).
//
// Subproblems normally cover disjoint items.  Where FP32 rounding makes a split step back
// (split_{k+1} < split_k, one or two items at N >= 2^22), two subproblems pack the same
// items and, in subproblem order, the later one's write stands.  `later` (null when the
// next kSplitLook splits do not step back into this subproblem's range) lists the splits of
// the following subproblems; an entry is then written only if none of them covers it.
struct LaterSplits {
    const uint32_t* si;  // shared-memory split arrays of the CTA
    const uint32_t* sj;
    int t;               // this subproblem's slot
    int count;           // later subproblems inside the window
};

__device__ __forceinline__ bool covered_later(const LaterSplits& L, uint32_t item, bool light) {
    const uint32_t* s = light ? L.si : L.sj;
    for (int d = 1; d <= L.count; ++d) {
        const uint32_t a = s[L.t + d], b = max(s[L.t + d + 1], a);
        if (a <= item && item < b) return true;
    }
    return false;
}

// The partition items a CTA's subproblems walk, staged in shared memory by one coalesced pass
// (the walks themselves read one item per step at positions that differ from thread to
// thread): heavy positions [hlo, hlo + hcnt) at s[0, hcnt), light ranks [llo, llo + lcnt)
// (partition position n - 1 - rank) at s[hcnt, hcnt + lcnt), each as (original index, weight
// bits).  Items outside the windows (a split stepping back, a window larger than kPackWin)
// are read from global memory; the values are the same.
constexpr uint32_t kPackWin = 6144;
struct PackWin {
    const uint2* s;
    uint32_t hlo, hcnt, llo, lcnt;
};

__device__ __forceinline__ uint2 item_global(const PackIn& c, uint32_t pos) {
    const uint32_t widx = __ldg(c.idx + pos);
    // widx < n holds for any partition this library wrote; the guard keeps a corrupt one
    // (e.g. after a lookback wait gave up) from reading out of bounds
    const float wt = c.elems ? __ldg(c.elems + pos) : (widx < c.n ? __ldg(c.w + widx) : 0.f);
    return make_uint2(widx, __float_as_uint(wt));
}
__device__ __forceinline__ uint2 heavy_item(const PackIn& c, const PackWin& win, uint32_t pos) {
    return pos - win.hlo < win.hcnt ? win.s[pos - win.hlo] : item_global(c, pos);
}
__device__ __forceinline__ uint2 light_item(const PackIn& c, const PackWin& win, uint32_t rank) {
    return rank - win.llo < win.lcnt ? win.s[win.hcnt + rank - win.llo]
                                     : item_global(c, c.n - 1u - rank);
}

//
// Table end (with the full light cap, c.lcap == c.lc): the shader takes the item at partition
// position j + 1 as the next heavy even when j + 1 = heavyCount, i.e. the first light one, so
// the last heavy bucket's residual -- and every light bucket packed after the heavies ran out
// -- aliases that light item, which may have weight zero.  Here the current heavy never leaves
// the heavy range: the last heavy item is packed as (1, itself) and later light buckets alias
// it.  In exact arithmetic its residual is exactly one mean there, so nothing moves; in
// floating point the residual's error stays on a heavy item and no zero-weight item can be
// drawn.
__device__ void pack(const PackIn& c, const PackWin& win, uint2* __restrict__ table, uint32_t i0,
                     uint32_t i1, uint32_t j0, uint32_t j1, float spill,
                     const LaterSplits* later) {
    uint32_t i = i0, j = j0;
    float wv = spill;
    const bool close_last = c.lcap == c.lc;
    // h: the original index of heavy item j, the current heavy; a heavy step moves it to
    // item j + 1, whose index that step has just read
    uint32_t h = 0;
    if (wv == 0.0f || i < i1 || j < j1) {
        const uint2 first = heavy_item(c, win, j);
        h = first.x;
        if (wv == 0.0f) wv = __uint_as_float(first.y);
        if (close_last && j >= c.hc) h = heavy_item(c, win, c.hc - 1u).x;
    }
    // The walk's two candidates are loaded one step ahead: the next heavy item (position j + 1,
    // needed while j < min(j1, hc)) and the next light item (rank i, while i < min(i1, lc)).  A
    // step takes one of them and loads its successor, so no load waits for the step's
    // decision (the values are those the step would load).
    const uint32_t jmax = min(j1, c.hc), imax = min(i1, c.lc);
    uint2 next_h = j < jmax ? heavy_item(c, win, j + 1u) : make_uint2(0u, 0u);
    uint2 next_l = i < imax ? light_item(c, win, i) : make_uint2(0u, 0u);
    while (i < i1 || j < j1) {
        bool heavy_step;
        if (j == j1 || j == c.hc)
            heavy_step = false;
        else if (i == i1 || i == c.lc)
            heavy_step = true;
        else
            heavy_step = wv <= c.mean;
        const uint2 it = heavy_step ? next_h : next_l;
        const uint32_t widx = it.x;
        const float weight = __uint_as_float(it.y);
        float p;
        uint32_t tidx, al;
        bool owned = true;
        if (heavy_step) {
            const bool last = close_last && j + 1u == c.hc;
            p = last ? 1.0f : __fdiv_rn(wv, c.mean);
            al = last ? h : widx;
            tidx = h;
            if (later) owned = !covered_later(*later, j, false);
            ++j;
            if (!last) h = widx;
            if (j < jmax) next_h = heavy_item(c, win, j + 1u);
        } else {
            p = __fdiv_rn(weight, c.mean);
            al = h;
            tidx = widx;
            if (later) owned = !covered_later(*later, i, true);
            ++i;
            if (i < imax) next_l = light_item(c, win, i);
        }
        if (owned && tidx < c.n) table[tidx] = make_uint2(__float_as_uint(p), al);
        wv = __fsub_rn(__fadd_rn(wv, weight), c.mean);
    }
}

// The inline split-pack's walk with its results staged for a coalesced write-out.  In a walk,
// only two things depend on the walk itself: the residual a heavy bucket is packed with (its
// p = residual / mean) and the heavy item current when a light bucket is packed (its alias).
// Everything else of an entry is a function of the item: a heavy bucket's table index and its
// alias are the original indices of positions j and j + 1, a light bucket's p is its weight /
// mean.  So the walk reads only the weights and records, per heavy position of the CTA's
// range, the residual, and per light rank the current heavy's position; the CTA then writes
// its entries position by position, consecutive lanes on consecutive positions, whose table
// indices increase (the partition is stable) -- instead of one scattered 8-byte store per
// step.  Decisions, arithmetic and the ownership of overlapping subproblems are pack()'s, so
// the table is the same bit for bit.  A position outside the staged ranges (a split stepping
// back past them) is written directly, as pack() writes it.
// The inline split-pack stages one word per heavy position and light rank its CTA's walks
// cover: kSplitPack * split_size items when the CTA's splits do not step back, plus the
// walks' margins.  At most 48 KB (four CTAs of 512 threads per SM); split sizes that need
// more stage nothing (0) and write their entries directly, rather than hold shared memory
// that lowers occupancy without use.
constexpr uint32_t kStageMaxEntries = 12288;
__host__ __device__ inline uint32_t stage_entries_for(uint32_t split_size) {
    const uint64_t e = static_cast<uint64_t>(kSplitPack) * split_size + 256u;
    return e <= kStageMaxEntries ? static_cast<uint32_t>(e) : 0u;
}
constexpr uint32_t kNotStaged = 0xffffffffu;
// One 32-bit word per staged position: heavy positions [h0, h0 + hcnt) at words [0, hcnt) hold
// the residual's bits (a NaN residual in its canonical form, so no residual equals kNotStaged;
// the NaN table entry it gives is the same), light ranks [l0, l0 + lcnt) at words
// [hcnt, hcnt + lcnt) the current heavy's position; kNotStaged where this CTA packed nothing.
struct EntryStage {
    uint32_t* w;
    uint32_t h0, hcnt, l0, lcnt;
};

__device__ __forceinline__ float item_weight(const PackIn& c, uint32_t pos) {
    if (c.elems) return __ldg(c.elems + pos);
    const uint32_t widx = __ldg(c.idx + pos);
    return widx < c.n ? __ldg(c.w + widx) : 0.f;
}

// the entry of heavy position j packed with residual res (pack()'s heavy step)
__device__ __forceinline__ void write_heavy(const PackIn& c, uint2* __restrict__ table,
                                            uint32_t j, float res, bool close_last) {
    const uint32_t tidx = __ldg(c.idx + j);
    const bool last = close_last && j + 1u == c.hc;
    const uint32_t al = last ? tidx : __ldg(c.idx + j + 1u);
    const float p = last ? 1.0f : __fdiv_rn(res, c.mean);
    if (tidx < c.n) table[tidx] = make_uint2(__float_as_uint(p), al);
}
// the entry of light rank i packed while heavy position J was current (pack()'s light step)
__device__ __forceinline__ void write_light(const PackIn& c, uint2* __restrict__ table,
                                            uint32_t i, uint32_t J) {
    const uint32_t pos = c.n - 1u - i;
    const uint32_t tidx = __ldg(c.idx + pos);
    const float weight = c.elems ? __ldg(c.elems + pos) : (tidx < c.n ? __ldg(c.w + tidx) : 0.f);
    if (tidx < c.n)
        table[tidx] = make_uint2(__float_as_uint(__fdiv_rn(weight, c.mean)), __ldg(c.idx + J));
}

// The walk's step is branch-free apart from the rare paths (ownership inside the look-ahead
// window, positions outside the staged ranges): the weight is selected from the two
// candidates, one 32-bit word is staged, and the stream that advanced loads its next weight.
__device__ void pack_staged(const PackIn& c, const EntryStage& st, uint2* __restrict__ table,
                            uint32_t i0, uint32_t i1, uint32_t j0, uint32_t j1, float spill,
                            const LaterSplits* later) {
    uint32_t i = i0, j = j0;
    float wv = spill;
    const bool close_last = c.lcap == c.lc;
    if (wv == 0.0f && (i < i1 || j < j1)) wv = item_weight(c, j);
    const uint32_t jmax = min(j1, c.hc), imax = min(i1, c.lc);
    float next_h = j < jmax ? item_weight(c, j + 1u) : 0.f;
    float next_l = i < imax ? item_weight(c, c.n - 1u - i) : 0.f;
    while (i < i1 || j < j1) {
        const bool heavy_step =
            !(j == j1 || j == c.hc) && ((i == i1 || i == c.lc) || wv <= c.mean);
        const float weight = heavy_step ? next_h : next_l;
        // the current heavy item: position j (pack()'s h), kept inside the heavy range by the
        // table-end rule
        const uint32_t J = close_last && j >= c.hc ? c.hc - 1u : j;
        const uint32_t rel = heavy_step ? j - st.h0 : i - st.l0;
        const bool staged = rel < (heavy_step ? st.hcnt : st.lcnt);
        const uint32_t word = heavy_step ? (wv != wv ? 0x7fffffffu : __float_as_uint(wv)) : J;
        const bool owned = !later || !covered_later(*later, heavy_step ? j : i, !heavy_step);
        if (owned) {
            if (staged)
                st.w[heavy_step ? rel : st.hcnt + rel] = word;
            else if (heavy_step)
                write_heavy(c, table, j, wv, close_last);
            else
                write_light(c, table, i, J);
        }
        j += heavy_step ? 1u : 0u;
        i += heavy_step ? 0u : 1u;
        const bool more = heavy_step ? j < jmax : i < imax;
        const float nw = more ? item_weight(c, heavy_step ? j + 1u : c.n - 1u - i) : 0.f;
        next_h = heavy_step ? nw : next_h;
        next_l = heavy_step ? next_l : nw;
        wv = __fsub_rn(__fadd_rn(wv, weight), c.mean);
    }
}

// pack_staged for a subproblem whose items all lie inside the staged ranges, inside the heavy
// and light ranges (j1 <= heavyCount, i1 <= the light count) and that no later subproblem in
// the window covers: every step is owned and staged, and the end tests reduce to j == j1 and
// i == i1.  Decisions, arithmetic and staged words are pack_staged's.
__device__ __forceinline__ void pack_staged_fast(const PackIn& c, const EntryStage& st,
                                                 uint32_t i0, uint32_t i1, uint32_t j0,
                                                 uint32_t j1, float spill) {
    uint32_t i = i0, j = j0;
    float wv = spill;
    const bool close_last = c.lcap == c.lc;
    if (wv == 0.0f && (i < i1 || j < j1)) wv = item_weight(c, j);
    float next_h = j < j1 ? item_weight(c, j + 1u) : 0.f;
    float next_l = i < i1 ? item_weight(c, c.n - 1u - i) : 0.f;
    uint32_t* const wh = st.w - st.h0;             // heavy position j -> its word
    uint32_t* const wl = st.w + st.hcnt - st.l0;   // light rank i -> its word
    while (i < i1 || j < j1) {
        const bool heavy_step = j != j1 && (i == i1 || wv <= c.mean);
        const float weight = heavy_step ? next_h : next_l;
        const uint32_t J = close_last && j >= c.hc ? c.hc - 1u : j;
        if (heavy_step)
            wh[j] = wv != wv ? 0x7fffffffu : __float_as_uint(wv);
        else
            wl[i] = J;
        j += heavy_step ? 1u : 0u;
        i += heavy_step ? 0u : 1u;
        const bool more = heavy_step ? j < j1 : i < i1;
        const float nw = more ? item_weight(c, heavy_step ? j + 1u : c.n - 1u - i) : 0.f;
        next_h = heavy_step ? nw : next_h;
        next_l = heavy_step ? next_l : nw;
        wv = __fsub_rn(__fadd_rn(wv, weight), c.mean);
    }
}

struct SplitArgs {
    const float* w;  // single distribution: weights, n, control block, table
    uint32_t n;
    const BuildCtrl* ctrl;
    uint2* table;
    const uint32_t* idx;  // partition arrays (a batch adds each distribution's base)
    const float* elems;
    const float* prefix;
    const float* prefix_lo;
    uint32_t* status;
    uint32_t split_size;
    uint32_t full_light;
    SplitRecord* records;  // serial split-pack: the split records (split k = records[k - 1])
    int2* descent;         // per CTA: the shared top of its bisections (k_split_descent) or null
    uint32_t stage;        // record packs: stage the CTA's items in shared memory (kPackWin of
                           // them); the inline kernel always stages its walks' results
};
constexpr uint32_t kStageEntriesMode = 2;

// One thread per split-pack CTA: the shared descent of its splits (k_split_pack's slots
// 1 .. kSplitSlots - 1 of the CTA, the look-ahead slots included).
// (BATCH: one thread per split-pack CTA of the whole batch, each of its distribution)
template <bool FF, bool BATCH>
__global__ __launch_bounds__(256) void k_split_descent(SplitArgs a, BatchView bv) {
    pdl_entry();
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;  // the split-pack CTA
    uint32_t blk = g, n = a.n;
    const BuildCtrl* ctrl = a.ctrl;
    const float* prefix = a.prefix;
    const float* prefix_lo = a.prefix_lo;
    int2* out = a.descent;
    if constexpr (BATCH) {
        if (g >= bv.split_blocks) return;
        const uint32_t d = __ldg(bv.split_map + g);
        const DistDesc* D = bv.dist + d;
        n = D->n;
        blk = g - D->split0;
        ctrl = bv.dctrl + d;
        prefix += D->base;
        if (prefix_lo) prefix_lo += D->base;
        out = bv.descent;
    } else {
        if (g >= split_blocks_for(n, a.split_size)) return;
    }
    const uint32_t K = splits_for(n, a.split_size);
    const uint32_t hc = ctrl->heavy_count;
    int2 st = make_int2(0, static_cast<int>(hc) - 1);
    const uint32_t k0 = max(1u, blk * kSplitPack);
    const uint32_t k1 = min(blk * kSplitPack + kSplitSlots - 1u, K - 1u);
    if (hc != 0u && hc < n && k0 <= k1) {
        const PackIn c{nullptr, nullptr, nullptr, prefix, prefix_lo, n, hc, n - hc,
                       a.full_light ? n - hc : n - hc - 1u, ctrl->mean, ctrl->mean_lo};
        split_descent<FF>(c, k0 * a.split_size, k1 * a.split_size, st.x, st.y);
    }
    out[g] = st;
}


// Slot t of CTA b (t < kSplitSlots; thread t % kSplitThreads holds slots t and t + 512) holds
// split k = b*kSplitPack + t (k in [0, K]) and packs subproblem k = [split_k, split_{k+1})
// for t < kSplitPack, k < K; split_{k+1} comes from the next slot through shared memory
// (shader.comp:225-270).  The last kSplitLook + 1 slots only hold look-ahead splits for the
// ownership window.
template <bool R64, bool FF, bool BATCH, bool RECORDS = false>
__global__ __launch_bounds__(kSplitThreads, 4) void k_split_pack(SplitArgs a, BatchView bv) {
    pdl_entry();
    __shared__ uint32_t s_i[kSplitSlots], s_j[kSplitSlots];
    __shared__ float s_spill[kSplitSlots];
    const float* w = a.w;
    uint32_t n = a.n;
    const BuildCtrl* ctrl = a.ctrl;
    uint2* table = a.table;
    const uint32_t* idx = a.idx;
    const float* elems = a.elems;
    const float* prefix = a.prefix;
    const float* prefix_lo = a.prefix_lo;
    uint32_t blk = blockIdx.x, nblk = gridDim.x;
    if constexpr (BATCH) {
        const uint32_t d = __ldg(bv.split_map + blockIdx.x);
        const DistDesc* D = bv.dist + d;
        w = D->w;
        n = D->n;
        ctrl = bv.dctrl + d;
        table = D->table;
        const uint64_t base = D->base;
        idx += base;
        if (elems) elems += base;
        prefix += base;
        if (prefix_lo) prefix_lo += base;
        blk -= D->split0;
        nblk = split_blocks_for(n, a.split_size);
    }
    // RECORDS (serial split-pack): K = ceil(N / splitSize) subproblems whose splits were
    // written by k_split_records; otherwise the inline split-pack's K = N / splitSize
    const uint32_t K = RECORDS ? records_for(n, a.split_size) : splits_for(n, a.split_size);
    const uint32_t hc = ctrl->heavy_count;
    if (hc == 0u || hc >= n) {
        // degenerate (all items light or all heavy): every bucket keeps itself
        const uint32_t nth = nblk * blockDim.x;
        for (uint32_t e = blk * blockDim.x + threadIdx.x; e < n; e += nth)
            table[e] = make_uint2(__float_as_uint(1.0f), e);
        return;
    }
    PackIn c{w,      idx,    elems,  prefix, prefix_lo, n, hc,
             n - hc, a.full_light ? n - hc : n - hc - 1u, ctrl->mean, ctrl->mean_lo};
    // slot t + v * kSplitThreads of this CTA holds split k = blk * kSplitPack + slot
    uint32_t kv[kSplitPerThread], nsplit[kSplitPerThread], si[kSplitPerThread], sj[kSplitPerThread];
    float sp[kSplitPerThread];
    bool on[kSplitPerThread];
#pragma unroll
    for (int v = 0; v < kSplitPerThread; ++v) {
        kv[v] = blk * kSplitPack + threadIdx.x + v * kSplitThreads;
        on[v] = kv[v] != 0u && kv[v] < K;
        nsplit[v] = on[v] ? kv[v] * a.split_size : 0u;
        si[v] = kv[v] == 0u ? 0u : c.lc;  // past split K: the final split
        sj[v] = kv[v] == 0u ? 0u : hc;
        sp[v] = 0.f;
    }
    if constexpr (RECORDS) {
#pragma unroll
        for (int v = 0; v < kSplitPerThread; ++v) {
            if (!on[v]) continue;
            const SplitRecord r = a.records[kv[v] - 1u];
            si[v] = r.i;
            sj[v] = r.j;
            sp[v] = r.spill;
        }
    } else {
        int2 d0 = make_int2(0, static_cast<int>(hc) - 1);
        const int2* desc = BATCH ? bv.descent : a.descent;
        if (desc) d0 = desc[BATCH ? blockIdx.x : blk];
        static_assert(kSplitPerThread == 1, "one bisection per thread");
        bisect_one<R64, FF>(c, nsplit[0], on[0], si[0], sj[0], sp[0], d0.x, d0.y);
    }
#pragma unroll
    for (int v = 0; v < kSplitPerThread; ++v) {
        const int slot = threadIdx.x + v * kSplitThreads;
        s_i[slot] = si[v];
        s_j[slot] = sj[v];
        s_spill[slot] = sp[v];
    }
    __syncthreads();
    // stage the items of this CTA's subproblems [split_kb, split_{kb + npack}) when the launch
    // gave the shared memory for it (the serial pack at small split sizes: measured faster
    // there; the inline kernel's bisections lose more to the smaller L1 than its walks gain)
    extern __shared__ uint2 s_items[];
    if constexpr (!RECORDS) {
        // the CTA's heavy positions [s_j[0], s_j[npack]) and light ranks [s_i[0], s_i[npack]),
        // with a margin for splits stepping back at the end; staged only if both fit
        const uint32_t kb = blk * kSplitPack;
        const uint32_t npack = min(static_cast<uint32_t>(kSplitPack), K - kb);
        constexpr uint32_t kMargin = 64;
        EntryStage es{reinterpret_cast<uint32_t*>(s_items), s_j[0], 0u, s_i[0], 0u};
        const uint32_t hext = (s_j[npack] > es.h0 ? s_j[npack] - es.h0 : 0u) + kMargin;
        const uint32_t lext = (s_i[npack] > es.l0 ? s_i[npack] - es.l0 : 0u) + kMargin;
        if (hext + lext <= stage_entries_for(a.split_size)) {
            es.hcnt = hext;
            es.lcnt = lext;
        }
        // the CTA's splits in slot order never step back (the common case): then no later
        // subproblem covers an earlier one's items, and the ownership window is not consulted
        bool mono = true;
#pragma unroll
        for (int v = 0; v < kSplitPerThread; ++v) {
            const int t = threadIdx.x + v * kSplitThreads;
            if (t + 1 < kSplitSlots) mono = mono && s_i[t + 1] >= s_i[t] && s_j[t + 1] >= s_j[t];
        }
        for (uint32_t q = threadIdx.x; q < es.hcnt + es.lcnt; q += blockDim.x) es.w[q] = kNotStaged;
        const bool all_mono = __syncthreads_and(mono);
#pragma unroll 1
        for (int v = 0; v < kSplitPerThread; ++v) {
            const int t = threadIdx.x + v * kSplitThreads;
            const uint32_t k = kv[v];
            if (t >= kSplitPack || k >= K) continue;
            const uint32_t i1 = max(s_i[t + 1], si[v]), j1 = max(s_j[t + 1], sj[v]);
            bool clean = true;
            int count = 0;
            if (!all_mono) {
                count = static_cast<int>(min(static_cast<uint32_t>(kSplitLook), K - 1u - k));
                for (int d = 1; d <= count; ++d)
                    clean = clean && s_i[t + d] >= i1 && s_j[t + d] >= j1;
                if (k + kSplitLook + 1u < K &&
                    (s_i[t + kSplitLook + 1] < i1 || s_j[t + kSplitLook + 1] < j1))
                    atomicOr(a.status, kStatusNonMonotone);
            }
            const LaterSplits later{s_i, s_j, t, count};
            const bool inside = sj[v] >= es.h0 && j1 - es.h0 <= es.hcnt && si[v] >= es.l0 &&
                                i1 - es.l0 <= es.lcnt && j1 <= c.hc && i1 <= c.lc;
            if (clean && inside)
                pack_staged_fast(c, es, si[v], i1, sj[v], j1, sp[v]);
            else
                pack_staged(c, es, table, si[v], i1, sj[v], j1, sp[v], clean ? nullptr : &later);
        }
        __syncthreads();
        // write-out: consecutive lanes on consecutive positions, kOutBatch positions per thread
        // with their loads in flight together (write_heavy / write_light's values; positions
        // clamped into [0, n) so that every load is in bounds, only staged entries stored)
        const bool close_last = c.lcap == c.lc;
        constexpr int kOutBatch = 4;
        const uint32_t bd = blockDim.x, nm1 = c.n - 1u;
        for (uint32_t q0 = threadIdx.x; q0 < es.hcnt; q0 += kOutBatch * bd) {
            uint32_t r[kOutBatch], t[kOutBatch], al[kOutBatch];
#pragma unroll
            for (int u = 0; u < kOutBatch; ++u) {
                const uint32_t q = q0 + u * bd;
                r[u] = q < es.hcnt ? es.w[q] : kNotStaged;
                const uint32_t j = min(es.h0 + q, nm1);
                t[u] = __ldg(c.idx + j);
                al[u] = __ldg(c.idx + min(j + 1u, nm1));
            }
#pragma unroll
            for (int u = 0; u < kOutBatch; ++u) {
                if (r[u] == kNotStaged || t[u] >= c.n) continue;
                const bool last = close_last && es.h0 + q0 + u * bd + 1u == c.hc;
                const float p = last ? 1.0f : __fdiv_rn(__uint_as_float(r[u]), c.mean);
                table[t[u]] = make_uint2(__float_as_uint(p), last ? t[u] : al[u]);
            }
        }
        for (uint32_t q0 = threadIdx.x; q0 < es.lcnt; q0 += kOutBatch * bd) {
            uint32_t J[kOutBatch], t[kOutBatch], aj[kOutBatch];
            float wt[kOutBatch];
#pragma unroll
            for (int u = 0; u < kOutBatch; ++u) {
                const uint32_t q = q0 + u * bd;
                J[u] = q < es.lcnt ? es.w[es.hcnt + q] : kNotStaged;
                const uint32_t pos = nm1 - min(es.l0 + q, nm1);
                t[u] = __ldg(c.idx + pos);
                wt[u] = c.elems ? __ldg(c.elems + pos) : (t[u] < c.n ? __ldg(c.w + t[u]) : 0.f);
                aj[u] = __ldg(c.idx + min(J[u], nm1));
            }
#pragma unroll
            for (int u = 0; u < kOutBatch; ++u) {
                if (J[u] == kNotStaged || t[u] >= c.n) continue;
                table[t[u]] = make_uint2(__float_as_uint(__fdiv_rn(wt[u], c.mean)), aj[u]);
            }
        }
        return;
    }
    PackWin win{s_items, 0u, 0u, 0u, 0u};
    if (a.stage) {
        const uint32_t kb = blk * kSplitPack;
        const uint32_t npack = min(static_cast<uint32_t>(kSplitPack), K - kb);
        win.s = s_items;
        win.hlo = s_j[0];
        const uint32_t hhi = min(s_j[npack] + 1u, hc);
        win.hcnt = min(hhi > win.hlo ? hhi - win.hlo : 0u, kPackWin);
        win.llo = s_i[0];
        const uint32_t lhi = s_i[npack];
        win.lcnt = min(lhi > win.llo ? lhi - win.llo : 0u, kPackWin - win.hcnt);
        for (uint32_t q = threadIdx.x; q < win.hcnt + win.lcnt; q += blockDim.x)
            s_items[q] = item_global(c, q < win.hcnt ? win.hlo + q
                                                     : n - 1u - (win.llo + (q - win.hcnt)));
    }
    __syncthreads();
#pragma unroll 1
    for (int v = 0; v < kSplitPerThread; ++v) {
        const int t = threadIdx.x + v * kSplitThreads;
        const uint32_t k = kv[v];
        if (t >= kSplitPack || k >= K) continue;
        const uint32_t i1 = max(s_i[t + 1], si[v]), j1 = max(s_j[t + 1], sj[v]);
        const int count = static_cast<int>(min(static_cast<uint32_t>(kSplitLook), K - 1u - k));
        bool clean = true;
        for (int d = 1; d <= count; ++d)
            clean = clean && s_i[t + d] >= i1 && s_j[t + d] >= j1;
        // a step back reaching past the window cannot be resolved here: report it
        if (k + kSplitLook + 1u < K &&
            (s_i[t + kSplitLook + 1] < i1 || s_j[t + kSplitLook + 1] < j1))
            atomicOr(a.status, kStatusNonMonotone);
        const LaterSplits later{s_i, s_j, t, count};
        pack(c, win, table, si[v], i1, sj[v], j1, sp[v], clean ? nullptr : &later);
    }
}

// the staging window is dynamic shared memory above the 48 KB static limit
constexpr size_t kPackWinBytes = kPackWin * sizeof(uint2);

template <bool R64, bool FF, bool BATCH, bool RECORDS>
static void launch_split_kernel(cudaStream_t st, uint32_t grid, const SplitArgs& a,
                                const BatchView& bv) {
    if (!RECORDS) {  // the inline kernel stages its walks' results (at most 48 KB)
        const size_t bytes = stage_entries_for(a.split_size) * sizeof(uint32_t);
        // with the kernel's static arrays, more than 40 KB needs the opt-in (set on the current
        // device's context, for every such launch; a failure shows as the launch's error)
        if (bytes > (40u << 10))
            cudaFuncSetAttribute(k_split_pack<R64, FF, BATCH, RECORDS>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(bytes));
        launch_pdl(k_split_pack<R64, FF, BATCH, RECORDS>, grid, kSplitThreads, bytes, st, a, bv);
        return;
    }
    if (!a.stage) {
        launch_pdl(k_split_pack<R64, FF, BATCH, RECORDS>, grid, kSplitThreads, 0, st, a, bv);
        return;
    }
    // the attribute belongs to the current device's context: set it for every launch (a
    // host-side call; a failure shows as the launch's error)
    cudaFuncSetAttribute(k_split_pack<R64, FF, BATCH, RECORDS>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kPackWinBytes));
    launch_pdl(k_split_pack<R64, FF, BATCH, RECORDS>, grid, kSplitThreads, kPackWinBytes, st, a, bv);
}

template <bool BATCH>
static void split_dispatch(cudaStream_t st, bool r64, bool ff, uint32_t grid, const SplitArgs& a,
                           const BatchView& bv) {
    if (ff)
        launch_split_kernel<true, true, BATCH, false>(st, grid, a, bv);
    else if (r64)
        launch_split_kernel<true, false, BATCH, false>(st, grid, a, bv);
    else
        launch_split_kernel<false, false, BATCH, false>(st, grid, a, bv);
}

constexpr uint32_t kDescentMinBlocks = 512;

cudaError_t launch_split_pack(cudaStream_t st, bool r64, bool full_light, const float* w,
                              const uint32_t* idx, const float* elems, const float* prefix,
                              const float* prefix_lo, const BuildCtrl* ctrl, uint32_t* status,
                              uint32_t n, uint32_t split_size, uint2* table, int2* descent) {
    const SplitArgs a{w,      n,         ctrl,   table,      idx,
                      elems,  prefix,    prefix_lo, status,  split_size,
                      full_light ? 1u : 0u, nullptr,
                      split_blocks_for(n, split_size) >= kDescentMinBlocks ? descent : nullptr,
                      kStageEntriesMode};
    const uint32_t blocks = split_blocks_for(n, split_size);
    // the extra launch pays off once there are several waves of split-pack CTAs
    if (descent && blocks >= kDescentMinBlocks) {
        if (prefix_lo)
            launch_pdl(k_split_descent<true, false>, (blocks + 255u) / 256u, 256, 0, st, a, BatchView{});
        else
            launch_pdl(k_split_descent<false, false>, (blocks + 255u) / 256u, 256, 0, st, a, BatchView{});
    }
    split_dispatch<false>(st, r64, prefix_lo != nullptr, blocks, a, BatchView{});
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// block-wise (reduce-then-scan) baselines
// ---------------------------------------------------------------------------------
//
// The reference's BlockWiseScan (src/device/prefix_sum/block_wise/BlockWiseScan.hpp:183-215)
// and BlockWisePrefixPartition (src/device/prefix_partition/block_wise/
// BlockWisePrefixPartition.hpp:226-329) are multi-pass baselines against the decoupled
// lookback: reduce every block, scan the block reductions, then scan every block again with
// its offset.  Here: k_bw_scan<false> / k_bw_part_reduce write each tile's FP32 aggregates
// (the same tile and thread order as the decoupled kernels), k_bw_tiles turns them into
// exclusive offsets in one CTA (fixed order), and k_bw_scan<true> / k_prefix_partition<...,
// BW> scan each tile again with its offset instead of a lookback.  FP32 carries, as the
// reference's; 12 B/weight for the scan (the weights are read twice) where the decoupled scan
// moves 8.

template <bool APPLY>
__global__ __launch_bounds__(kTileThreads) void k_bw_scan(const float* __restrict__ in, uint32_t n,
                                                          float* __restrict__ out,
                                                          float* __restrict__ tile_val) {
    pdl_entry();
    __shared__ float s_w[kTileWarps];
    const uint32_t tile = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tbase = tile * kTileItems;
    const uint32_t wbase = tbase + warp * kWarpItems;
    float x[4][4];
    load_tile(in, n, tile, x);
    float lex[4], voff[4], run = 0.f;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const float t = __fadd_rn(__fadd_rn(__fadd_rn(x[v][0], x[v][1]), x[v][2]), x[v][3]);
        const float inc = warp_incl_f(t, lane);
        const float e = __shfl_up_sync(0xffffffffu, inc, 1);
        lex[v] = lane ? e : 0.f;
        voff[v] = run;
        run = __fadd_rn(run, __shfl_sync(0xffffffffu, inc, 31));
    }
    if (lane == 0) s_w[warp] = run;
    __syncthreads();
    if (warp == 0) {
        const float t = lane < kTileWarps ? s_w[lane] : 0.f;
        const float inc = warp_incl_f(t, lane);
        const float e = __shfl_up_sync(0xffffffffu, inc, 1);
        if (!APPLY && lane == kTileWarps - 1) tile_val[tile] = inc;  // the tile's aggregate
        __syncwarp();
        if (lane < kTileWarps) s_w[lane] = lane ? e : 0.f;
    }
    if constexpr (!APPLY) return;
    __syncthreads();
    const float ex = __ldg(tile_val + tile);  // exclusive offset (k_bw_tiles)
    const float wex = s_w[warp];
    const bool full = (static_cast<uint64_t>(tbase) + kTileItems <= n) &&
                      ((reinterpret_cast<uintptr_t>(out) & 15u) == 0);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        float r = __fadd_rn(__fadd_rn(wex, voff[v]), lex[v]);
        float y[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            r = __fadd_rn(r, x[v][c]);
            y[c] = __fadd_rn(ex, r);
        }
        const uint32_t e0 = wbase + v * 128 + lane * 4;
        if (full) {
            __stcs(reinterpret_cast<float4*>(out + e0), make_float4(y[0], y[1], y[2], y[3]));
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (e0 + c < n) out[e0 + c] = y[c];
        }
    }
}

// Per-tile heavy count, heavy sum and light sum (items above / not above the mean).
__global__ __launch_bounds__(kTileThreads) void k_bw_part_reduce(const float* __restrict__ w,
                                                                 uint32_t n,
                                                                 const BuildCtrl* __restrict__ ctrl,
                                                                 uint32_t* __restrict__ tc,
                                                                 float* __restrict__ th,
                                                                 float* __restrict__ tl) {
    pdl_entry();
    __shared__ uint32_t s_c[kTileWarps];
    __shared__ float s_h[kTileWarps], s_l[kTileWarps];
    const uint32_t tile = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float pivot = ctrl->mean;
    float x[4][4];
    load_tile(w, n, tile, x);
    uint32_t c = 0;
    float h = 0.f, l = 0.f;
    const uint32_t wbase = tile * kTileItems + warp * kWarpItems;
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (wbase + v * 128 + lane * 4 + k >= n) continue;
            if (x[v][k] > pivot) {
                ++c;
                h = __fadd_rn(h, x[v][k]);
            } else {
                l = __fadd_rn(l, x[v][k]);
            }
        }
    const uint32_t ic = warp_incl_u(c, lane);
    const float ih = warp_incl_f(h, lane), il = warp_incl_f(l, lane);
    if (lane == 31) {
        s_c[warp] = ic;
        s_h[warp] = ih;
        s_l[warp] = il;
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t cc = warp_incl_u(lane < kTileWarps ? s_c[lane] : 0u, lane);
        const float hh = warp_incl_f(lane < kTileWarps ? s_h[lane] : 0.f, lane);
        const float ll = warp_incl_f(lane < kTileWarps ? s_l[lane] : 0.f, lane);
        if (lane == kTileWarps - 1) {
            tc[tile] = cc;
            th[tile] = hh;
            tl[tile] = ll;
        }
    }
}

// Exclusive scans, in place, of up to three per-tile arrays (any may be null) in one CTA of
// 1024 threads: thread t sums its chunk of consecutive tiles in order, the chunk totals are
// scanned across the CTA, then each thread rewrites its chunk as exclusive prefixes.
constexpr int kBwThreads = 1024;

__global__ __launch_bounds__(kBwThreads) void k_bw_tiles(uint32_t T, uint32_t* __restrict__ c,
                                                         float* __restrict__ h,
                                                         float* __restrict__ l) {
    pdl_entry();
    __shared__ uint32_t s_c[32];
    __shared__ float s_h[32], s_l[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t chunk = (T + kBwThreads - 1) / kBwThreads;
    const uint32_t b0 = min(T, threadIdx.x * chunk), b1 = min(T, b0 + chunk);
    uint32_t sc = 0;
    float sh = 0.f, sl = 0.f;
    for (uint32_t t = b0; t < b1; ++t) {
        if (c) sc += c[t];
        if (h) sh = __fadd_rn(sh, h[t]);
        if (l) sl = __fadd_rn(sl, l[t]);
    }
    const uint32_t ic = warp_incl_u(sc, lane);
    const float ih = warp_incl_f(sh, lane), il = warp_incl_f(sl, lane);
    if (lane == 31) {
        s_c[warp] = ic;
        s_h[warp] = ih;
        s_l[warp] = il;
    }
    __syncthreads();
    if (warp == 0) {
        const uint32_t wc = warp_incl_u(s_c[lane], lane);
        const float wh = warp_incl_f(s_h[lane], lane), wl = warp_incl_f(s_l[lane], lane);
        const uint32_t ec = __shfl_up_sync(0xffffffffu, wc, 1);
        const float eh = __shfl_up_sync(0xffffffffu, wh, 1);
        const float el = __shfl_up_sync(0xffffffffu, wl, 1);
        __syncwarp();
        s_c[lane] = lane ? ec : 0u;
        s_h[lane] = lane ? eh : 0.f;
        s_l[lane] = lane ? el : 0.f;
    }
    __syncthreads();
    // exclusive start of this thread's chunk: the warp's offset plus the lanes before it
    const float eh = __shfl_up_sync(0xffffffffu, ih, 1), el = __shfl_up_sync(0xffffffffu, il, 1);
    uint32_t rc = s_c[warp] + (ic - sc);
    float rh = __fadd_rn(s_h[warp], lane ? eh : 0.f);
    float rl = __fadd_rn(s_l[warp], lane ? el : 0.f);
    for (uint32_t t = b0; t < b1; ++t) {
        if (c) {
            const uint32_t v = c[t];
            c[t] = rc;
            rc += v;
        }
        if (h) {
            const float v = h[t];
            h[t] = rh;
            rh = __fadd_rn(rh, v);
        }
        if (l) {
            const float v = l[t];
            l[t] = rl;
            rl = __fadd_rn(rl, v);
        }
    }
}

cudaError_t launch_prefix_sum_blockwise(cudaStream_t st, const float* in, uint32_t n, float* out,
                                        float* tile_scratch) {
    const uint32_t T = tiles_for(n);
    launch_pdl(k_bw_scan<false>, T, kTileThreads, 0, st, in, n, out, tile_scratch);
    launch_pdl(k_bw_tiles, 1, kBwThreads, 0, st, T, nullptr, tile_scratch, nullptr);
    launch_pdl(k_bw_scan<true>, T, kTileThreads, 0, st, in, n, out, tile_scratch);
    return cudaGetLastError();
}

cudaError_t launch_prefix_partition_blockwise(cudaStream_t st, const float* w, uint32_t n,
                                              BuildCtrl* ctrl, uint32_t* tile_scratch,
                                              uint32_t* idx_out, float* prefix_out,
                                              float* elems_out) {
    const uint32_t T = tiles_for(n);
    uint32_t* tc = tile_scratch;
    float* th = reinterpret_cast<float*>(tile_scratch + T);
    float* tl = reinterpret_cast<float*>(tile_scratch + 2 * static_cast<size_t>(T));
    launch_pdl(k_bw_part_reduce, T, kTileThreads, 0, st, w, n, ctrl, tc, th, tl);
    launch_pdl(k_bw_tiles, 1, kBwThreads, 0, st, T, tc, th, tl);
    const PartArgs a{w,       n,        ctrl,     nullptr,  nullptr,   0u,
                     0u,      &ctrl->status, idx_out, prefix_out, elems_out, nullptr,
                     tc,      th,       tl};
    launch_pdl(k_prefix_partition<false, false, false, true>, T, kTileThreads, 0, st, a, BatchView{});
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// serial split-pack: split records persisted between two kernels
// ---------------------------------------------------------------------------------

// split/scalar/shader.comp:72-133 (ScalarSplit): K = ceil(N / splitSize) records; record k - 1
// (k in [1, K)) is computeSplit at n = ceil(N * k / K) (ceilMulDiv, 64-bit), record K - 1 =
// (lightCount, heavyCount, 0).  Each split is compute_split's bisection (the same probe
// sequence, comparisons and precision options as the inline kernel).  All heavy or all
// light: every record is the final one (the shader's bisection would underflow).
template <bool R64, bool FF>
__global__ __launch_bounds__(256) void k_split_records(SplitArgs a) {
    pdl_entry();
    const uint32_t n = a.n;
    const uint32_t K = records_for(n, a.split_size);
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;  // record t: split k = t + 1
    if (t >= K) return;
    const uint32_t hc = a.ctrl->heavy_count;
    SplitRecord r{n - min(hc, n), min(hc, n), 0.0f};
    if (t + 1u < K && hc != 0u && hc < n) {
        const PackIn c{a.w,    a.idx, a.elems, a.prefix, a.prefix_lo, n, hc, n - hc,
                       a.full_light ? n - hc : n - hc - 1u, a.ctrl->mean, a.ctrl->mean_lo};
        const uint32_t nk = static_cast<uint32_t>(
            (static_cast<uint64_t>(n) * (t + 1u) + K - 1u) / K);
        compute_split<R64, FF>(c, nk, r.i, r.j, r.spill);
    }
    a.records[t] = r;
}

cudaError_t launch_split_records(cudaStream_t st, bool r64, bool full_light, const float* prefix,
                                 const float* prefix_lo, const BuildCtrl* ctrl, uint32_t n,
                                 uint32_t split_size, SplitRecord* records) {
    const SplitArgs a{nullptr, n,         ctrl,    nullptr, nullptr,    nullptr,
                      prefix,  prefix_lo, nullptr, split_size, full_light ? 1u : 0u, records};
    const uint32_t K = records_for(n, split_size);
    const uint32_t blocks = (K + 255u) / 256u;
    if (prefix_lo)
        launch_pdl(k_split_records<true, true>, blocks, 256, 0, st, a);
    else if (r64)
        launch_pdl(k_split_records<true, false>, blocks, 256, 0, st, a);
    else
        launch_pdl(k_split_records<false, false>, blocks, 256, 0, st, a);
    return cudaGetLastError();
}

// pack/scalar/float.comp (ScalarPack): one thread per subproblem [split_k, split_{k+1}) with the
// splits read from the records; the same pack loop, ownership window and status bit as the
// inline kernel (whose slot machinery k_split_pack<..., RECORDS> reuses).
cudaError_t launch_pack_records(cudaStream_t st, bool full_light, const float* w,
                                const uint32_t* idx, const float* elems, const BuildCtrl* ctrl,
                                uint32_t* status, uint32_t n, uint32_t split_size,
                                const SplitRecord* records, uint2* table) {
    // the CTA's items fit the staging window up to split size kPackWin / kSplitPack (12)
    const uint32_t stage = split_size * kSplitPack <= kPackWin ? 1u : 0u;
    const SplitArgs a{w,       n,       ctrl,   table,      idx, elems,
                      nullptr, nullptr, status, split_size, full_light ? 1u : 0u,
                      const_cast<SplitRecord*>(records), nullptr, stage};
    const uint32_t blocks = (records_for(n, split_size) + kSplitPack - 1) / kSplitPack;
    launch_split_kernel<false, false, false, true>(st, blocks, a, BatchView{});
    return cudaGetLastError();
}

// SubgroupPack's strategy (pack/subgroup/shader.comp): one warp per subproblem.  The lanes load
// the subproblem's heavy and light items 32 at a time (coalesced; without partition elements
// the 32 weight gathers are in flight together), the walk runs in lockstep with every item
// fetched from its lane by a shuffle, and each lane keeps one table entry of every 32 steps,
// written together (the serial loop carries only the residual and the decisions; each lane
// divides its entry's numerator by the mean when the group is written, so the warp issues
// one division per 32 steps).  Decisions and arithmetic are the scalar pack's operation for operation,
// so the table is bit-identical to launch_pack_records'.  (The reference's subgroup shader
// updates the residual as w + (weight - mean) and keeps a zero spill; here one arithmetic
// serves both strategies.)  Ownership: a later subproblem within kWarpLook overrides, as in
// the scalar kernel; a step back beyond that raises kStatusNonMonotone.
constexpr uint32_t kWarpLook = 31;

__device__ __forceinline__ void split_at(const SplitRecord* __restrict__ rec, uint32_t K,
                                         uint32_t k, uint32_t lc, uint32_t hc, uint32_t& i,
                                         uint32_t& j, float& spill) {
    if (k == 0u) {
        i = j = 0u;
        spill = 0.0f;
    } else if (k >= K) {
        i = lc;
        j = hc;
        spill = 0.0f;
    } else {
        const SplitRecord r = rec[k - 1u];
        i = r.i;
        j = r.j;
        spill = r.spill;
    }
}

// Is the entry at light rank / heavy position `pos` packed by one of the later subproblems
// k + 1 .. k + count?  Lane d holds split_{k+1+d} in (li, lj); subproblem k + d covers
// [split_{k+d}, max(split_{k+d+1}, split_{k+d})).  Called by all lanes of the warp.
__device__ __forceinline__ bool covered_later_warp(uint32_t li, uint32_t lj, uint32_t count,
                                                   uint32_t pos, bool light) {
    bool covered = false;
    for (uint32_t d = 1; d <= count; ++d) {
        const uint32_t ai = __shfl_sync(0xffffffffu, li, d - 1u);
        const uint32_t aj = __shfl_sync(0xffffffffu, lj, d - 1u);
        const uint32_t bi = max(__shfl_sync(0xffffffffu, li, d), ai);
        const uint32_t bj = max(__shfl_sync(0xffffffffu, lj, d), aj);
        covered = covered || (light ? (ai <= pos && pos < bi) : (aj <= pos && pos < bj));
    }
    return covered;
}

__global__ __launch_bounds__(256) void k_pack_records_warp(SplitArgs a) {
    pdl_entry();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // subproblem
    const uint32_t n = a.n;
    const uint32_t K = records_for(n, a.split_size);
    if (k >= K) return;  // whole warps
    const uint32_t hc = a.ctrl->heavy_count;
    uint2* table = a.table;
    if (hc == 0u || hc >= n) {
        const uint32_t per = (n + K - 1u) / K;
        for (uint32_t e = k * per + lane; e < min(n, (k + 1u) * per); e += 32u)
            table[e] = make_uint2(__float_as_uint(1.0f), e);
        return;
    }
    const uint32_t lc = n - hc, last = n - 1u;
    const float mean = a.ctrl->mean;
    const SplitRecord* rec = a.records;
    uint32_t i0, j0, i1, j1;
    float spill, dummy;
    split_at(rec, K, k, lc, hc, i0, j0, spill);
    split_at(rec, K, k + 1u, lc, hc, i1, j1, dummy);
    i1 = max(i1, i0);
    j1 = max(j1, j0);
    // later splits: lane d holds split_{k + 1 + d}; subproblem k + d (d >= 1) covers
    // [split_{k+d}, max(split_{k+d+1}, split_{k+d}))
    const uint32_t count = min(kWarpLook, K - 1u - k);
    uint32_t li, lj;
    split_at(rec, K, k + 1u + lane, lc, hc, li, lj, dummy);
    const bool clean = __all_sync(0xffffffffu, lane >= count || (li >= i1 && lj >= j1));
    if (lane == 0 && k + kWarpLook + 1u < K) {
        uint32_t bi, bj;
        split_at(rec, K, k + kWarpLook + 1u, lc, hc, bi, bj, dummy);
        if (bi < i1 || bj < j1) atomicOr(a.status, kStatusNonMonotone);
    }
    const uint32_t* idx = a.idx;
    const float* elems = a.elems;
    const float* w = a.w;
    auto elem_at = [&](uint32_t pos, uint32_t widx) -> float {
        return elems ? __ldg(elems + pos) : (widx < n ? __ldg(w + widx) : 0.0f);
    };
    // chunks: heavy positions hb + lane, light ranks lb + lane
    uint32_t hb = j0, lb = i0;
    uint32_t hidx = 0, lidx = 0;
    float hw = 0.0f, lw = 0.0f;
    auto load_heavy = [&]() {
        const uint32_t pos = hb + lane;
        hidx = pos < n ? __ldg(idx + pos) : 0u;
        hw = pos < n ? elem_at(pos, hidx) : 0.0f;
    };
    auto load_light = [&]() {
        const uint32_t r = lb + lane;
        lidx = r < n ? __ldg(idx + last - r) : 0u;
        lw = r < n ? elem_at(last - r, lidx) : 0.0f;
    };
    load_heavy();
    load_light();
    uint32_t i = i0, j = j0;
    float wv = spill;
    if (wv == 0.0f) wv = __shfl_sync(0xffffffffu, hw, 0);  // elem(j0): lane 0 of the heavy chunk
    // the current heavy item's original index (lane 0 of the heavy chunk); a heavy step moves
    // it to item j + 1, whose index that step fetches.  With the table-end rule (full light
    // cap, as pack()) it never leaves the heavy range.
    const bool close_last = a.full_light != 0u;
    uint32_t h = __shfl_sync(0xffffffffu, hidx, 0);
    if (close_last && j0 >= hc) h = __ldg(idx + hc - 1u);
    // pending entries: lane e holds step e of the current group of 32 -- the numerator of its
    // p (divided by the mean when the group is written, one division per lane), its alias,
    // its table index and its partition position
    uint32_t e_out = 0u, e_a = 0u, e_pos = 0u;
    float e_num = 0.0f;
    bool e_light = false, e_one = false;
    uint32_t pend = 0;
    while (i < i1 || j < j1) {
        bool heavy_step;
        if (j == j1 || j == hc)
            heavy_step = false;
        else if (i == i1 || i == lc)
            heavy_step = true;
        else
            heavy_step = wv <= mean;
        if (j + 1u - hb >= 32u) {  // keep j and j + 1 inside the heavy chunk
            hb = j;
            load_heavy();
        }
        uint32_t widx;
        float weight;
        if (heavy_step) {
            widx = __shfl_sync(0xffffffffu, hidx, j + 1u - hb);
            weight = __shfl_sync(0xffffffffu, hw, j + 1u - hb);
        } else {
            if (i - lb >= 32u) {
                lb = i;
                load_light();
            }
            widx = __shfl_sync(0xffffffffu, lidx, i - lb);
            weight = __shfl_sync(0xffffffffu, lw, i - lb);
        }
        const bool last = heavy_step && close_last && j + 1u == hc;
        if (lane == pend) {
            e_num = heavy_step ? wv : weight;
            e_a = heavy_step && !last ? widx : h;
            e_out = heavy_step ? h : widx;
            e_pos = heavy_step ? j : i;
            e_light = !heavy_step;
            e_one = last;
        }
        if (heavy_step) {
            ++j;
            if (!last) h = widx;
        } else {
            ++i;
        }
        wv = __fsub_rn(__fadd_rn(wv, weight), mean);
        if (++pend == 32u) {
            // whole warp: the shuffles of the ownership test need every lane
            const bool owned = clean || !covered_later_warp(li, lj, count, e_pos, e_light);
            if (owned && e_out < n)
                table[e_out] = make_uint2(
                    __float_as_uint(e_one ? 1.0f : __fdiv_rn(e_num, mean)), e_a);
            pend = 0;
        }
    }
    // the last, partial group
    const bool owned = clean || !covered_later_warp(li, lj, count, e_pos, e_light);
    if (lane < pend && owned && e_out < n)
        table[e_out] = make_uint2(__float_as_uint(e_one ? 1.0f : __fdiv_rn(e_num, mean)), e_a);
}

cudaError_t launch_pack_records_warp(cudaStream_t st, bool full_light, const float* w,
                                     const uint32_t* idx, const float* elems,
                                     const BuildCtrl* ctrl, uint32_t* status, uint32_t n,
                                     uint32_t split_size, const SplitRecord* records,
                                     uint2* table) {
    const SplitArgs a{w,       n,       ctrl,   table,      idx, elems,
                      nullptr, nullptr, status, split_size, full_light ? 1u : 0u,
                      const_cast<SplitRecord*>(records)};
    const uint64_t threads = static_cast<uint64_t>(records_for(n, split_size)) * 32u;
    launch_pdl(k_pack_records_warp, static_cast<unsigned>((threads + 255u) / 256u), 256, 0, st, a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------------

// One CTA per distribution fills its ranges of the tile, split-block and sampling-block maps.
__global__ __launch_bounds__(256) void k_batch_maps(const DistDesc* __restrict__ dist,
                                                    uint32_t* __restrict__ tile_map,
                                                    uint32_t* __restrict__ split_map,
                                                    uint32_t* __restrict__ sample_map,
                                                    uint32_t split_size) {
    const uint32_t d = blockIdx.x;
    const DistDesc D = dist[d];
    if (D.w) {
        const uint32_t nt = tiles_for(D.n);
        for (uint32_t i = threadIdx.x; i < nt; i += blockDim.x) tile_map[D.tile0 + i] = d;
        const uint32_t ns = split_blocks_for(D.n, split_size);
        for (uint32_t i = threadIdx.x; i < ns; i += blockDim.x) split_map[D.split0 + i] = d;
    }
    if (D.out) {
        const uint64_t nb = alias_blocks_for(D.s);
        for (uint64_t i = threadIdx.x; i < nb; i += blockDim.x) sample_map[D.sample0 + i] = d;
    }
}

cudaError_t launch_batch_maps(cudaStream_t st, const DistDesc* dist, uint32_t count,
                              uint32_t* tile_map, uint32_t* split_map, uint32_t* sample_map,
                              uint32_t split_size) {
    if (count == 0) return cudaSuccess;
    k_batch_maps<<<count, 256, 0, st>>>(dist, tile_map, split_map, sample_map, split_size);
    return cudaGetLastError();
}

// total mass -> prefix-partition -> split+pack over every distribution of the batch that
// has weights: four launches (the split descent included), whatever the number and sizes of
// the distributions.
cudaError_t launch_batch_build(cudaStream_t st, uint32_t precision, bool r64, const BatchView& b) {
    if (b.tiles == 0) return cudaSuccess;
    launch_pdl(k_total_mass<true>, b.tiles, kTileThreads, 0, st, nullptr, 0u, b.partials, nullptr, b);
    const PartArgs pa{nullptr,    0u,       nullptr,  b.lb,   b.states,  b.cap_tiles,
                      kSpinLimit, b.status, b.idx,    b.prefix, b.elems, b.prefix_lo};
    part_dispatch<true>(st, precision, b.tiles, pa, b);
    const SplitArgs sa{nullptr,  0u,          nullptr,  nullptr,      b.idx,
                       b.elems,  b.prefix,    b.prefix_lo, b.status, b.split_size,
                       b.full_light, nullptr, nullptr, kStageEntriesMode};
    if (b.descent && b.split_blocks) {
        const uint32_t g = (b.split_blocks + 255u) / 256u;
        if (precision == 2)
            launch_pdl(k_split_descent<true, true>, g, 256, 0, st, sa, b);
        else
            launch_pdl(k_split_descent<false, true>, g, 256, 0, st, sa, b);
    }
    split_dispatch<true>(st, r64, precision == 2, b.split_blocks, sa, b);
    return cudaGetLastError();
}

}  // namespace wrs

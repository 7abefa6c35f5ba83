// wrs_build.cu -- build kernels of the WRS hot path for sm_103a.
//
//   k_total_mass        total mass / mean                 (reference: src/device/mean/atomic/shader.comp)
//   k_prefix_partition  fused heavy/light stable partition + heavy and light inclusive
//                       prefix sums + heavyCount, single pass with decoupled lookback
//                                                          (src/device/prefix_partition/decoupled/shader.comp)
//   k_scan              inclusive FP32 scan, single pass    (src/device/prefix_sum/decoupled/shader.comp)
//   k_split_pack        PSA split search + pack, one thread per split
//                                                          (src/device/wrs/alias/psa/splitpack/inline/shader.comp)
//
// All lookback kernels take their tile index from an atomic ticket (a tile only ever
// waits for tiles whose CTAs already run), bound every spin (kSpinLimit polls, then
// raise kStatusTimeout and continue), and clean up after themselves: the state buffer
// is double-buffered by an epoch; each launch clears the half the next launch will use,
// and its last CTA resets the ticket and advances the epoch.
#include "wrs_device.cuh"
#include "wrs_internal.cuh"

namespace wrs {

// ---------------------------------------------------------------------------------
// total mass
// ---------------------------------------------------------------------------------

// Per-thread compensated FP32 accumulation (two-sum) over 16-byte vector loads, FP64
// across threads and CTAs.  The last CTA sums the per-CTA partials in a fixed order, so
// the result depends only on N and the data (deterministic).
__global__ __launch_bounds__(kMassThreads) void k_total_mass(const float* __restrict__ w,
                                                             uint32_t n,
                                                             double* __restrict__ partials,
                                                             BuildCtrl* __restrict__ ctrl) {
    __shared__ double s_red[kMassThreads / 32];
    __shared__ bool s_last;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nth = gridDim.x * blockDim.x;

    ff acc = {0.0f, 0.0f};
    uint32_t head = static_cast<uint32_t>(((16u - (reinterpret_cast<uintptr_t>(w) & 15u)) & 15u) / 4u);
    if (head > n) head = n;
    if (tid < head) acc = carry_add<true>(acc, ff{__ldg(w + tid), 0.0f});
    const float4* w4 = reinterpret_cast<const float4*>(w + head);
    const uint32_t n4 = (n - head) / 4u;
    uint32_t i = tid;
    for (; i + 3u * nth < n4; i += 4u * nth) {
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = __ldcs(w4 + i + u * nth);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            acc = carry_add<true>(acc, ff{v[u].x, 0.0f});
            acc = carry_add<true>(acc, ff{v[u].y, 0.0f});
            acc = carry_add<true>(acc, ff{v[u].z, 0.0f});
            acc = carry_add<true>(acc, ff{v[u].w, 0.0f});
        }
    }
    for (; i < n4; i += nth) {
        float4 v = __ldcs(w4 + i);
        acc = carry_add<true>(acc, ff{v.x, 0.0f});
        acc = carry_add<true>(acc, ff{v.y, 0.0f});
        acc = carry_add<true>(acc, ff{v.z, 0.0f});
        acc = carry_add<true>(acc, ff{v.w, 0.0f});
    }
    for (uint32_t t = head + 4u * n4 + tid; t < n; t += nth)
        acc = carry_add<true>(acc, ff{__ldg(w + t), 0.0f});

    double d = __dadd_rn(static_cast<double>(acc.hi), static_cast<double>(acc.lo));
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) d = __dadd_rn(d, __shfl_xor_sync(0xffffffffu, d, m));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) s_red[warp] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int k = 0; k < kMassThreads / 32; ++k) b = __dadd_rn(b, s_red[k]);
        partials[blockIdx.x] = b;
        __threadfence();
        uint32_t prev = atomicAdd(&ctrl->mass_done, 1u);
        s_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double t = 0.0;
    for (uint32_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) t = __dadd_rn(t, __ldcg(partials + k));
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) t = __dadd_rn(t, __shfl_xor_sync(0xffffffffu, t, m));
    if (lane == 0) s_red[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0.0;
        for (int k = 0; k < kMassThreads / 32; ++k) total = __dadd_rn(total, s_red[k]);
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
    uint32_t blocks = static_cast<uint32_t>((static_cast<uint64_t>(n) + kMassThreads * 16 - 1) /
                                            (kMassThreads * 16));
    if (blocks < 1) blocks = 1;
    if (blocks > static_cast<uint32_t>(kMassMaxBlocks)) blocks = kMassMaxBlocks;
    k_total_mass<<<blocks, kMassThreads, 0, st>>>(w, n, partials, ctrl);
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

// ---------------------------------------------------------------------------------
// fused prefix-partition
// ---------------------------------------------------------------------------------

struct PartCarry {
    ff h, l;
    uint32_t c;
};

template <bool COMP>
__device__ __forceinline__ PartCarry part_add(PartCarry a, PartCarry b) {
    return {carry_add<COMP>(a.h, b.h), carry_add<COMP>(a.l, b.l), a.c + b.c};
}

template <bool COMP>
__device__ __forceinline__ PartCarry part_warp_sum(PartCarry v) {
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
        PartCarry o{shfl_xor_ff(v.h, m), shfl_xor_ff(v.l, m), __shfl_xor_sync(0xffffffffu, v.c, m)};
        v = part_add<COMP>(v, o);
    }
    return v;
}

// Runs on warp 0 only; returns the exclusive prefix of `tile` in every lane.
template <bool COMP>
__device__ PartCarry part_lookback(const PartState* st, uint32_t tile, uint32_t* status,
                                   uint32_t spin_limit) {
    const int lane = threadIdx.x & 31;
    PartCarry ex{{0.f, 0.f}, {0.f, 0.f}, 0u};
    int64_t base = static_cast<int64_t>(tile) - 1;
    uint32_t spins = 0;
    for (;;) {
        const int64_t pos = base - lane;
        int s = 2;
        PartCarry v{{0.f, 0.f}, {0.f, 0.f}, 0u};
        if (pos >= 0) {
            const unsigned long long* q = reinterpret_cast<const unsigned long long*>(st + pos);
            unsigned long long ah, al, ac, pc, ph, pl;
            ld_relaxed_v2(q + 0, ah, al);
            ld_relaxed_v2(q + 2, ac, pc);
            ld_relaxed_v2(q + 4, ph, pl);
            if (ff_ready(ph) && ff_ready(pl) && cnt_ready(pc)) {
                s = 2;
                v = {unpack_ff(ph), unpack_ff(pl), static_cast<uint32_t>(pc)};
            } else if (ff_ready(ah) && ff_ready(al) && cnt_ready(ac)) {
                s = 1;
                v = {unpack_ff(ah), unpack_ff(al), static_cast<uint32_t>(ac)};
            } else {
                s = 0;
            }
        }
        const unsigned nr = __ballot_sync(0xffffffffu, s == 0);
        const unsigned dn = __ballot_sync(0xffffffffu, s == 2);
        const int first_nr = nr ? __ffs(nr) - 1 : 32;
        const int first_dn = dn ? __ffs(dn) - 1 : 32;
        const bool finish = first_dn < first_nr;
        const int take = finish ? first_dn + 1 : first_nr;
        if (take > 0) {
            PartCarry c = lane < take ? v : PartCarry{{0.f, 0.f}, {0.f, 0.f}, 0u};
            ex = part_add<COMP>(ex, part_warp_sum<COMP>(c));
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

__device__ __forceinline__ void part_publish_agg(PartState* s, const PartCarry& a) {
    unsigned long long* q = reinterpret_cast<unsigned long long*>(s);
    st_relaxed_v2(q + 0, pack_ff(a.h), pack_ff(a.l));
    st_relaxed(q + 2, pack_cnt(a.c));
}
__device__ __forceinline__ void part_publish_pre(PartState* s, const PartCarry& p) {
    unsigned long long* q = reinterpret_cast<unsigned long long*>(s);
    st_relaxed_v2(q + 4, pack_ff(p.h), pack_ff(p.l));
    st_relaxed(q + 3, pack_cnt(p.c));
}

// One CTA = one tile of 4096 weights; warp w owns items [w*512, w*512+512) of the tile and
// lane L holds, for v = 0..3, the 4 consecutive items at v*128 + L*4 (16-byte loads, fully
// coalesced).  Heavy (w > mean) items go to idx[heavyRank], light items to
// idx[N-1-lightRank]; prefix[] holds the inclusive heavy resp. light prefix sum, elems[] the
// weight (shader.comp:329-361).  FFOUT (with the compensated carry) also writes prefix_lo[],
// the low word of the prefix as a float-float pair (prefix[] is its high word).
template <bool COMP, bool FFOUT>
__global__ __launch_bounds__(kTileThreads) void k_prefix_partition(
    const float* __restrict__ w, uint32_t n, BuildCtrl* __restrict__ ctrl,
    PartState* __restrict__ states, uint32_t cap_tiles, uint32_t* __restrict__ idx_out,
    float* __restrict__ prefix_out, float* __restrict__ elems_out,
    float* __restrict__ prefix_lo_out, uint32_t spin_limit) {
    __shared__ float s_wh[kTileWarps], s_wl[kTileWarps];
    __shared__ uint32_t s_wc[kTileWarps];
    __shared__ ff s_fh[kTileWarps], s_fl[kTileWarps];  // FFOUT: exact warp totals
    __shared__ PartCarry s_ex;
    __shared__ PartCarry s_agg;

    PartState* cur;
    const uint32_t tile = lookback_begin(&ctrl->part, states, cap_tiles, cur);
    const float pivot = ctrl->mean;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tbase = tile * kTileItems;
    const uint32_t wbase = tbase + warp * kWarpItems;

    float x[4][4];
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
                x[v][c] = e < n ? __ldg(w + e) : 0.0f;  // out of range: light, weight 0
            }
    }

    // per-v warp scans of the thread totals
    float lex_h[4], lex_l[4], voff_h[4], voff_l[4];
    uint32_t lex_c[4], voff_c[4];
    float run_h = 0.f, run_l = 0.f;
    uint32_t run_c = 0;
    // FFOUT: the tile aggregate is also summed exactly (float-float), so that its FP32
    // rounding does not accumulate along the lookback carry
    ff fh{0.f, 0.f}, fl{0.f, 0.f};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        float th = 0.f, tl = 0.f;
        uint32_t tc = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (x[v][c] > pivot) {
                if constexpr (FFOUT)
                    fh = ff_add_f(fh, x[v][c]);
                else
                    th = __fadd_rn(th, x[v][c]);
                ++tc;
            } else {
                if constexpr (FFOUT)
                    fl = ff_add_f(fl, x[v][c]);
                else
                    tl = __fadd_rn(tl, x[v][c]);
            }
        }
        uint32_t ic = warp_incl_u(tc, lane);
        uint32_t ec = __shfl_up_sync(0xffffffffu, ic, 1);
        lex_c[v] = lane ? ec : 0u;
        voff_c[v] = run_c;
        run_c += __shfl_sync(0xffffffffu, ic, 31);
        if constexpr (!FFOUT) {
            // FP32 local scans (the float-float mode redoes them exactly after the lookback)
            float ih = warp_incl_f(th, lane), il = warp_incl_f(tl, lane);
            float eh = __shfl_up_sync(0xffffffffu, ih, 1), el = __shfl_up_sync(0xffffffffu, il, 1);
            lex_h[v] = lane ? eh : 0.f;
            lex_l[v] = lane ? el : 0.f;
            voff_h[v] = run_h;
            voff_l[v] = run_l;
            run_h = __fadd_rn(run_h, __shfl_sync(0xffffffffu, ih, 31));
            run_l = __fadd_rn(run_l, __shfl_sync(0xffffffffu, il, 31));
        }
    }
    if constexpr (FFOUT) {
        fh = ff_warp_total(fh);
        fl = ff_warp_total(fl);
    }
    if (lane == 0) {
        s_wh[warp] = run_h;
        s_wl[warp] = run_l;
        s_wc[warp] = run_c;
        if constexpr (FFOUT) {
            s_fh[warp] = fh;
            s_fl[warp] = fl;
        }
    }
    __syncthreads();
    if (warp == 0) {
        float th = lane < kTileWarps ? s_wh[lane] : 0.f;
        float tl = lane < kTileWarps ? s_wl[lane] : 0.f;
        uint32_t tc = lane < kTileWarps ? s_wc[lane] : 0u;
        float ih = warp_incl_f(th, lane), il = warp_incl_f(tl, lane);
        uint32_t ic = warp_incl_u(tc, lane);
        float eh = __shfl_up_sync(0xffffffffu, ih, 1), el = __shfl_up_sync(0xffffffffu, il, 1);
        uint32_t ec = __shfl_up_sync(0xffffffffu, ic, 1);
        PartCarry agg{{__shfl_sync(0xffffffffu, ih, kTileWarps - 1), 0.f},
                      {__shfl_sync(0xffffffffu, il, kTileWarps - 1), 0.f},
                      __shfl_sync(0xffffffffu, ic, kTileWarps - 1)};
        ff fxh{0.f, 0.f}, fxl{0.f, 0.f};  // FFOUT: exact warp-exclusive offsets
        if constexpr (FFOUT) {
            const ff ith = ff_warp_incl(lane < kTileWarps ? s_fh[lane] : ff{0.f, 0.f}, lane);
            const ff itl = ff_warp_incl(lane < kTileWarps ? s_fl[lane] : ff{0.f, 0.f}, lane);
            agg.h = ff_shfl(ith, kTileWarps - 1);
            agg.l = ff_shfl(itl, kTileWarps - 1);
            fxh = ff_shfl_up_excl(ith, lane);
            fxl = ff_shfl_up_excl(itl, lane);
        }
        __syncwarp();
        if (lane < kTileWarps) {
            s_wh[lane] = lane ? eh : 0.f;
            s_wl[lane] = lane ? el : 0.f;
            s_wc[lane] = lane ? ec : 0u;
            if constexpr (FFOUT) {
                s_fh[lane] = fxh;
                s_fl[lane] = fxl;
            }
        }
        PartCarry ex{{0.f, 0.f}, {0.f, 0.f}, 0u};
        if (tile == 0) {
            if (lane == 0) {
                part_publish_agg(cur, agg);
                part_publish_pre(cur, agg);
            }
        } else {
            if (lane == 0) part_publish_agg(cur + tile, agg);
            ex = part_lookback<COMP>(cur, tile, &ctrl->status, spin_limit);
            if (lane == 0) part_publish_pre(cur + tile, part_add<COMP>(ex, agg));
        }
        if (lane == 0) {
            s_ex = ex;
            s_agg = agg;
        }
    }
    __syncthreads();

    const PartCarry ex = s_ex;
    const uint32_t light_before = tbase - ex.c;  // light items in tiles before this one
    const float wh = s_wh[warp], wl = s_wl[warp];
    const uint32_t wc = s_wc[warp];
    // FFOUT: float-float running offsets (warp-exclusive, then per-v warp totals)
    ff oh{0.f, 0.f}, ol{0.f, 0.f};
    if constexpr (FFOUT) {
        oh = s_fh[warp];
        ol = s_fl[warp];
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        float rh = 0.f, rl = 0.f;
        ff fr_h{0.f, 0.f}, fr_l{0.f, 0.f};
        if constexpr (FFOUT) {
            // exact local scan: thread totals, float-float warp scan, running offsets
            ff th{0.f, 0.f}, tl{0.f, 0.f};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (x[v][c] > pivot)
                    th = ff_add_f(th, x[v][c]);
                else
                    tl = ff_add_f(tl, x[v][c]);
            }
            const ff ih = ff_warp_incl(th, lane), il = ff_warp_incl(tl, lane);
            fr_h = carry_add<true>(oh, ff_shfl_up_excl(ih, lane));
            fr_l = carry_add<true>(ol, ff_shfl_up_excl(il, lane));
            oh = carry_add<true>(oh, ff_shfl(ih, 31));
            ol = carry_add<true>(ol, ff_shfl(il, 31));
        } else {
            rh = __fadd_rn(__fadd_rn(wh, voff_h[v]), lex_h[v]);
            rl = __fadd_rn(__fadd_rn(wl, voff_l[v]), lex_l[v]);
        }
        uint32_t rc = wc + voff_c[v] + lex_c[v];  // heavy items before this one in the tile
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const uint32_t local = warp * kWarpItems + v * 128 + lane * 4 + c;
            const uint32_t e = tbase + local;
            if (e < n) {
                const float xv = x[v][c];
                uint32_t pos;
                ff val;
                if (xv > pivot) {
                    pos = ex.c + rc;
                    if constexpr (FFOUT) {
                        fr_h = ff_add_f(fr_h, xv);
                        val = carry_add<true>(ex.h, fr_h);
                    } else {
                        rh = __fadd_rn(rh, xv);
                        val = {carry_apply<COMP>(ex.h, rh), 0.f};
                    }
                    ++rc;
                } else {
                    pos = n - 1u - (light_before + (local - rc));
                    if constexpr (FFOUT) {
                        fr_l = ff_add_f(fr_l, xv);
                        val = carry_add<true>(ex.l, fr_l);
                    } else {
                        rl = __fadd_rn(rl, xv);
                        val = {carry_apply<COMP>(ex.l, rl), 0.f};
                    }
                }
                if (pos < n) {  // always true unless a lookback wait gave up
                    idx_out[pos] = e;
                    prefix_out[pos] = val.hi;
                    if constexpr (FFOUT) prefix_lo_out[pos] = val.lo;
                    if (elems_out) elems_out[pos] = xv;
                }
            }
        }
    }
    if (threadIdx.x == 0 && tile == (n - 1u) / kTileItems) ctrl->heavy_count = ex.c + s_agg.c;
    lookback_end(&ctrl->part);
}

cudaError_t launch_prefix_partition(cudaStream_t st, bool comp, const float* w, uint32_t n,
                                    BuildCtrl* ctrl, PartState* states, uint32_t cap_tiles,
                                    uint32_t* idx_out, float* prefix_out, float* elems_out,
                                    float* prefix_lo_out) {
    const uint32_t tiles = tiles_for(n);
    if (prefix_lo_out)
        k_prefix_partition<true, true><<<tiles, kTileThreads, 0, st>>>(
            w, n, ctrl, states, cap_tiles, idx_out, prefix_out, elems_out, prefix_lo_out,
            kSpinLimit);
    else if (comp)
        k_prefix_partition<true, false><<<tiles, kTileThreads, 0, st>>>(
            w, n, ctrl, states, cap_tiles, idx_out, prefix_out, elems_out, nullptr, kSpinLimit);
    else
        k_prefix_partition<false, false><<<tiles, kTileThreads, 0, st>>>(
            w, n, ctrl, states, cap_tiles, idx_out, prefix_out, elems_out, nullptr, kSpinLimit);
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
    const int lane = threadIdx.x & 31;
    ff ex{0.f, 0.f};
    int64_t base = static_cast<int64_t>(tile) - 1;
    uint32_t spins = 0;
    for (;;) {
        const int64_t pos = base - lane;
        int s = 2;
        ff v{0.f, 0.f};
        if (pos >= 0) {
            unsigned long long a, p;
            ld_relaxed_v2(reinterpret_cast<const unsigned long long*>(st + pos), a, p);
            if (ff_ready(p)) {
                s = 2;
                v = unpack_ff(p);
            } else if (ff_ready(a)) {
                s = 1;
                v = unpack_ff(a);
            } else {
                s = 0;
            }
        }
        const unsigned nr = __ballot_sync(0xffffffffu, s == 0);
        const unsigned dn = __ballot_sync(0xffffffffu, s == 2);
        const int first_nr = nr ? __ffs(nr) - 1 : 32;
        const int first_dn = dn ? __ffs(dn) - 1 : 32;
        const bool finish = first_dn < first_nr;
        const int take = finish ? first_dn + 1 : first_nr;
        if (take > 0) {
            ff c = lane < take ? v : ff{0.f, 0.f};
            ex = carry_add<COMP>(ex, ff_warp_sum<COMP>(c));
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

template <bool COMP>
__global__ __launch_bounds__(kTileThreads) void k_scan(const float* __restrict__ in, uint32_t n,
                                                       float* __restrict__ out,
                                                       BuildCtrl* __restrict__ ctrl,
                                                       ScanState* __restrict__ states,
                                                       uint32_t cap_tiles, uint32_t spin_limit) {
    __shared__ float s_w[kTileWarps];
    __shared__ ff s_ex;
    ScanState* cur;
    const uint32_t tile = lookback_begin(&ctrl->scan, states, cap_tiles, cur);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tbase = tile * kTileItems;
    const uint32_t wbase = tbase + warp * kWarpItems;
    const bool full = (static_cast<uint64_t>(tbase) + kTileItems <= n) &&
                      ((reinterpret_cast<uintptr_t>(in) & 15u) == 0) &&
                      ((reinterpret_cast<uintptr_t>(out) & 15u) == 0);
    float x[4][4];
    if (full) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            float4 q = __ldcs(reinterpret_cast<const float4*>(in + wbase + v * 128 + lane * 4));
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
                x[v][c] = e < n ? __ldg(in + e) : 0.0f;
            }
    }
    float lex[4], voff[4], run = 0.f;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        float t = __fadd_rn(__fadd_rn(__fadd_rn(x[v][0], x[v][1]), x[v][2]), x[v][3]);
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
        unsigned long long* q = reinterpret_cast<unsigned long long*>(cur + tile);
        if (tile == 0) {
            if (lane == 0) st_relaxed_v2(q, pack_ff(agg), pack_ff(agg));
        } else {
            if (lane == 0) st_relaxed(q, pack_ff(agg));
            ex = scan_lookback<COMP>(cur, tile, &ctrl->status, spin_limit);
            if (lane == 0) st_relaxed(q + 1, pack_ff(carry_add<COMP>(ex, agg)));
        }
        if (lane == 0) s_ex = ex;
    }
    __syncthreads();
    const ff ex = s_ex;
    const float wex = s_w[warp];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        float r = __fadd_rn(__fadd_rn(wex, voff[v]), lex[v]);
        float y[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            r = __fadd_rn(r, x[v][c]);
            y[c] = carry_apply<COMP>(ex, r);
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
    lookback_end(&ctrl->scan);
}

cudaError_t launch_scan(cudaStream_t st, bool comp, const float* in, uint32_t n, float* out,
                        BuildCtrl* ctrl, ScanState* states, uint32_t cap_tiles,
                        uint32_t spin_limit) {
    const uint32_t tiles = tiles_for(n);
    if (comp)
        k_scan<true><<<tiles, kTileThreads, 0, st>>>(in, n, out, ctrl, states, cap_tiles, spin_limit);
    else
        k_scan<false><<<tiles, kTileThreads, 0, st>>>(in, n, out, ctrl, states, cap_tiles, spin_limit);
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

__device__ __forceinline__ float elem_at(const PackIn& c, uint32_t pos) {
    if (c.elems) return __ldg(c.elems + pos);
    const uint32_t widx = __ldg(c.idx + pos);
    return widx < c.n ? __ldg(c.w + widx) : 0.f;
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

__device__ void pack(const PackIn& c, uint2* __restrict__ table, uint32_t i0, uint32_t i1,
                     uint32_t j0, uint32_t j1, float spill, const LaterSplits* later) {
    uint32_t i = i0, j = j0;
    float wv = spill;
    if (wv == 0.0f) wv = elem_at(c, j);
    const uint32_t last_light = c.n - 1u;
    while (i < i1 || j < j1) {
        bool heavy_step;
        if (j == j1 || j == c.hc)
            heavy_step = false;
        else if (i == i1 || i == c.lc)
            heavy_step = true;
        else
            heavy_step = wv <= c.mean;
        const uint32_t h = __ldg(c.idx + j);
        const uint32_t pos = heavy_step ? j + 1u : last_light - i;
        const uint32_t widx = __ldg(c.idx + pos);
        // widx < n holds for any partition this library wrote; the guards keep a corrupt
        // one (e.g. after a lookback wait gave up) from reading or writing out of bounds
        const float weight = c.elems ? __ldg(c.elems + pos) : (widx < c.n ? __ldg(c.w + widx) : 0.f);
        float p;
        uint32_t tidx, al;
        bool owned = true;
        if (heavy_step) {
            p = __fdiv_rn(wv, c.mean);
            al = widx;
            tidx = h;
            if (later) owned = !covered_later(*later, j, false);
            ++j;
        } else {
            p = __fdiv_rn(weight, c.mean);
            al = h;
            tidx = widx;
            if (later) owned = !covered_later(*later, i, true);
            ++i;
        }
        if (owned && tidx < c.n) table[tidx] = make_uint2(__float_as_uint(p), al);
        wv = __fsub_rn(__fadd_rn(wv, weight), c.mean);
    }
}

// Thread t of CTA b computes split k = b*kSplitPack + t (k in [0, K]) and packs subproblem
// k = [split_k, split_{k+1}) for t < kSplitPack, k < K; split_{k+1} comes from the
// neighbouring thread through shared memory (shader.comp:225-270).  The last
// kSplitLook + 1 threads only compute look-ahead splits for the ownership window.
constexpr int kSplitPack = kSplitThreads - kSplitLook - 1;

template <bool R64, bool FF>
__global__ __launch_bounds__(kSplitThreads) void k_split_pack(
    const float* __restrict__ w, const uint32_t* __restrict__ idx,
    const float* __restrict__ elems, const float* __restrict__ prefix,
    const float* __restrict__ prefix_lo, const BuildCtrl* __restrict__ ctrl, uint32_t* status,
    uint32_t n, uint32_t K, uint32_t split_size, uint32_t full_light,
    uint2* __restrict__ table) {
    __shared__ uint32_t s_i[kSplitThreads], s_j[kSplitThreads];
    __shared__ float s_spill[kSplitThreads];
    const uint32_t hc = ctrl->heavy_count;
    if (hc == 0u || hc >= n) {
        // degenerate (all items light or all heavy): every bucket keeps itself
        const uint32_t nth = gridDim.x * blockDim.x;
        for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += nth)
            table[e] = make_uint2(__float_as_uint(1.0f), e);
        return;
    }
    PackIn c{w,      idx,    elems,  prefix, prefix_lo, n, hc,
             n - hc, full_light ? n - hc : n - hc - 1u, ctrl->mean, ctrl->mean_lo};
    const uint32_t k = blockIdx.x * kSplitPack + threadIdx.x;
    uint32_t si = c.lc, sj = hc;  // past split K: the final split
    float sp = 0.f;
    if (k == 0u) {
        si = 0;
        sj = 0;
    } else if (k < K) {
        compute_split<R64, FF>(c, k * split_size, si, sj, sp);
    }
    s_i[threadIdx.x] = si;
    s_j[threadIdx.x] = sj;
    s_spill[threadIdx.x] = sp;
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= kSplitPack || k >= K) return;
    const uint32_t i1 = max(s_i[t + 1], si), j1 = max(s_j[t + 1], sj);
    const int count = static_cast<int>(min(static_cast<uint32_t>(kSplitLook), K - 1u - k));
    bool clean = true;
    for (int d = 1; d <= count; ++d)
        clean = clean && s_i[t + d] >= i1 && s_j[t + d] >= j1;
    // a step back reaching past the window cannot be resolved here: report it
    if (k + kSplitLook + 1u < K && (s_i[t + kSplitLook + 1] < i1 || s_j[t + kSplitLook + 1] < j1))
        atomicOr(status, kStatusNonMonotone);
    const LaterSplits later{s_i, s_j, t, count};
    pack(c, table, si, i1, sj, j1, sp, clean ? nullptr : &later);
}

cudaError_t launch_split_pack(cudaStream_t st, bool r64, bool full_light, const float* w,
                              const uint32_t* idx, const float* elems, const float* prefix,
                              const float* prefix_lo, const BuildCtrl* ctrl, uint32_t* status,
                              uint32_t n, uint32_t split_size, uint2* table) {
    uint32_t K = n / split_size;
    if (K == 0) K = 1;
    const uint32_t blocks = (K + kSplitPack - 1) / kSplitPack;
    if (prefix_lo)
        k_split_pack<true, true><<<blocks, kSplitThreads, 0, st>>>(
            w, idx, elems, prefix, prefix_lo, ctrl, status, n, K, split_size, full_light, table);
    else if (r64)
        k_split_pack<true, false><<<blocks, kSplitThreads, 0, st>>>(
            w, idx, elems, prefix, nullptr, ctrl, status, n, K, split_size, full_light, table);
    else
        k_split_pack<false, false><<<blocks, kSplitThreads, 0, st>>>(
            w, idx, elems, prefix, nullptr, ctrl, status, n, K, split_size, full_light, table);
    return cudaGetLastError();
}

}  // namespace wrs

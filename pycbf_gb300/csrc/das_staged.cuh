// Tabbed delay-and-sum with channel windows staged in shared memory by TMA.
//
// The pixels of a CTA (a "tile": 128 consecutive table columns, which the
// host stores in Morton order of their delays) need, for each (tx, rx)
// channel, only the samples between the smallest and largest delay of the
// tile's pixels that the receive can reach.  A plan, built once per table set
// (tabbed_plan_kernel), records per tile the receives that can contribute at
// all (the exact reject fl(max|apodtx| * |apodrx|) >= thresh of at least one
// pixel) and, per live receive and transmit, that window: the exact index rule
// of the taps applied to the smallest and largest delay sum fl(tautx + taurx)
// over the pixels the receive reaches (indices are monotonic in the delay, so
// every contributing tap falls inside), aligned to 16 bytes.  In the main
// kernel one warp per live receive issues one cp.async.bulk per transmit into
// a 4-stage ring, completing on an mbarrier; all warps then gather from
// shared memory.  A receive whose windows exceed a stage is not staged and its
// taps gather from global memory instead.
//
// Every mbarrier wait is bounded.  A wait that runs out marks the CTA's
// outputs NaN, sets the plan's status word, waits (bounded) for its copies in
// flight and returns.
#pragma once

#include <algorithm>

#include "das_impl.cuh"

namespace pgb {

// Four stages of 10.5 KB: with the receive codes a CTA holds ~43 KB of shared
// memory, so five CTAs (20 warps) fit an SM -- the kernel waits on short
// dependency chains and on loads, and 16 warps per SM measured 5 % slower
// (12 warps: 15 % slower).  A receive whose windows exceed a stage (about 5 %
// of the live receive-tiles of the 128-element plane-wave workload) is
// gathered from global memory instead.
constexpr int kStages = 4;
constexpr int kStageBytes = 10752;
constexpr unsigned kWaitLimit = 1u << 30;  // polls; the ~1 s clock bound ends a wait first

// plan layout (int32 words): [0] status, [1] work-queue head of the staged
// kernel, [2] number of block items, [3] pad, then per tile a record of
// plan_tile_words(nrx) words:
//   [0] nlive, [1..3] pad, then per live receive k (in receive order) 16 words
//   at 4 + 16 k: [0] code (receive index, | kUnstaged when its windows exceed
//   a stage), [1] total staged elements, [2..3] pad, [4 + t] the window of
//   transmit t: first element e0 | (elements << 19) (staged receives; the
//   stage holds the windows one after another in transmit order)
// then the tile order (one int per tile, most live receives first), a
// per-tile counter, the block items (int4 each: tile, first and one-past-last
// position in the tile's live list, block ordinal << 16 | blocks of the
// tile; largest first) and the partial sums of multi-block tiles (kBlock
// floats per tile and block).
//
// Receives are summed in blocks of kRxBlock consecutive receive indices:
// the image is sum over blocks (in order) of the block's sequential sum, in
// every kernel (staged, generic, batched), so all of them give the same bits.
// A single-frame staged launch makes each (tile, block with live receives)
// one work item -- the heaviest tiles (every receive live) no longer outlast
// the average CTA's share -- and the last item of a tile to finish adds the
// tile's block sums in block order.
constexpr int kRxBlock = kRxBlockSum;
constexpr int kRxWords = 16;           // plan words per live receive
constexpr int kUnstaged = 0x40000000;  // receive code flag: gathered from global memory
constexpr int kCodeFlags = kUnstaged;
constexpr int kWinBits = 19;           // window start bits (the staged path needs nt <= 2^19)
constexpr int kStagedMaxNt = 1 << kWinBits;
__host__ __device__ inline long long plan_tile_words(int nrx) {
    return 4 + (long long)kRxWords * nrx;
}
constexpr int kPlanHeaderWords = 4;
struct PlanLayout {
    long long tiles, tile_words, max_blocks, order, counters, items, partials, total;
};
__host__ __device__ inline PlanLayout plan_layout(long long np, int ntx, int nrx) {
    (void)ntx;
    PlanLayout L;
    L.tiles = (np + kBlock - 1) / kBlock;
    L.tile_words = plan_tile_words(nrx);
    L.max_blocks = (nrx + kRxBlock - 1) / kRxBlock;
    L.order = kPlanHeaderWords + L.tiles * L.tile_words;
    L.counters = L.order + L.tiles;
    L.items = (L.counters + L.tiles + 3) & ~3LL;  // int4: 16-byte aligned
    L.partials = L.items + 4 * L.tiles * L.max_blocks;
    L.total = L.partials + L.tiles * L.max_blocks * kBlock;
    return L;
}

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// try_wait: true once the phase with this parity has completed (a suspend-time
// hint makes each wait ~500 cycles slower to wake, so none is given)
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after kWaitLimit polls or `limit` SM cycles (by
// default 2^31, ~1 s at ~2 GHz), whichever comes first.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity,
                                                  long long limit = 1LL << 31) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    for (unsigned it = 0; it < kWaitLimit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > limit) break;
    }
    return false;
}
// 1-D bulk copy global -> shared (both 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void tma_bulk_load(void *dst, const void *src, unsigned bytes,
                                              unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Element (record or sample) of the staged data and its window rule.
template <int KIND, typename T> struct StagedElem {
    using E = T;  // samples
    static constexpr int kExtra = (KIND == PYCBF_GB_INTERP_LINEAR) ? 1 : 0;  // j+1 is read
};
template <typename T> struct StagedElem<PYCBF_GB_INTERP_CUBIC, T> {
    using E = typename CoefRec<T>::raw;  // spline records
    static constexpr int kExtra = 0;
};

// First and one-past-last element of the window of delays [xlo, xhi], aligned
// to 16 bytes (nt * sizeof(E) is a multiple of 16, checked on the host); empty
// (e0 == e1) when no delay in the range can be in range.  The index rule is
// the taps' own exact rule, and it is monotonic in the delay.
template <int KIND, typename T>
__device__ __forceinline__ void staged_window(float xlo, float xhi, const DasArgs &a, int &e0,
                                              int &e1) {
    using E = typename StagedElem<KIND, T>::E;
    constexpr int per16 = 16 / (int)sizeof(E);
    e0 = e1 = 0;
    if (xlo != xlo || xhi != xhi || xhi < xlo) return;
    int i0, i1;
    if (KIND == PYCBF_GB_INTERP_NEAREST) {
        Kind<KIND, T>::index_exact(xlo, a, i0);
        Kind<KIND, T>::index_exact(xhi, a, i1);
        if (i1 < 0 || i0 >= a.nt) return;
    } else {
        if (xhi < a.t0 || xlo > a.xmax) return;
        i0 = (xlo <= a.t0) ? 0 : (int)floorf(__fdiv_rn(__fsub_rn(xlo, a.t0), a.dt));
        i1 = (xhi >= a.xmax) ? a.nt - 1 : (int)floorf(__fdiv_rn(__fsub_rn(xhi, a.t0), a.dt));
    }
    i0 = min(max(i0, 0), a.nt - 1);
    i1 = min(max(i1 + StagedElem<KIND, T>::kExtra, 0), a.nt - 1);
    if (i1 < i0) return;
    e0 = (i0 / per16) * per16;
    e1 = min(((i1 + per16) / per16) * per16, a.nt);
}

// one payload from a staged window (indices clamped into the stage: a tap
// outside its window cannot occur, and if it did it would read a wrong value,
// never outside shared memory)
template <int KIND, typename T>
__device__ __forceinline__ typename Kind<KIND, T>::P staged_load(
    const typename StagedElem<KIND, T>::E *stage, int base, int idx, unsigned cap,
    const DasArgs &a) {
    const unsigned e = min((unsigned)(base + idx), cap - 1u);
    if constexpr (KIND == PYCBF_GB_INTERP_CUBIC) {
        return CoefRec<T>::unpack(stage[e]);
    } else if constexpr (KIND == PYCBF_GB_INTERP_LINEAR) {
        const float y0 = load_sample_reg(stage[e]);
        const float y1 = (idx + 1 < a.nt) ? load_sample_reg(stage[min(e + 1u, cap - 1u)]) : 0.f;
        return make_float2(y0, y1);
    } else {
        return load_sample_reg(stage[e]);
    }
}

// ---------------------------------------------------------------------------
// plan: one CTA per tile.  Pass 1 marks the live receives (a warp per
// receive, each lane four of the tile's pixels); thread 0 numbers them in
// receive order; pass 2 computes each live receive's windows: per transmit
// the smallest and largest delay sum over the pixels the receive reaches,
// reduced over the warp, through the exact window rule.  The windows of a
// receive are packed one after another (each 16-byte aligned) into one stage;
// a receive whose windows exceed a stage is marked unstaged.
// ---------------------------------------------------------------------------
template <int KIND, typename T>
__global__ void __launch_bounds__(kBlock) tabbed_plan_kernel(const __grid_constant__ DasArgs a,
                                                             int *plan) {
    using E = typename StagedElem<KIND, T>::E;
    constexpr unsigned kFull = 0xffffffffu;
    extern __shared__ int s_pos[];  // nrx: position of each receive in the live list, or -1
    __shared__ float s_tt[kTxReg][kBlock];
    __shared__ float s_amax[kBlock];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    constexpr int kWarps = kBlock / 32;
    const long long tile = blockIdx.x;
    const long long np = a.np;
    const int ntx = a.ntx, nrx = a.nrx;
    int *rec = plan + kPlanHeaderWords + tile * plan_tile_words(nrx);
    const float nan = __int_as_float(0x7fc00000);
    {
        const long long i = tile * kBlock + tid;
        const bool valid = i < np;
        float amax = 0.f;
        for (int t = 0; t < ntx; ++t) {
            s_tt[t][tid] = valid ? __ldg(a.tautx + (long long)t * np + i) : nan;
            if (valid) amax = fmaxf(amax, fabsf(__ldg(a.apodtx + (long long)t * np + i)));
        }
        s_amax[tid] = amax;  // 0 for pixels past the end: never live
    }
    __syncthreads();
    // the receive's delay at pixel lane + 32 m and whether the receive reaches it
    auto rx_pixels = [&](int r, float (&tr)[kBlock / 32], bool (&lv)[kBlock / 32]) {
#pragma unroll
        for (int m = 0; m < kBlock / 32; ++m) {
            const int p = lane + 32 * m;
            const long long i = tile * kBlock + p;
            tr[m] = 0.f;
            lv[m] = false;
            if (i < np) {
                tr[m] = __ldg(a.taurx + (long long)r * np + i);
                const float ar = __ldg(a.apodrx + (long long)r * np + i);
                lv[m] = (__fmul_rn(s_amax[p], fabsf(ar)) >= a.thresh) && (tr[m] == tr[m]);
            }
        }
    };
    for (int r = w; r < nrx; r += kWarps) {
        float tr[kBlock / 32];
        bool lv[kBlock / 32];
        rx_pixels(r, tr, lv);
        bool any = false;
#pragma unroll
        for (int m = 0; m < kBlock / 32; ++m) any |= lv[m];
        any = __any_sync(kFull, any);
        if (lane == 0) s_pos[r] = any ? 1 : 0;
    }
    __syncthreads();
    if (tid == 0) {
        int run = 0;
        for (int r = 0; r < nrx; ++r) s_pos[r] = s_pos[r] ? run++ : -1;
        rec[0] = run;
        rec[1] = rec[2] = rec[3] = 0;
    }
    __syncthreads();
    for (int r = w; r < nrx; r += kWarps) {
        const int k = s_pos[r];
        if (k < 0) continue;
        float tr[kBlock / 32];
        bool lv[kBlock / 32];
        rx_pixels(r, tr, lv);
        int my_e0 = 0, my_cnt = 0;
        for (int t = 0; t < ntx; ++t) {
            float lo = __int_as_float(0x7f800000), hi = -lo;
#pragma unroll
            for (int m = 0; m < kBlock / 32; ++m) {
                const float x = __fadd_rn(s_tt[t][lane + 32 * m], tr[m]);
                if (lv[m] && x == x) {
                    lo = fminf(lo, x);
                    hi = fmaxf(hi, x);
                }
            }
            for (int o = 16; o; o >>= 1) {
                lo = fminf(lo, __shfl_xor_sync(kFull, lo, o));
                hi = fmaxf(hi, __shfl_xor_sync(kFull, hi, o));
            }
            int e0, e1;
            staged_window<KIND, T>(lo, hi, a, e0, e1);
            if (lane == t) {
                my_e0 = e0;
                my_cnt = e1 - e0;
            }
        }
        // stage offsets: exclusive prefix of the window lengths over the transmits
        int off = my_cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFull, off, o);
            if (lane >= o) off += v;
        }
        const int total = __shfl_sync(kFull, off, 31);
        off -= my_cnt;
        const bool staged = (long long)total * (long long)sizeof(E) <= kStageBytes &&
                            a.nt <= kStagedMaxNt;
        int *rr = rec + 4 + (long long)kRxWords * k;
        if (lane == 0) {
            rr[0] = staged ? r : (r | kUnstaged);
            rr[1] = staged ? total : 0;
            rr[2] = rr[3] = 0;
        }
        if (lane < kTxReg)
            rr[4 + lane] = (staged && lane < ntx)
                               ? (int)((unsigned)my_e0 | ((unsigned)my_cnt << kWinBits))
                               : 0;
    }
}

// ---------------------------------------------------------------------------
// the staged kernel (Tabbed, ntx <= kTxReg, sums over transmits per receive)
//
// Per receive and transmit group (4 taps, transmits padded with zero weights)
// the inner loop has no data-dependent branch: indices are computed for all
// taps, the gathers read shared memory at clamped indices (always inside the
// stage), and a tap is added only where it contributes, by a select.  The
// exact-quotient redo runs only when some tap of the group is within eps of a
// rounding boundary.
//
// Ring protocol: full[s] completes when the copies of a stage land (one arrive
// with the byte count); empty[s] completes when all warps are done with it.
// Warp 0 refills the slot of iteration it-1 at the end of iteration it, so it
// waits only for warps that are a whole receive behind.
// ---------------------------------------------------------------------------
constexpr int kTapGroup = 4;

// One group of N <= kTapGroup taps of receive (trx, arx): index, gather, weight,
// accumulate.  STAGED gathers from the shared-memory stage at clamped
// indices, otherwise from global memory.  A tap whose quotient lies within
// a few ulp of a rounding boundary has its index redone with the IEEE
// division; the group branches only when some tap needs it.
__device__ __forceinline__ float pair_lane(const float2 *v, int k) {
    return (k & 1) ? v[k >> 1].y : v[k >> 1].x;
}

template <int KIND, typename T, bool STAGED, int N>
__device__ __forceinline__ float staged_group(const DasArgs &a, const float2 *tt2, const float2 *at2,
                                              float trx, float arx, const int *bk,
                                              const typename StagedElem<KIND, T>::E *stage,
                                              long long ch_first, long long chs, int g, int ntx,
                                              float accr) {
    using K = Kind<KIND, T>;
    constexpr unsigned cap = kStageBytes / sizeof(typename StagedElem<KIND, T>::E);
    float xs[N], ap[N], fl[N];
    bool ok[N];
    bool nearb = false;
    // delay sums, weights and quotients two taps at a time in packed float32
    // pairs (each lane rounded as the scalar operation: the same bits)
    float px[N], pa[N], pq[N];
#pragma unroll
    for (int k = 0; k < N; k += 2) {
        if (k + 1 < N) {
            const float2 x2 = add2_rn(make_float2(pair_lane(tt2, k), pair_lane(tt2, k + 1)),
                                      make_float2(trx, trx));
            const float2 a2 = mul2_rn(make_float2(pair_lane(at2, k), pair_lane(at2, k + 1)),
                                      make_float2(arx, arx));
            const float2 q2 = mul2_rn(add2_rn(x2, make_float2(-a.t0, -a.t0)),
                                         make_float2(a.inv_dt, a.inv_dt));
            px[k] = x2.x;
            px[k + 1] = x2.y;
            pa[k] = a2.x;
            pa[k + 1] = a2.y;
            pq[k] = q2.x;
            pq[k + 1] = q2.y;
        } else {
            px[k] = __fadd_rn(pair_lane(tt2, k), trx);
            pa[k] = __fmul_rn(pair_lane(at2, k), arx);
            pq[k] = __fmul_rn(__fsub_rn(px[k], a.t0), a.inv_dt);
        }
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float x = px[k];
        const float apod = pa[k];
        const float q = pq[k];
        // q_fast = fl(fl(x - t0) * fl(1/dt)) and q_exact = fl(fl(x - t0) / dt) differ by at
        // most 3 roundings: |q_fast - q_exact| <= 1.5 |q| 2^-23 (1 + 2^-22).  The floor of a
        // quotient farther than that from every integer is the floor of q_exact.  Nearest
        // rounds q + 0.5 once more (the sum's own rounding can move a q within half an ulp
        // of the boundary across it), so it flags within 4 |q| 2^-23.
        const float tol = fmaf(fabsf(q), KIND == PYCBF_GB_INTERP_NEAREST ? 4.76837158e-7f : 1.8e-7f,
                               1e-30f);
        float flk;
        bool inr;
        if (KIND == PYCBF_GB_INTERP_NEAREST) {
            flk = truncf(q + 0.5f);
            inr = (x == x) && (flk >= 0.f) && (flk < (float)a.nt);
            nearb |= fabsf(q - floorf(q) - 0.5f) < tol;
        } else {
            flk = floorf(q);
            inr = (x >= a.t0) && (x <= a.xmax);
            nearb |= fabsf(q - rintf(q)) < tol;  // distance to the nearest integer (exact)
        }
        xs[k] = x;
        ap[k] = apod;
        fl[k] = flk;
        ok[k] = inr && (fabsf(apod) >= a.thresh);
    }
    if (nearb) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float qe = __fdiv_rn(__fsub_rn(xs[k], a.t0), a.dt);
            if (KIND == PYCBF_GB_INTERP_NEAREST) {
                fl[k] = truncf(qe + 0.5f);
                ok[k] = (xs[k] == xs[k]) && (fl[k] >= 0.f) && (fl[k] < (float)a.nt) &&
                        (fabsf(ap[k]) >= a.thresh);
            } else {
                fl[k] = floorf(qe);
            }
        }
    }
    typename K::P pv[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const int j = min(max((int)fl[k], 0), a.nt - 1);
        if (STAGED) {
            pv[k] = staged_load<KIND, T>(stage, bk[k], j, cap, a);
        } else {
            // padded transmit slots (g + k >= ntx) read the last real channel:
            // their weight is zero and the select below drops them
            const int t = min(g + k, ntx - 1);
            pv[k] = K::load(a.data, ch_first + (long long)t * chs, j, a);
        }
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float c = fmaf(ap[k], K::value(pv[k], xs[k], fl[k], a), accr);
        accr = ok[k] ? c : accr;
    }
    return accr;
}

// Cubic taps from float32 polynomial records in a stage: N <= kTapGroup
// transmits of receive (trx, arx), their delays and weights as float32 pairs
// tt2/at2 (the pair's second lane past N is padding), sb[k] the element base
// of transmit k's window in the stage.  The delay sums, weights and quotients
// are formed two taps per instruction (each lane rounded as the scalar
// operation).  The knot: for the fast quotient q = fl(fl(x - t0) * fl(1/dt)),
// s = q - 1/2 is exact for 0 <= q < 2^22, and adding 1.5 * 2^23 rounds it to
// an integer j held in the low bits of the sum, so h = s - j lies in
// [-1/2, 1/2].  Where |h| <= 1/2 - eps_fast (eps_fast exceeds 1.5 |q| 2^-23,
// the largest gap between q and the reference's correctly rounded quotient
// fl(fl(x - t0) / dt), for every q below nt), both quotients lie strictly
// between j and j + 1, so j is the reference's knot; the sum's bit pattern
// minus that of 1.5 * 2^23 is j itself.  A group holding any other tap (q
// within eps_fast of an integer; NaN and infinite delays too) takes
// staged_cubic_exact instead, which decides every tap with the IEEE division.
// The two paths share nothing after the branch but the running sum, so the
// common one carries no merge of gathered records.
template <int N>
__device__ __forceinline__ float staged_cubic_exact(const DasArgs &a, const float2 *tt2,
                                                 const float2 *at2, float trx, float arx,
                                                 const int *sb, const float4 *stage, float accr) {
    constexpr unsigned cap = kStageBytes / sizeof(float4);
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float x = __fadd_rn(pair_lane(tt2, k), trx);
        const float apod = __fmul_rn(pair_lane(at2, k), arx);
        const float fl = floorf(__fdiv_rn(__fsub_rn(x, a.t0), a.dt));
        const int j = (int)fminf(fmaxf(fl, -1.f), (float)a.nt);  // NaN: -1
        const float4 c = stage[min((unsigned)(sb[k] + j), cap - 1u)];
        const float xlo = __fadd_rn(a.t0, __fmul_rn(a.dt, fl));
        const float b = __fmul_rn(__fsub_rn(x, xlo), a.inv_dt);
        const float v = fmaf(fmaf(fmaf(c.w, b, c.z), b, c.y), b, c.x);
        const bool ok = (x >= a.t0) && (x <= a.xmax) && (fabsf(apod) >= a.thresh);
        const float r = fmaf(apod, v, accr);
        accr = ok ? r : accr;
    }
    return accr;
}

template <int N>
__device__ __forceinline__ float staged_cubic_group(const DasArgs &a, const float2 *tt2,
                                                    const float2 *at2, float trx, float arx,
                                                    const int *sb, const float4 *stage,
                                                    float accr) {
    constexpr unsigned cap = kStageBytes / sizeof(float4);
    constexpr int NP = (N + 1) / 2;
    const float2 trx2 = make_float2(trx, trx), arx2 = make_float2(arx, arx);
    const float2 t02 = make_float2(a.t0, a.t0), inv2 = make_float2(a.inv_dt, a.inv_dt);
    const float2 half2 = make_float2(0.5f, 0.5f), mag2 = make_float2(12582912.f, 12582912.f);
    const float hmax = 0.5f - a.eps_fast;
    float2 x2[NP], ap2[NP], fj2[NP];
    int e[2 * NP];
    bool nearb = false;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        x2[p] = add2_rn(tt2[p], trx2);
        ap2[p] = mul2_rn(at2[p], arx2);
        const float2 q2 = mul2_rn(sub2_rn(x2[p], t02), inv2);
        const float2 s2 = sub2_rn(q2, half2);
        const float2 r2 = add2_rn(s2, mag2);
        fj2[p] = sub2_rn(r2, mag2);
        const float2 h2 = sub2_rn(s2, fj2[p]);
        e[2 * p] = sb[2 * p] + (__float_as_int(r2.x) - 0x4B400000);
        e[2 * p + 1] = sb[2 * p + 1] + (__float_as_int(r2.y) - 0x4B400000);
        nearb |= !(fabsf(h2.x) <= hmax);
        if (2 * p + 1 < N) nearb |= !(fabsf(h2.y) <= hmax);
    }
    if (nearb) return staged_cubic_exact<N>(a, tt2, at2, trx, arx, sb, stage, accr);
    float4 pv[N];
#pragma unroll
    for (int k = 0; k < N; ++k) pv[k] = stage[min((unsigned)e[k], cap - 1u)];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        // b = (x - xlo) / dt, xlo = fl(t0 + fl(dt j)) as the reference rounds the
        // knot (two scalar roundings: no product feeds a packed add)
        const float2 xlo2 = make_float2(__fadd_rn(a.t0, __fmul_rn(a.dt, fj2[p].x)),
                                        __fadd_rn(a.t0, __fmul_rn(a.dt, fj2[p].y)));
        const float2 b2 = mul2_rn(sub2_rn(x2[p], xlo2), inv2);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * p + h;
            if (k < N) {
                const float b = h ? b2.y : b2.x;
                const float x = h ? x2[p].y : x2[p].x;
                const float apod = h ? ap2[p].y : ap2[p].x;
                const float v = fmaf(fmaf(fmaf(pv[k].w, b, pv[k].z), b, pv[k].y), b, pv[k].x);
                const bool ok = (x >= a.t0) && (x <= a.xmax) && (fabsf(apod) >= a.thresh);
                const float c = fmaf(apod, v, accr);
                accr = ok ? c : accr;
            }
        }
    }
    return accr;
}

// Delay gradients of N <= kTapGroup cubic taps of receive (trx, arx), the
// adjoint of the delay-and-sum with respect to tautx and taurx: for every tap
// the forward counts (the same decisions: range, threshold, knot), d = apod *
// (gp * dS/dx) with dS/dx = (p1 + 2 p2 b + 3 p3 b^2) / dt from the interval's
// polynomial record; d is added into gt[k] (this pixel's dL/dtautx of the
// group's transmit k, over receives in order) and into the returned gr
// (dL/dtaurx, over transmits in order).  Records come from the stage
// (STAGED; sb the element bases of the windows in the stage) or from global memory
// (grec: the record row of the group's first transmit, chs between
// transmits).
template <int N, bool STAGED>
__device__ __forceinline__ float adj_cubic_group(const DasArgs &a, const float2 *tt2,
                                                 const float2 *at2, float trx, float arx, float gp,
                                                 const int *sb, const float4 *stage,
                                                 const float4 *grec, long long chs, float *gt,
                                                 float gr) {
    constexpr unsigned cap = kStageBytes / sizeof(float4);
    constexpr int NP = (N + 1) / 2;
    const float2 trx2 = make_float2(trx, trx), arx2 = make_float2(arx, arx);
    const float2 t02 = make_float2(a.t0, a.t0), inv2 = make_float2(a.inv_dt, a.inv_dt);
    const float2 half2 = make_float2(0.5f, 0.5f), mag2 = make_float2(12582912.f, 12582912.f);
    const float hmax = 0.5f - a.eps_fast;
    float2 x2[NP], ap2[NP], fj2[NP];
    int jj[2 * NP];
    bool nearb = false;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        x2[p] = add2_rn(tt2[p], trx2);
        ap2[p] = mul2_rn(at2[p], arx2);
        const float2 s2 = sub2_rn(mul2_rn(sub2_rn(x2[p], t02), inv2), half2);
        const float2 r2 = add2_rn(s2, mag2);
        fj2[p] = sub2_rn(r2, mag2);
        const float2 h2 = sub2_rn(s2, fj2[p]);
        jj[2 * p] = __float_as_int(r2.x) - 0x4B400000;
        jj[2 * p + 1] = __float_as_int(r2.y) - 0x4B400000;
        nearb |= !(fabsf(h2.x) <= hmax);
        if (2 * p + 1 < N) nearb |= !(fabsf(h2.y) <= hmax);
    }
    if (nearb) {  // rare: every tap of the group with the IEEE quotient
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float x = (k & 1) ? x2[k >> 1].y : x2[k >> 1].x;
            const float fl = floorf(__fdiv_rn(__fsub_rn(x, a.t0), a.dt));
            jj[k] = (int)fminf(fmaxf(fl, -1.f), (float)a.nt);  // NaN: -1
            if (k & 1) fj2[k >> 1].y = fl;
            else fj2[k >> 1].x = fl;
        }
    }
    float4 pv[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (STAGED) {
            pv[k] = stage[min((unsigned)(sb[k] + jj[k]), cap - 1u)];
        } else {
            const int j = min(max(jj[k], 0), a.nt - 1);
            pv[k] = __ldg(grec + k * chs + j);
        }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float2 xlo2 = make_float2(__fadd_rn(a.t0, __fmul_rn(a.dt, fj2[p].x)),
                                        __fadd_rn(a.t0, __fmul_rn(a.dt, fj2[p].y)));
        const float2 b2 = mul2_rn(sub2_rn(x2[p], xlo2), inv2);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * p + h;
            if (k < N) {
                const float b = h ? b2.y : b2.x;
                const float x = h ? x2[p].y : x2[p].x;
                const float apod = h ? ap2[p].y : ap2[p].x;
                const float slope =
                    fmaf(fmaf(3.f * pv[k].w, b, 2.f * pv[k].z), b, pv[k].y) * a.inv_dt;
                const float d = apod * (gp * slope);
                const bool ok = (x >= a.t0) && (x <= a.xmax) && (fabsf(apod) >= a.thresh);
                if (ok) {
                    gt[k] += d;
                    gr += d;
                }
            }
        }
    }
    return gr;
}

// Persistent: a grid sized to the GPU takes work items from the plan's queue
// head (plan[1], zeroed before the launch) in the plan's order, largest first,
// so the slowest items start first and the last wave is short: (tile, block
// of receives) items for one frame summed over receives, (frame, tile) items
// otherwise.  The ring's barriers live across items: ring entry number g
// (counted over all items this CTA has run) uses slot g % kStages and phase
// parity (g / kStages) & 1.  Each item is computed entirely by one CTA (and a
// tile's blocks are added in block order), so the results do not depend on
// the scheduling.
//
// Producers: warp 0 stages an item's first kStages receives; after that the
// warp whose turn it is (receive it, warp it % 4) refills the slot of receive
// it - 1 with receive it + 3 once every warp has left that slot.  Each warp
// keeps the plan words of the next receive it will stage in registers,
// loaded one turn ahead.
//
// ADJ: the delay gradients instead of the image (cubic, float32 records, one
// frame): whole tiles as items, the upstream gradient a.gk (kernel pixel
// order; per pixel for TX_AND_RX, per receive and pixel for TX_ONLY), dL/dtaurx
// written per live receive into a.grx and dL/dtautx per item into a.gtx (the
// rows of receives a tile cannot use stay as the caller zeroed them).
template <int KIND, int SUM, typename T, bool ADJ = false>
__global__ void __launch_bounds__(kBlock, ADJ ? 4 : 5) das_staged_kernel(const __grid_constant__ DasArgs a,
                                                              int *__restrict__ plan) {
    using E = typename StagedElem<KIND, T>::E;
    constexpr bool kPolyCubic = KIND == PYCBF_GB_INTERP_CUBIC && CoefRec<T>::kPoly;
    constexpr int kWarps = kBlock / 32;
    constexpr unsigned kFull = 0xffffffffu;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long full[kStages];
    __shared__ __align__(8) unsigned long long empty[kStages];
    __shared__ __align__(16) int sbase[kStages][kTxReg];  // element base of each window - its e0
    __shared__ int sstaged[kStages];
    __shared__ int s_copies[kStages];  // the slot's latest phase has bulk copies in flight
    __shared__ int s_failed;
    __shared__ int s_produced;  // ring entries (over all items) whose copies have been issued
    __shared__ long long s_item;
    __shared__ int s_last;
    int *s_rx = reinterpret_cast<int *>(smem_raw + kStages * kStageBytes);  // the item's receive codes

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int ntx = a.ntx, nrx = a.nrx;
    const long long np = a.np;
    const PlanLayout L = plan_layout(np, ntx, nrx);
    const long long tiles = L.tiles;
    const long long tile_words = L.tile_words;
    constexpr bool kBlockSum = SUM == PYCBF_GB_SUM_TX_AND_RX || SUM == PYCBF_GB_SUM_TX_ONLY;
    const bool by_block = !ADJ && kBlockSum && a.nframes == 1;
    const long long nitems = by_block ? (long long)__ldg(plan + 2) : tiles * a.nframes;
    const int *order = plan + L.order;
    const int4 *bitems = reinterpret_cast<const int4 *>(plan + L.items);
    int *counters = plan + L.counters;
    float *partials = reinterpret_cast<float *>(plan + L.partials);
    unsigned *queue = reinterpret_cast<unsigned *>(plan + 1);
    const long long wait_lim = a.wait_cycles > 0 ? a.wait_cycles : (1LL << 31);

    if (tid < kStages) {
        mbar_init(&full[tid], 1);
        mbar_init(&empty[tid], kWarps);
        s_copies[tid] = 0;
    }
    if (tid == 0) {
        s_failed = 0;
        s_produced = 0;
    }
    mbar_fence_init();

    int g0 = 0;  // ring entries this CTA has run before the current item
    for (;;) {
        if (tid == 0) s_item = (long long)atomicAdd(queue, 1u);
        __syncthreads();  // also: every warp is done with the previous item's ring and codes
        const long long item = s_item;
        if (item >= nitems || s_failed) break;
        int f = 0, first = 0, bord = 0, nblocks = 1;
        long long tile;
        int nlive;
        const int *rec;
        if (by_block) {
            const int4 it4 = __ldg(bitems + item);
            tile = it4.x;
            first = it4.y;
            nlive = it4.z - it4.y;
            bord = it4.w >> 16;
            nblocks = it4.w & 0xffff;
            rec = plan + kPlanHeaderWords + tile * tile_words;
        } else {
            f = (int)(item / tiles);
            tile = __ldg(order + (item - (long long)f * tiles));
            rec = plan + kPlanHeaderWords + tile * tile_words;
            nlive = __ldg(rec);
        }
        const long long i = tile * kBlock + tid;
        const bool valid = i < np;
        // this item's live receives: plan words of receive k at rx0 + kRxWords k
        const int *rx0 = rec + 4 + (long long)kRxWords * first;
        const long long frame_ch = (long long)f * ntx * nrx;
        const long long op = valid ? (a.pixel_index ? (long long)__ldg(a.pixel_index + i) : i) : 0;
        for (int k = tid; k < nlive; k += kBlock) s_rx[k] = __ldg(rx0 + (long long)kRxWords * k);
        __syncthreads();

        // stage receive `it` of this item into its ring slot with the plan words
        // wv (this lane's transmit window) and tot (the receive's total elements)
        auto produce = [&](int it, int wv, int tot) {
            const int gi = g0 + it;
            const int slot = gi & (kStages - 1);
            const int code = s_rx[it];
            const bool staged = !(code & kUnstaged);
            const int r = code & ~kCodeFlags;
            const int e0 = wv & ((1 << kWinBits) - 1);
            const int cnt = (staged && lane < ntx) ? (int)((unsigned)wv >> kWinBits) : 0;
            // this transmit's offset in the stage: exclusive prefix of the lengths
            int off = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(kFull, off, o);
                if (lane >= o) off += v;
            }
            off -= cnt;
            if (lane < kTxReg) sbase[slot][lane] = (staged && lane < ntx) ? off - e0 : 0;
            // stall test: the item's first receive announces its bytes (at least 16)
            // and issues no copy, so its phase never completes and nothing is in flight
            const bool stall = a.stall_test && it == 0;
            const unsigned bytes = staged ? (unsigned)(tot * (int)sizeof(E)) : 0u;
            if (lane == 0) {
                sstaged[slot] = staged ? 1 : 0;
                s_copies[slot] = (staged && bytes > 0 && !stall) ? 1 : 0;
                mbar_arrive_expect_tx(&full[slot], stall ? max(bytes, 16u) : bytes);
            }
            __syncwarp();
            if (cnt > 0 && !stall) {
                const E *src = static_cast<const E *>(a.data) +
                               (frame_ch + (long long)lane * nrx + r) * a.nt + e0;
                E *dst = reinterpret_cast<E *>(smem_raw + (size_t)slot * kStageBytes) + off;
                tma_bulk_load(dst, src, (unsigned)(cnt * (int)sizeof(E)), &full[slot]);
            }
            if (lane == 0) atomicMax(&s_produced, gi + 1);
        };
        auto plan_words = [&](int it, int &wv, int &tot) {
            const int *p = rx0 + (long long)kRxWords * it;
            wv = (lane < ntx) ? __ldg(p + 4 + lane) : 0;
            tot = __ldg(p + 1);
        };
        // warp 0 stages the item's first kStages receives (their slots were freed
        // by every warp before the barrier above)
        if (w == 0) {
            int wv[kStages], tot[kStages];
#pragma unroll
            for (int it = 0; it < kStages; ++it)
                if (it < nlive) plan_words(it, wv[it], tot[it]);
#pragma unroll
            for (int it = 0; it < kStages; ++it)
                if (it < nlive) produce(it, wv[it], tot[it]);
        }
        // this warp's next turn: receive it_w (it_w % 4 == w, it_w >= 1) stages it_w + 3
        int next_it = (w == 0 ? kWarps : w) + kStages - 1;
        int nwv = 0, ntot = 0;
        if (next_it < nlive) plan_words(next_it, nwv, ntot);

        // transmit side of this pixel as float32 pairs; slots past ntx carry zero weights
        float2 tt2[kTxReg / 2], at2[kTxReg / 2];
        float amax = 0.f;
#pragma unroll
        for (int k = 0; k < kTxReg; ++k) {
            float tv = a.t0, av = 0.f;
            if (k < ntx && valid) {
                tv = __ldg(a.tautx + (long long)k * np + i);
                av = __ldg(a.apodtx + (long long)k * np + i);
                amax = fmaxf(amax, fabsf(av));
            }
            if (k & 1) {
                tt2[k >> 1].y = tv;
                at2[k >> 1].y = av;
            } else {
                tt2[k >> 1].x = tv;
                at2[k >> 1].x = av;
            }
        }

        float acc = 0.f, s1 = 0.f;
        float bacc = 0.f;  // the current receive block's sequential sum (TX_AND_RX)
        int cur_block = -1;
        bool failed = false;
        // ADJ: this pixel's dL/dtautx per transmit, and its upstream gradient
        float gt[kTxReg];
#pragma unroll
        for (int k = 0; k < kTxReg; ++k) gt[k] = 0.f;
        const float gpix = (ADJ && SUM == PYCBF_GB_SUM_TX_AND_RX && valid) ? __ldg(a.gk + i) : 0.f;
        // receive-side values, fetched two receives ahead
        const float *trp = a.taurx + i, *arp = a.apodrx + i;
        auto rx_load = [&](int it, float &trx, float &arx, float &gpr) {
            const long long ro = (long long)(s_rx[it] & ~kCodeFlags) * np;
            trx = valid ? __ldg(trp + ro) : 0.f;
            arx = valid ? __ldg(arp + ro) : 0.f;
            gpr = (ADJ && SUM == PYCBF_GB_SUM_TX_ONLY && valid) ? __ldg(a.gk + ro + i) : gpix;
        };
        float trx1 = 0.f, arx1 = 0.f, trx2 = 0.f, arx2 = 0.f, gp1 = 0.f, gp2 = 0.f;
        if (nlive > 0) rx_load(0, trx1, arx1, gp1);
        if (nlive > 1) rx_load(1, trx2, arx2, gp2);

        for (int it = 0; it < nlive; ++it) {
            const int gi = g0 + it;
            const int slot = gi & (kStages - 1);
            const int r = s_rx[it] & ~kCodeFlags;
            const float trx = trx1, arx = arx1, gp = gp1;
            trx1 = trx2;
            arx1 = arx2;
            gp1 = gp2;
            if (it + 2 < nlive) rx_load(it + 2, trx2, arx2, gp2);
            if (!mbar_try_wait(&full[slot], (unsigned)(gi >> 2) & 1u)) {
                if (*(volatile int *)&s_failed ||
                    !mbar_wait_bounded(&full[slot], (unsigned)(gi >> 2) & 1u, wait_lim)) {
                    failed = true;
                    s_failed = 1;
                    break;
                }
            }

            if (SUM == PYCBF_GB_SUM_TX_AND_RX && r / kRxBlock != cur_block) {
                acc += bacc;  // blocks without a live receive add exact zeros elsewhere
                bacc = 0.f;
                cur_block = r / kRxBlock;
            }
            const bool live = valid && (__fmul_rn(amax, fabsf(arx)) >= a.thresh);
            float accr = 0.f;
            if constexpr (ADJ) {
                // delay gradients of this receive's taps (dL/dtaurx of a
                // non-live pixel is 0: every tap of it fails the threshold)
                float gr = 0.f;
                if (live) {
                    const long long chs = (long long)nrx * a.nt;
                    const float4 *grow = static_cast<const float4 *>(a.data) + (frame_ch + r) * a.nt;
                    const bool stg = sstaged[slot] != 0;
                    const float4 *st4 =
                        reinterpret_cast<const float4 *>(smem_raw + (size_t)slot * kStageBytes);
                    int sb[kTxReg];
#pragma unroll
                    for (int g = 0; g < kTxReg; g += 4) {
                        const int4 b = *reinterpret_cast<const int4 *>(&sbase[slot][g]);
                        sb[g] = b.x;
                        sb[g + 1] = b.y;
                        sb[g + 2] = b.z;
                        sb[g + 3] = b.w;
                    }
#pragma unroll
                    for (int g = 0; g < kTxReg; g += kTapGroup) {
                        if (g < ntx) {
                            const int rem = ntx - g;
#define PGB_AGROUP(n, st)                                                                         \
    adj_cubic_group<n, st>(a, tt2 + g / 2, at2 + g / 2, trx, arx, gp, sb + g, st4,                \
                           grow + (long long)g * chs, chs, gt + g, gr)
                            if (stg) {
                                if (rem >= 4) gr = PGB_AGROUP(4, true);
                                else if (rem == 3) gr = PGB_AGROUP(3, true);
                                else if (rem == 2) gr = PGB_AGROUP(2, true);
                                else gr = PGB_AGROUP(1, true);
                            } else {
                                if (rem >= 4) gr = PGB_AGROUP(4, false);
                                else if (rem == 3) gr = PGB_AGROUP(3, false);
                                else if (rem == 2) gr = PGB_AGROUP(2, false);
                                else gr = PGB_AGROUP(1, false);
                            }
#undef PGB_AGROUP
                        }
                    }
                }
                if (valid && a.grx) a.grx[(long long)r * np + i] = gr;
            } else if (live) {
                if (sstaged[slot]) {
                    const E *stage = reinterpret_cast<const E *>(smem_raw + (size_t)slot * kStageBytes);
                    int sb[kTxReg];
#pragma unroll
                    for (int g = 0; g < kTxReg; g += 4) {
                        const int4 b = *reinterpret_cast<const int4 *>(&sbase[slot][g]);
                        sb[g] = b.x;
                        sb[g + 1] = b.y;
                        sb[g + 2] = b.z;
                        sb[g + 3] = b.w;
                    }
#pragma unroll
                    for (int g = 0; g < kTxReg; g += kTapGroup) {
                        if (g < ntx) {
                            // the last group holds only the transmits left (no padded tap)
                            const int rem = ntx - g;
                            if constexpr (kPolyCubic) {
                                const float4 *st4 = reinterpret_cast<const float4 *>(stage);
#define PGB_CGROUP(n) staged_cubic_group<n>(a, tt2 + g / 2, at2 + g / 2, trx, arx, sb + g, st4, accr)
                                if (rem >= 4) accr = PGB_CGROUP(4);
                                else if (rem == 3) accr = PGB_CGROUP(3);
                                else if (rem == 2) accr = PGB_CGROUP(2);
                                else accr = PGB_CGROUP(1);
#undef PGB_CGROUP
                            } else {
#define PGB_GROUP(n)                                                                              \
    staged_group<KIND, T, true, n>(a, tt2 + g / 2, at2 + g / 2, trx, arx, sb + g, stage, 0, 0, g, ntx, \
                                   accr)
                                if (rem >= 4) accr = PGB_GROUP(4);
                                else if (rem == 3) accr = PGB_GROUP(3);
                                else if (rem == 2) accr = PGB_GROUP(2);
                                else accr = PGB_GROUP(1);
#undef PGB_GROUP
                            }
                        }
                    }
                } else {
                    const long long ch_first = (frame_ch + r) * a.nt;
                    const long long chs = (long long)nrx * a.nt;
#pragma unroll
                    for (int g = 0; g < kTxReg; g += kTapGroup) {
                        if (g < ntx) {
                            const int bk[kTapGroup] = {0, 0, 0, 0};
                            accr = staged_group<KIND, T, false, kTapGroup>(a, tt2 + g / 2, at2 + g / 2, trx,
                                                                arx, bk, nullptr, ch_first, chs, g,
                                                                ntx, accr);
                        }
                    }
                }
            }
            if (SUM == PYCBF_GB_SUM_TX_AND_RX) bacc += accr;
            if (!ADJ && SUM == PYCBF_GB_SUM_TX_ONLY && valid)
                a.out[((long long)f * nrx + r) * np + op] = accr;
            if (SUM == PYCBF_GB_SUM_DMAS_SSR || SUM == PYCBF_GB_SUM_DMAS_POWER) {
                const float sv = (SUM == PYCBF_GB_SUM_DMAS_SSR) ? copysignf(sqrtf(fabsf(accr)), accr) : accr;
                acc = fmaf(sv, s1, acc);
                s1 += sv;
            }
            // this warp is done with the slot
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[slot]);
            // this warp's turn: refill the slot of the previous receive once every warp left it
            if (it + kStages - 1 == next_it && next_it < nlive) {
                const int pg = gi - 1;
                if (!mbar_wait_bounded(&empty[pg & (kStages - 1)], (unsigned)(pg >> 2) & 1u, wait_lim)) {
                    failed = true;
                    s_failed = 1;
                    break;
                }
                produce(next_it, nwv, ntot);
                next_it += kWarps;
                if (next_it < nlive) plan_words(next_it, nwv, ntot);
            }
        }
        __syncthreads();
        if constexpr (ADJ) {
            if (valid && a.gtx) {
                const float nan = __int_as_float(0x7fc00000);
#pragma unroll
                for (int k = 0; k < kTxReg; ++k)
                    if (k < ntx) a.gtx[(long long)k * np + i] = s_failed ? nan : gt[k];
            }
            if (s_failed) break;
            g0 += nlive;
            continue;
        }
        if (s_failed) {
            if (valid) {
                const float nan = __int_as_float(0x7fc00000);
                if (SUM == PYCBF_GB_SUM_TX_ONLY)
                    for (int r = 0; r < nrx; ++r) a.out[((long long)f * nrx + r) * np + op] = nan;
                else
                    a.out[(long long)f * np + op] = nan;
            }
            break;
        }
        if (SUM == PYCBF_GB_SUM_TX_AND_RX) acc += bacc;
        if (SUM != PYCBF_GB_SUM_TX_ONLY) {
            if (!by_block || nblocks == 1) {
                if (valid) a.out[(long long)f * np + op] = acc;
            } else {
                // one block of a multi-block tile: the last block to finish adds the
                // tile's block sums in block order (the same bits whatever the order
                // the blocks finish in)
                float *pt = partials + tile * L.max_blocks * kBlock + tid;
                pt[(long long)bord * kBlock] = acc;
                __threadfence();
                __syncthreads();
                if (tid == 0) s_last = atomicAdd(counters + tile, 1) == nblocks - 1;
                __syncthreads();
                if (s_last) {
                    __threadfence();
                    float sum = __ldcg(pt);
                    for (int c = 1; c < nblocks; ++c) sum += __ldcg(pt + (long long)c * kBlock);
                    if (valid) a.out[op] = sum;
                }
            }
        }
        g0 += nlive;
    }
    __syncthreads();
    if (s_failed && tid == 0) {
        // drain the bulk copies still in flight before the CTA's shared memory
        // goes away: the latest phase of each slot is one of the last kStages
        // entries issued; a phase with copies lands in microseconds, so it gets
        // the full (~1 s) bound, and a phase without copies (the stall test's) is
        // not waited for
        atomicExch(plan, 1);
        const int produced = *(volatile int *)&s_produced;
        for (int j = max(0, produced - kStages); j < produced; ++j)
            if (s_copies[j & (kStages - 1)])
                (void)mbar_wait_bounded(&full[j & (kStages - 1)], (unsigned)(j >> 2) & 1u);
    }
}

inline size_t staged_smem_bytes(int nrx) {
    return (size_t)kStages * kStageBytes + sizeof(int) * (size_t)nrx;
}

// The order the persistent kernel takes the tiles in: most live receives
// first (a counting sort over nlive, one CTA).  Ties may come in any order;
// the images do not depend on it.
static __global__ void __launch_bounds__(1024) plan_order_kernel(int *plan, long long tiles, int ntx,
                                                          int nrx) {
    extern __shared__ int bins[];  // nrx + 1 bins, nlive = nrx first
    const long long tw = plan_tile_words(nrx);
    const PlanLayout L = plan_layout(tiles * kBlock, ntx, nrx);
    int *order = plan + L.order;
    for (int b = threadIdx.x; b <= nrx; b += blockDim.x) bins[b] = 0;
    __syncthreads();
    for (long long t = threadIdx.x; t < tiles; t += blockDim.x)
        atomicAdd(&bins[nrx - min(max(plan[kPlanHeaderWords + t * tw], 0), nrx)], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int b = 0; b <= nrx; ++b) {
            const int c = bins[b];
            bins[b] = run;
            run += c;
        }
    }
    __syncthreads();
    for (long long t = threadIdx.x; t < tiles; t += blockDim.x) {
        const int b = nrx - min(max(plan[kPlanHeaderWords + t * tw], 0), nrx);
        order[atomicAdd(&bins[b], 1)] = (int)t;
    }
    __syncthreads();

    // block items: every (tile, block of kRxBlock receive indices with a live
    // receive), a tile without live receives as one empty item; counting sort
    // on the item's receive count, largest first
    int *sz = bins;  // kRxBlock + 1 bins
    for (int b = threadIdx.x; b <= kRxBlock; b += blockDim.x) sz[b] = 0;
    __syncthreads();
    // walk the blocks of tile t's live list: f(first, last, ordinal, count)
    auto blocks = [&](long long t, auto &&f) {
        const int *rec = plan + kPlanHeaderWords + t * tw;
        const int nlive = min(max(rec[0], 0), nrx);
        if (nlive == 0) {
            f(0, 0, 0, 1);
            return;
        }
        // the block of live receive k
        auto blk = [&](int k) { return (rec[4 + kRxWords * k] & ~kCodeFlags) / kRxBlock; };
        int nb = 0;
        for (int k = 0; k < nlive; ++k)
            if (k == 0 || blk(k) != blk(k - 1)) ++nb;
        int first = 0, ord = 0;
        for (int k = 1; k <= nlive; ++k) {
            if (k == nlive || blk(k) != blk(k - 1)) {
                f(first, k, ord++, nb);
                first = k;
            }
        }
    };
    for (long long t = threadIdx.x; t < tiles; t += blockDim.x)
        blocks(t, [&](int b0, int b1, int, int) { atomicAdd(&sz[kRxBlock - (b1 - b0)], 1); });
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int b = 0; b <= kRxBlock; ++b) {
            const int c = sz[b];
            sz[b] = run;
            run += c;
        }
        plan[2] = run;
    }
    __syncthreads();
    int4 *items = reinterpret_cast<int4 *>(plan + L.items);
    for (long long t = threadIdx.x; t < tiles; t += blockDim.x)
        blocks(t, [&](int b0, int b1, int ord, int nb) {
            items[atomicAdd(&sz[kRxBlock - (b1 - b0)], 1)] = make_int4((int)t, b0, b1, (ord << 16) | nb);
        });
}

template <int KIND, typename T>
cudaError_t launch_plan_one(const DasArgs &a, int *plan, cudaStream_t s) {
    const long long tiles = (a.np + kBlock - 1) / kBlock;
    const size_t psmem = sizeof(int) * (size_t)a.nrx;
    if (psmem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(tabbed_plan_kernel<KIND, T>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem);
        if (e != cudaSuccess) return e;
    }
    tabbed_plan_kernel<KIND, T><<<(unsigned)tiles, kBlock, psmem, s>>>(a, plan);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    const size_t smem = sizeof(int) * ((size_t)max(a.nrx, kRxBlock) + 1);
    plan_order_kernel<<<1, 1024, smem, s>>>(plan, tiles, a.ntx, a.nrx);
    return cudaGetLastError();
}

template <int KIND, int SUM, typename T>
cudaError_t launch_staged_one(const DasArgs &a, const int *plan, int *status, cudaStream_t s) {
    auto kern = das_staged_kernel<KIND, SUM, T>;
    const int smem = (int)staged_smem_bytes(a.nrx);
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (err != cudaSuccess) return err;
    int dev = 0, nsm = 0, per_sm = 0;
    if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
    if ((err = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return err;
    if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, smem)) !=
        cudaSuccess)
        return err;
    const PlanLayout L = plan_layout(a.np, a.ntx, a.nrx);
    constexpr bool kBlockSum = SUM == PYCBF_GB_SUM_TX_AND_RX || SUM == PYCBF_GB_SUM_TX_ONLY;
    const bool by_block = kBlockSum && a.nframes == 1;
    const long long items = by_block ? L.tiles * L.max_blocks : L.tiles * (long long)a.nframes;
    const long long grid = std::min<long long>(items, (long long)std::max(1, per_sm) * nsm);
    // the queue head, plan[1], and the tiles' block counters start at zero
    err = cudaMemsetAsync(status + 1, 0, sizeof(int), s);
    if (err != cudaSuccess) return err;
    if (by_block && SUM == PYCBF_GB_SUM_TX_AND_RX) {
        err = cudaMemsetAsync(const_cast<int *>(plan) + L.counters, 0, sizeof(int) * L.tiles, s);
        if (err != cudaSuccess) return err;
    }
    kern<<<(unsigned)grid, kBlock, smem, s>>>(a, const_cast<int *>(plan));
    return cudaGetLastError();
}

// The delay gradients on the staging plan (ADJ mode; cubic, float32 records,
// one frame, sumtype TX_AND_RX or TX_ONLY).  dL/dtaurx rows of receives a tile
// cannot use are zeroed first.
template <typename T>
cudaError_t launch_staged_adj(const DasArgs &a, int sum, const int *plan, cudaStream_t s) {
    if (!CoefRec<T>::kPoly || a.nframes != 1) return cudaErrorInvalidValue;
    auto kern = sum == PYCBF_GB_SUM_TX_AND_RX
                    ? das_staged_kernel<PYCBF_GB_INTERP_CUBIC, PYCBF_GB_SUM_TX_AND_RX, T, true>
                    : das_staged_kernel<PYCBF_GB_INTERP_CUBIC, PYCBF_GB_SUM_TX_ONLY, T, true>;
    const int smem = (int)staged_smem_bytes(a.nrx);
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (err != cudaSuccess) return err;
    int dev = 0, nsm = 0, per_sm = 0;
    if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
    if ((err = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return err;
    if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, smem)) !=
        cudaSuccess)
        return err;
    const PlanLayout L = plan_layout(a.np, a.ntx, a.nrx);
    const long long grid = std::min<long long>(L.tiles, (long long)std::max(1, per_sm) * nsm);
    int *pl = const_cast<int *>(plan);
    if ((err = cudaMemsetAsync(pl + 1, 0, sizeof(int), s)) != cudaSuccess) return err;
    if (a.grx && (err = cudaMemsetAsync(a.grx, 0, sizeof(float) * (size_t)a.nrx * a.np, s)) !=
                     cudaSuccess)
        return err;
    kern<<<(unsigned)grid, kBlock, smem, s>>>(a, pl);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_plan_type(const DasArgs &a, int interp, int *plan, cudaStream_t s) {
    switch (interp) {
        case PYCBF_GB_INTERP_CUBIC: return launch_plan_one<PYCBF_GB_INTERP_CUBIC, T>(a, plan, s);
        case PYCBF_GB_INTERP_LINEAR: return launch_plan_one<PYCBF_GB_INTERP_LINEAR, T>(a, plan, s);
        case PYCBF_GB_INTERP_NEAREST: return launch_plan_one<PYCBF_GB_INTERP_NEAREST, T>(a, plan, s);
        default: return cudaErrorInvalidValue;
    }
}

template <int KIND, typename T>
cudaError_t launch_staged_kind(const DasArgs &a, int sum, const int *plan, int *status, cudaStream_t s) {
    switch (sum) {
        case PYCBF_GB_SUM_TX_AND_RX: return launch_staged_one<KIND, PYCBF_GB_SUM_TX_AND_RX, T>(a, plan, status, s);
        case PYCBF_GB_SUM_TX_ONLY: return launch_staged_one<KIND, PYCBF_GB_SUM_TX_ONLY, T>(a, plan, status, s);
        case PYCBF_GB_SUM_DMAS_SSR: return launch_staged_one<KIND, PYCBF_GB_SUM_DMAS_SSR, T>(a, plan, status, s);
        case PYCBF_GB_SUM_DMAS_POWER: return launch_staged_one<KIND, PYCBF_GB_SUM_DMAS_POWER, T>(a, plan, status, s);
        default: return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t launch_staged_type(const DasArgs &a, int interp, int sum, const int *plan, int *status,
                               cudaStream_t s) {
    switch (interp) {
        case PYCBF_GB_INTERP_CUBIC: return launch_staged_kind<PYCBF_GB_INTERP_CUBIC, T>(a, sum, plan, status, s);
        case PYCBF_GB_INTERP_LINEAR: return launch_staged_kind<PYCBF_GB_INTERP_LINEAR, T>(a, sum, plan, status, s);
        case PYCBF_GB_INTERP_NEAREST: return launch_staged_kind<PYCBF_GB_INTERP_NEAREST, T>(a, sum, plan, status, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace pgb

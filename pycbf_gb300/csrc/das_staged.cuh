// Tabbed delay-and-sum with channel windows staged in shared memory by TMA.
//
// The pixels of a CTA (a "tile": 128 consecutive table columns, which the
// host stores in Morton order of their delays) need, for each (tx, rx)
// channel, only the samples between the smallest and largest delay of the
// tile.  A plan, built once per table set (tabbed_plan_kernel), records per
// tile the receives that can contribute at all (the exact reject
// fl(max|apodtx| * |apodrx|) >= thresh of at least one pixel), and per tile
// the delay bounds of every transmit and of every live receive.  In the main
// kernel warp 0 turns those bounds into sample windows (the same exact index
// rule as the taps, and indices are monotonic in the delay, so every
// contributing tap falls inside) and issues one cp.async.bulk per transmit
// into a 4-stage ring, completing on an mbarrier; all warps then gather from
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

constexpr int kStages = 4;
constexpr int kStageBytes = 12 * 1024;
constexpr unsigned kWaitLimit = 1u << 30;  // polls; the ~1 s clock bound ends a wait first

// plan layout (int32 words): [0] status, [1] work-queue head of the staged
// kernel, [2] number of block items, [3] pad, then per tile a record of
// plan_tile_words(ntx, nrx) words:
//   nlive | rx index per live receive (nrx) | rx lo,hi per live receive (2*nrx floats)
//   | tx lo,hi per transmit (2*ntx floats)
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
__host__ __device__ inline long long plan_tile_words(int ntx, int nrx) {
    return 1 + (long long)nrx + 2LL * nrx + 2LL * ntx;
}
constexpr int kPlanHeaderWords = 4;
struct PlanLayout {
    long long tiles, tile_words, max_blocks, order, counters, items, partials, total;
};
__host__ __device__ inline PlanLayout plan_layout(long long np, int ntx, int nrx) {
    PlanLayout L;
    L.tiles = (np + kBlock - 1) / kBlock;
    L.tile_words = plan_tile_words(ntx, nrx);
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
// plan: one CTA per tile
// ---------------------------------------------------------------------------
template <int KIND, typename T>
__global__ void __launch_bounds__(kBlock) tabbed_plan_kernel(const __grid_constant__ DasArgs a,
                                                             int *plan) {
    using E = typename StagedElem<KIND, T>::E;
    __shared__ float red[3][kBlock / 32];
    __shared__ int s_any;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const long long tile = blockIdx.x;
    const long long i = tile * kBlock + tid;
    const bool valid = i < a.np;
    const int ntx = a.ntx, nrx = a.nrx;
    int *rec = plan + kPlanHeaderWords + tile * plan_tile_words(ntx, nrx);
    int *rxidx = rec + 1;
    float *rxlh = reinterpret_cast<float *>(rec + 1 + nrx);
    float *txlh = rxlh + 2 * nrx;
    const float inf = __int_as_float(0x7f800000);

    auto block_minmax = [&](float lo, float hi, int any, float &blo, float &bhi, int &bany) {
        for (int o = 16; o; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            any |= __shfl_xor_sync(0xffffffffu, any, o);
        }
        __syncthreads();
        if (lane == 0) {
            red[0][w] = lo;
            red[1][w] = hi;
            red[2][w] = __int_as_float(any);
        }
        __syncthreads();
        blo = red[0][0];
        bhi = red[1][0];
        bany = __float_as_int(red[2][0]);
        for (int k = 1; k < kBlock / 32; ++k) {
            blo = fminf(blo, red[0][k]);
            bhi = fmaxf(bhi, red[1][k]);
            bany |= __float_as_int(red[2][k]);
        }
    };

    float amax = 0.f;
    for (int t = 0; t < ntx; ++t) {
        float tau = inf, taun = -inf;
        if (valid) {
            tau = taun = __ldg(a.tautx + (long long)t * a.np + i);
            amax = fmaxf(amax, fabsf(__ldg(a.apodtx + (long long)t * a.np + i)));
        }
        float lo, hi;
        int any;
        block_minmax(tau == tau ? tau : inf, taun == taun ? taun : -inf, 0, lo, hi, any);
        if (tid == 0) {
            txlh[2 * t] = lo;
            txlh[2 * t + 1] = hi;
        }
    }
    __syncthreads();
    int nlive = 0;
    for (int r = 0; r < nrx; ++r) {
        float trx = 0.f, arx = 0.f;
        if (valid) {
            trx = __ldg(a.taurx + (long long)r * a.np + i);
            arx = __ldg(a.apodrx + (long long)r * a.np + i);
        }
        const bool live = valid && (__fmul_rn(amax, fabsf(arx)) >= a.thresh) && (trx == trx);
        float lo, hi;
        int any;
        block_minmax(live ? trx : inf, live ? trx : -inf, live ? 1 : 0, lo, hi, any);
        if (!any) continue;
        // staged only if all windows of this receive fit one stage
        int bytes = 0;
        if (tid < ntx) {
            const float xlo = __fadd_rn(txlh[2 * tid], lo), xhi = __fadd_rn(txlh[2 * tid + 1], hi);
            int e0, e1;
            staged_window<KIND, T>(xlo, xhi, a, e0, e1);
            bytes = (e1 - e0) * (int)sizeof(E);
        }
        for (int o = 16; o; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
        if (w == 0 && lane == 0) s_any = bytes;
        __syncthreads();
        const bool staged = s_any <= kStageBytes;
        if (tid == 0) {
            rxidx[nlive] = staged ? r : (r | 0x40000000);
            rxlh[2 * nlive] = lo;
            rxlh[2 * nlive + 1] = hi;
        }
        ++nlive;
        __syncthreads();
    }
    if (tid == 0) rec[0] = nlive;
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
template <int KIND, typename T, bool STAGED, int N>
__device__ __forceinline__ float staged_group(const DasArgs &a, const float *tt, const float *at,
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
            const float2 x2 = add2_rn(make_float2(tt[k], tt[k + 1]), make_float2(trx, trx));
            const float2 a2 = mul2_rn(make_float2(at[k], at[k + 1]), make_float2(arx, arx));
            const float2 q2 = mul2_rn(add2_rn(x2, make_float2(-a.t0, -a.t0)),
                                         make_float2(a.inv_dt, a.inv_dt));
            px[k] = x2.x;
            px[k + 1] = x2.y;
            pa[k] = a2.x;
            pa[k + 1] = a2.y;
            pq[k] = q2.x;
            pq[k + 1] = q2.y;
        } else {
            px[k] = __fadd_rn(tt[k], trx);
            pa[k] = __fmul_rn(at[k], arx);
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

// Persistent: a grid sized to the GPU takes (frame, tile) items from the
// plan's queue head (plan[1], zeroed before the launch) in the plan's order,
// the tiles with most live receives first, so the slowest tiles start first
// and the last wave is short.  The ring's barriers live across tiles: item
// number g (counted over all tiles this CTA has run) uses slot g % kStages and
// phase parity (g / kStages) & 1.  Each tile is computed entirely by one CTA,
// so the results do not depend on the scheduling.
template <int KIND, int SUM, typename T>
__global__ void __launch_bounds__(kBlock, 4) das_staged_kernel(const __grid_constant__ DasArgs a,
                                                              int *__restrict__ plan) {
    using E = typename StagedElem<KIND, T>::E;
    constexpr int kWarps = kBlock / 32;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long full[kStages];
    __shared__ __align__(8) unsigned long long empty[kStages];
    __shared__ __align__(16) int sbase[kStages][kTxReg];  // element base of each window - its e0
    __shared__ int sstaged[kStages];
    __shared__ float s_txlh[2 * kTxReg];
    __shared__ int s_failed;
    __shared__ long long s_produced;  // items (over all tiles) whose copies have been issued
    __shared__ long long s_item;
    __shared__ int s_last;
    // the tile's plan: live receive indices and their delay bounds
    int *s_rx = reinterpret_cast<int *>(smem_raw + kStages * kStageBytes);
    float *s_rxlh = reinterpret_cast<float *>(s_rx + a.nrx);

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int ntx = a.ntx, nrx = a.nrx;
    const long long np = a.np;
    const PlanLayout L = plan_layout(np, ntx, nrx);
    const long long tiles = L.tiles;
    const long long tile_words = L.tile_words;
    // one frame summed over receives: (tile, receive block) items; otherwise (frame, tile)
    constexpr bool kBlockSum = SUM == PYCBF_GB_SUM_TX_AND_RX || SUM == PYCBF_GB_SUM_TX_ONLY;
    const bool by_block = kBlockSum && a.nframes == 1;
    const long long nitems = by_block ? (long long)__ldg(plan + 2) : tiles * a.nframes;
    const int *order = plan + L.order;
    const int4 *bitems = reinterpret_cast<const int4 *>(plan + L.items);
    int *counters = plan + L.counters;
    float *partials = reinterpret_cast<float *>(plan + L.partials);
    unsigned *queue = reinterpret_cast<unsigned *>(plan + 1);
    const long long chs = (long long)nrx * a.nt;
    const long long wait_lim = a.wait_cycles > 0 ? a.wait_cycles : (1LL << 31);

    if (tid < kStages) {
        mbar_init(&full[tid], 1);
        mbar_init(&empty[tid], kWarps);
    }
    if (tid == 0) {
        s_failed = 0;
        s_produced = 0;
    }
    mbar_fence_init();

    long long g0 = 0;  // ring items this CTA has run before the current tile
    for (;;) {
        if (tid == 0) s_item = (long long)atomicAdd(queue, 1u);
        __syncthreads();  // also: every warp is done with the previous tile's ring and plan data
        const long long item = s_item;
        if (item >= nitems || s_failed) break;
        int f = 0, first = 0, bord = 0, nblocks = 1;
        long long tile;
        int nlive;
        if (by_block) {
            const int4 it4 = __ldg(bitems + item);
            tile = it4.x;
            first = it4.y;
            nlive = it4.z - it4.y;
            bord = it4.w >> 16;
            nblocks = it4.w & 0xffff;
        } else {
            f = (int)(item / tiles);
            tile = __ldg(order + (item - (long long)f * tiles));
        }
        const long long i = tile * kBlock + tid;
        const bool valid = i < np;
        const int *rec = plan + kPlanHeaderWords + tile * tile_words;
        if (!by_block) nlive = __ldg(rec);
        const long long frame_ch = (long long)f * ntx * nrx;
        const long long op = valid ? (a.pixel_index ? (long long)__ldg(a.pixel_index + i) : i) : 0;
        {
            // this item's live receives: the whole list, or one block of it
            const float *txlh = reinterpret_cast<const float *>(rec + 1 + 3 * nrx);
            if (tid < 2 * ntx) s_txlh[tid] = __ldg(txlh + tid);
            for (int k = tid; k < nlive; k += kBlock) s_rx[k] = __ldg(rec + 1 + first + k);
            const float *rxlh = reinterpret_cast<const float *>(rec + 1 + nrx) + 2 * first;
            for (int k = tid; k < 2 * nlive; k += kBlock) s_rxlh[k] = __ldg(rxlh + k);
        }
        __syncthreads();

        // producer: windows of live receive `it` of this tile into its ring slot
        auto produce = [&](int it) {
            const long long gi = g0 + it;
            const int slot = (int)(gi % kStages);
            const int code = s_rx[it];
            bool staged = !(code & 0x40000000);
            const int r = code & 0x3fffffff;
            int e0 = 0, e1 = 0;
            if (staged && lane < ntx) {
                const float xlo = __fadd_rn(s_txlh[2 * lane], s_rxlh[2 * it]);
                const float xhi = __fadd_rn(s_txlh[2 * lane + 1], s_rxlh[2 * it + 1]);
                staged_window<KIND, T>(xlo, xhi, a, e0, e1);
            }
            const int cnt = e1 - e0;
            int off = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, off, o);
                if (lane >= o) off += v;
            }
            const int total = __shfl_sync(0xffffffffu, off, 31);
            off -= cnt;
            // the plan sized these windows to fit; a plan from other tables could
            // not, and then this receive is gathered from global memory instead
            if ((long long)total * (long long)sizeof(E) > kStageBytes) staged = false;
            if (lane < kTxReg) sbase[slot][lane] = (staged && lane < ntx) ? off - e0 : 0;
            if (lane == 0) sstaged[slot] = staged ? 1 : 0;
            __syncwarp();
            // stall test: the tile's first receive announces its bytes (at least 16)
            // and issues no copy, so its phase never completes and nothing is in flight
            const bool stall = a.stall_test && it == 0;
            const unsigned bytes = staged ? (unsigned)(total * sizeof(E)) : 0u;
            if (lane == 0) mbar_arrive_expect_tx(&full[slot], stall ? max(bytes, 16u) : bytes);
            __syncwarp();
            if (staged && lane < ntx && cnt > 0 && !stall) {
                const E *src = static_cast<const E *>(a.data) + (frame_ch + (long long)lane * nrx + r) * a.nt + e0;
                E *dst = reinterpret_cast<E *>(smem_raw + (size_t)slot * kStageBytes) + off;
                tma_bulk_load(dst, src, (unsigned)(cnt * sizeof(E)), &full[slot]);
            }
        };
        // warp 0 stages the tile's first kStages receives (their slots were freed
        // by every warp before the barrier above); after that the producer role
        // rotates over the warps (a bulk copy costs ~100 cycles to issue, and one
        // warp issuing every receive's copies starved the others)
        if (w == 0) {
            for (int it = 0; it < kStages && it < nlive; ++it) produce(it);
            if (lane == 0 && nlive > 0) atomicMax(&s_produced, g0 + min(kStages, nlive));
        }

        // transmit side of this pixel; slots past ntx carry zero weights
        float rtau[kTxReg], rapod[kTxReg];
        float amax = 0.f;
#pragma unroll
        for (int k = 0; k < kTxReg; ++k) {
            rtau[k] = a.t0;
            rapod[k] = 0.f;
            if (k < ntx && valid) {
                rtau[k] = __ldg(a.tautx + (long long)k * np + i);
                rapod[k] = __ldg(a.apodtx + (long long)k * np + i);
                amax = fmaxf(amax, fabsf(rapod[k]));
            }
        }

        float acc = 0.f, s1 = 0.f;
        float bacc = 0.f;  // the current receive block's sequential sum (TX_AND_RX)
        int cur_block = -1;
        bool failed = false;
        // receive-side values, fetched two receives ahead
        auto rx_load = [&](int it, float &trx, float &arx) {
            const int r = s_rx[it] & 0x3fffffff;
            trx = valid ? __ldg(a.taurx + (long long)r * np + i) : 0.f;
            arx = valid ? __ldg(a.apodrx + (long long)r * np + i) : 0.f;
        };
        float trx1 = 0.f, arx1 = 0.f, trx2 = 0.f, arx2 = 0.f;
        if (nlive > 0) rx_load(0, trx1, arx1);
        if (nlive > 1) rx_load(1, trx2, arx2);

        for (int it = 0; it < nlive; ++it) {
            const long long gi = g0 + it;
            const int slot = (int)(gi % kStages);
            const int r = s_rx[it] & 0x3fffffff;
            const float trx = trx1, arx = arx1;
            trx1 = trx2;
            arx1 = arx2;
            if (it + 2 < nlive) rx_load(it + 2, trx2, arx2);
            if (!mbar_wait_bounded(&full[slot], (unsigned)(gi / kStages) & 1u, wait_lim)) failed = true;
            if (failed || *(volatile int *)&s_failed) {
                failed = true;
                s_failed = 1;
                break;
            }

            if (SUM == PYCBF_GB_SUM_TX_AND_RX && r / kRxBlock != cur_block) {
                acc += bacc;  // blocks without a live receive add exact zeros elsewhere
                bacc = 0.f;
                cur_block = r / kRxBlock;
            }
            const bool live = valid && (__fmul_rn(amax, fabsf(arx)) >= a.thresh);
            float accr = 0.f;
            if (live) {
                const long long ch_first = (frame_ch + r) * a.nt;
                if (sstaged[slot]) {
                    const E *stage = reinterpret_cast<const E *>(smem_raw + (size_t)slot * kStageBytes);
#pragma unroll
                    for (int g = 0; g < kTxReg; g += kTapGroup) {
                        if (g < ntx) {
                            const int4 b = *reinterpret_cast<const int4 *>(&sbase[slot][g]);
                            const int bk[kTapGroup] = {b.x, b.y, b.z, b.w};
                            // the last group holds only the transmits left (no padded tap)
                            const int rem = ntx - g;
#define PGB_GROUP(n)                                                                            \
    staged_group<KIND, T, true, n>(a, rtau + g, rapod + g, trx, arx, bk, stage, ch_first, chs, g, \
                                   ntx, accr)
                            if (rem >= 4) accr = PGB_GROUP(4);
                            else if (rem == 3) accr = PGB_GROUP(3);
                            else if (rem == 2) accr = PGB_GROUP(2);
                            else accr = PGB_GROUP(1);
#undef PGB_GROUP
                        }
                    }
                } else {
#pragma unroll
                    for (int g = 0; g < kTxReg; g += kTapGroup) {
                        if (g < ntx) {
                            const int bk[kTapGroup] = {0, 0, 0, 0};
                            accr = staged_group<KIND, T, false, kTapGroup>(a, rtau + g, rapod + g, trx, arx, bk,
                                                                nullptr, ch_first, chs, g, ntx, accr);
                        }
                    }
                }
            }
            if (SUM == PYCBF_GB_SUM_TX_AND_RX) bacc += accr;
            if (SUM == PYCBF_GB_SUM_TX_ONLY && valid) a.out[((long long)f * nrx + r) * np + op] = accr;
            if (SUM == PYCBF_GB_SUM_DMAS_SSR || SUM == PYCBF_GB_SUM_DMAS_POWER) {
                const float sv = (SUM == PYCBF_GB_SUM_DMAS_SSR) ? copysignf(sqrtf(fabsf(accr)), accr) : accr;
                acc = fmaf(sv, s1, acc);
                s1 += sv;
            }
            // this warp is done with the slot
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[slot]);
            // warp it % kWarps refills the slot of the previous receive once every
            // warp left it
            if (w == it % kWarps && it >= 1 && it - 1 + kStages < nlive) {
                const long long pg = gi - 1;
                if (!mbar_wait_bounded(&empty[pg % kStages], (unsigned)(pg / kStages) & 1u, wait_lim)) {
                    failed = true;
                    s_failed = 1;
                    break;
                }
                produce(it - 1 + kStages);
                if (lane == 0) atomicMax(&s_produced, pg + kStages + 1);
            }
        }
        __syncthreads();
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
        // drain the copies still in flight before the CTA's shared memory goes
        // away: the latest phase of each slot is one of the last kStages issued
        atomicExch(plan, 1);
        const long long produced = *(volatile long long *)&s_produced;
        for (long long j = max(0LL, produced - kStages); j < produced; ++j)
            (void)mbar_wait_bounded(&full[j % kStages], (unsigned)(j / kStages) & 1u, wait_lim);
    }
}

inline size_t staged_smem_bytes(int nrx) {
    return (size_t)kStages * kStageBytes + sizeof(int) * 3 * (size_t)nrx;
}

// The order the persistent kernel takes the tiles in: most live receives
// first (a counting sort over nlive, one CTA).  Ties may come in any order;
// the images do not depend on it.
static __global__ void __launch_bounds__(1024) plan_order_kernel(int *plan, long long tiles, int ntx,
                                                          int nrx) {
    extern __shared__ int bins[];  // nrx + 1 bins, nlive = nrx first
    const long long tw = plan_tile_words(ntx, nrx);
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
        int nb = 0;
        for (int k = 0; k < nlive; ++k)
            if (k == 0 || ((rec[1 + k] & 0x3fffffff) / kRxBlock) != ((rec[k] & 0x3fffffff) / kRxBlock)) ++nb;
        int first = 0, ord = 0;
        for (int k = 1; k <= nlive; ++k) {
            if (k == nlive || ((rec[1 + k] & 0x3fffffff) / kRxBlock) != ((rec[k] & 0x3fffffff) / kRxBlock)) {
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
    tabbed_plan_kernel<KIND, T><<<(unsigned)tiles, kBlock, 0, s>>>(a, plan);
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

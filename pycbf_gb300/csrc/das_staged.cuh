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

#include "das_impl.cuh"

namespace pgb {

constexpr int kStages = 4;
constexpr int kStageBytes = 12 * 1024;     // one stage: receive rows + channel windows
constexpr int kRowBytes = 2 * kBlock * 4;  // the tile's taurx and apodrx of the receive
constexpr int kWindowBytes = kStageBytes - kRowBytes;
constexpr unsigned kWaitLimit = 1u << 16;

// A tile's work is a list of items: one receive and a run of whole transmit
// groups (kTapGroup transmits each) whose windows fit one stage together; a
// receive whose windows are too large for one stage becomes several items.
constexpr int kTapGroup = 4;
constexpr int kTxGroups = (kTxReg + kTapGroup - 1) / kTapGroup;
// item code: receive (bits 0-15), first group (16-19), end group (20-23),
// last item of its receive (bit 28), not staged (bit 30)
constexpr int kItemLast = 1 << 28;
constexpr int kItemUnstaged = 1 << 30;

// plan layout (int32 words): [0] status, [1] reserved, [2..3] pad, then per
// tile a record of plan_tile_words(ntx, nrx) words:
//   nitems | item code (imax) | receive lo,hi delay per item (2*imax floats)
//   | transmit lo,hi delay (2*ntx floats),  imax = nrx * kTxGroups
__host__ __device__ inline long long plan_tile_words(int ntx, int nrx) {
    const long long imax = (long long)nrx * kTxGroups;
    return 1 + imax + 2 * imax + 2LL * ntx;
}
constexpr int kPlanHeaderWords = 4;

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
// try_wait: true once the phase with this parity has completed
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
// Bounded wait: gives up after kWaitLimit polls or ~1 s of SM clock (2^31
// cycles at ~2 GHz), whichever comes first.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    for (unsigned it = 0; it < kWaitLimit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - t0 > (1LL << 31)) break;
    }
    return false;
}
// asynchronous 16-byte / 4-byte copies global -> shared (LSU path)
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// arrive on bar once this thread's earlier cp.async copies have landed (the
// barrier's expected count includes this arrival)
__device__ __forceinline__ void cp_async_arrive(unsigned long long *bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

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

// First and one-past-last element of a window that contains the sample index
// of every delay in [xlo, xhi], aligned to 16 bytes (nt * sizeof(E) is a
// multiple of 16, checked on the host); empty (e0 == e1) when no such delay
// can be in range.  The reciprocal quotient is within 2 ulp of the IEEE one,
// so its index, widened by one sample each way, bounds the taps' exact index,
// which is monotonic in the delay.
template <int KIND, typename T>
__device__ __forceinline__ void staged_window(float xlo, float xhi, const DasArgs &a, int &e0,
                                              int &e1) {
    using E = typename StagedElem<KIND, T>::E;
    constexpr int per16 = 16 / (int)sizeof(E);
    e0 = e1 = 0;
    if (!(xlo <= xhi)) return;  // also rejects NaN
    const float q0 = __fmul_rn(__fsub_rn(xlo, a.t0), a.inv_dt);
    const float q1 = __fmul_rn(__fsub_rn(xhi, a.t0), a.inv_dt);
    const float h = (KIND == PYCBF_GB_INTERP_NEAREST) ? 0.5f : 0.f;
    const float last = (float)(a.nt - 1);
    const float f0 = fmaxf(floorf(q0 + h) - 1.f, 0.f);
    // nearest truncates q + 0.5 toward zero, so q in (-1.5, -0.5) reads sample 0:
    // one more sample of headroom above
    const float up = (KIND == PYCBF_GB_INTERP_NEAREST) ? 2.f : 1.f + (float)StagedElem<KIND, T>::kExtra;
    const float f1 = fminf(floorf(q1 + h) + up, last);
    if (!(f0 <= f1)) return;  // window entirely before sample 0 or after the last
    const int i0 = (int)f0, i1 = (int)f1;
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
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const long long tile = blockIdx.x;
    const long long i = tile * kBlock + tid;
    const bool valid = i < a.np;
    const int ntx = a.ntx, nrx = a.nrx;
    const long long imax = (long long)nrx * kTxGroups;
    int *rec = plan + kPlanHeaderWords + tile * plan_tile_words(ntx, nrx);
    int *codes = rec + 1;
    float *rxlh = reinterpret_cast<float *>(rec + 1 + imax);
    float *txlh = rxlh + 2 * imax;
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
    float txl = 0.f, txh = 0.f;  // this thread's transmit bounds (tid < ntx)
    for (int t = 0; t < ntx; ++t) {
        float tau = inf, taun = -inf;
        if (valid) {
            tau = taun = __ldg(a.tautx + (long long)t * a.np + i);
            amax = fmaxf(amax, fabsf(__ldg(a.apodtx + (long long)t * a.np + i)));
        }
        float lo, hi;
        int any;
        block_minmax(tau == tau ? tau : inf, taun == taun ? taun : -inf, 0, lo, hi, any);
        if (tid == t) {
            txl = lo;
            txh = hi;
        }
        if (tid == 0) {
            txlh[2 * t] = lo;
            txlh[2 * t + 1] = hi;
        }
    }
    int nitems = 0;
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
        if (!any) continue;  // block-uniform
        if (w == 0) {
            // window bytes of this thread's transmit, summed per transmit group
            int bytes = 0;
            if (lane < ntx) {
                int e0, e1;
                staged_window<KIND, T>(__fadd_rn(txl, lo), __fadd_rn(txh, hi), a, e0, e1);
                bytes = (e1 - e0) * (int)sizeof(E);
            }
            for (int o = 1; o < kTapGroup; o <<= 1) bytes += __shfl_down_sync(0xffffffffu, bytes, o);
            int gb[kTxGroups];
            for (int g = 0; g < kTxGroups; ++g) gb[g] = __shfl_sync(0xffffffffu, bytes, g * kTapGroup);
            if (lane == 0) {
                const int ng = (ntx + kTapGroup - 1) / kTapGroup;
                int g0 = 0;
                while (g0 < ng) {
                    int g1 = g0 + 1, tot = gb[g0];
                    while (g1 < ng && tot + gb[g1] <= kWindowBytes) tot += gb[g1++];
                    int code = r | (g0 << 16) | (g1 << 20);
                    if (tot > kWindowBytes) code |= kItemUnstaged;
                    if (g1 == ng) code |= kItemLast;
                    codes[nitems] = code;
                    rxlh[2 * nitems] = lo;
                    rxlh[2 * nitems + 1] = hi;
                    ++nitems;
                    g0 = g1;
                }
            }
            nitems = __shfl_sync(0xffffffffu, nitems, 0);
        }
    }
    if (tid == 0) rec[0] = nitems;
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
// One group of kTapGroup taps of receive (trx, arx): index, gather, weight,
// accumulate.  STAGED gathers from the shared-memory stage at clamped
// indices, otherwise from global memory.  A tap whose quotient lies within
// a few ulp of a rounding boundary has its index redone with the IEEE
// division; the group branches only when some tap needs it.
template <int KIND, typename T, bool STAGED>
__device__ __forceinline__ float staged_group(const DasArgs &a, const float *tt, const float *at,
                                              float trx, float arx, const int *bk,
                                              const typename StagedElem<KIND, T>::E *stage,
                                              long long ch_first, long long chs, int g, int ntx,
                                              float accr) {
    using K = Kind<KIND, T>;
    constexpr unsigned cap = kWindowBytes / sizeof(typename StagedElem<KIND, T>::E);
    float xs[kTapGroup], ap[kTapGroup], fl[kTapGroup];
    bool ok[kTapGroup];
    bool nearb = false;
#pragma unroll
    for (int k = 0; k < kTapGroup; ++k) {
        const float x = __fadd_rn(tt[k], trx);
        const float apod = __fmul_rn(at[k], arx);
        const float q = __fmul_rn(__fsub_rn(x, a.t0), a.inv_dt);
        // |q_fast - q_exact| <= 1.5 ulp(q) <= 1.5 |q| 2^-23; flag within |q| 2^-21
        const float tol = fmaf(fabsf(q), 4.76837158e-7f, 1e-30f);
        float flk;
        bool inr;
        if (KIND == PYCBF_GB_INTERP_NEAREST) {
            flk = truncf(q + 0.5f);
            inr = (x == x) && (flk >= 0.f) && (flk < (float)a.nt);
            nearb |= fabsf(q - floorf(q) - 0.5f) < tol;
        } else {
            flk = floorf(q);
            inr = (x >= a.t0) && (x <= a.xmax);
            nearb |= (q - flk < tol) || (flk + 1.f - q < tol);
        }
        xs[k] = x;
        ap[k] = apod;
        fl[k] = flk;
        ok[k] = inr && (fabsf(apod) >= a.thresh);
    }
    if (nearb) {
#pragma unroll
        for (int k = 0; k < kTapGroup; ++k) {
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
    typename K::P pv[kTapGroup];
#pragma unroll
    for (int k = 0; k < kTapGroup; ++k) {
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
    for (int k = 0; k < kTapGroup; ++k) {
        const float c = fmaf(ap[k], K::value(pv[k], xs[k], fl[k], a), accr);
        accr = ok[k] ? c : accr;
    }
    return accr;
}

template <int KIND, int SUM, typename T>
__global__ void __launch_bounds__(kBlock, 4) das_staged_kernel(const __grid_constant__ DasArgs a,
                                                              const int *__restrict__ plan,
                                                              int *status) {
    using E = typename StagedElem<KIND, T>::E;
    constexpr int kWarps = kBlock / 32;
    constexpr int per16 = 16 / (int)sizeof(E);  // elements per 16-byte copy
    constexpr int kAhead = kStages - 1;          // items staged ahead of the one consumed
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long full[kStages];
    __shared__ __align__(8) unsigned long long empty[kStages];
    __shared__ float s_txlh[2 * kTxReg];
    __shared__ int s_failed;
    // per warp and slot: the stage base (offset - e0) of each transmit's window,
    // written by the warp when it stages the item and read by it when it consumes
    __shared__ __align__(16) int s_base[kStages][kBlock / 32][32];
    __shared__ int s_staged[kStages][kBlock / 32];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const long long tile = blockIdx.x;
    const long long i = tile * kBlock + tid;
    const bool valid = i < a.np;
    const int f = blockIdx.y;
    const int ntx = a.ntx, nrx = a.nrx;
    const long long np = a.np;
    const long long imax = (long long)nrx * kTxGroups;
    const int *rec = plan + kPlanHeaderWords + tile * plan_tile_words(ntx, nrx);
    const int nitems = __ldg(rec);
    const long long frame_ch = (long long)f * ntx * nrx;
    const long long chs = (long long)nrx * a.nt;
    const long long op = valid ? (a.pixel_index ? (long long)__ldg(a.pixel_index + i) : i) : 0;
    int *s_code = reinterpret_cast<int *>(smem_raw + kStages * kStageBytes);
    float *s_rxlh = reinterpret_cast<float *>(s_code + imax);

    if (tid < kStages) {
        mbar_init(&full[tid], kBlock);  // one cp.async arrival per thread
        mbar_init(&empty[tid], kWarps);
    }
    {
        const float *txlh = reinterpret_cast<const float *>(rec + 1 + 3 * imax);
        if (tid < 2 * ntx) s_txlh[tid] = __ldg(txlh + tid);
        for (int k = tid; k < nitems; k += kBlock) s_code[k] = __ldg(rec + 1 + k);
        const float *rxlh = reinterpret_cast<const float *>(rec + 1 + imax);
        for (int k = tid; k < 2 * nitems; k += kBlock) s_rxlh[k] = __ldg(rxlh + k);
    }
    if (tid == 0) s_failed = 0;
    mbar_fence_init();
    __syncthreads();

    // Window table of item `it` in this warp: lane t < ntx holds transmit t's
    // first element e0 and, through the scan, its offset in the stage; returns
    // the stage base (offset - e0) of the lane's transmit and its count.
    auto windows = [&](int it, int &base, int &cnt, int &e0_out, bool &staged) {
        const int code = s_code[it];
        staged = !(code & kItemUnstaged);
        const int t0g = ((code >> 16) & 0xf) * kTapGroup, t1g = ((code >> 20) & 0xf) * kTapGroup;
        const bool mine = lane >= t0g && lane < t1g && lane < ntx;
        int e0 = 0, e1 = 0;
        if (staged && mine) {
            const float xlo = __fadd_rn(s_txlh[2 * lane], s_rxlh[2 * it]);
            const float xhi = __fadd_rn(s_txlh[2 * lane + 1], s_rxlh[2 * it + 1]);
            staged_window<KIND, T>(xlo, xhi, a, e0, e1);
        }
        cnt = e1 - e0;
        int off = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, off, o);
            if (lane >= o) off += v;
        }
        const int total = __shfl_sync(0xffffffffu, off, 31);
        off -= cnt;
        // the plan sized the windows to fit; a plan from other tables could not
        if ((long long)total * (long long)sizeof(E) > kWindowBytes) staged = false;
        base = staged && mine ? off - e0 : 0;
        e0_out = e0;
        if (!staged) cnt = 0;
    };

    // every warp stages its share of item `it`: the windows of transmits
    // w, w+kWarps, ... and, per thread, its pixel's receive row entries
    auto produce = [&](int it) {
        const int slot = it % kStages;
        unsigned char *st = smem_raw + (size_t)slot * kStageBytes;
        const int r = s_code[it] & 0xffff;
        if (valid) {
            cp_async4(st + 4 * tid, a.taurx + (long long)r * np + i);
            cp_async4(st + kRowBytes / 2 + 4 * tid, a.apodrx + (long long)r * np + i);
        }
        int base, cnt, e0;
        bool staged;
        windows(it, base, cnt, e0, staged);
        s_base[slot][w][lane] = base;
        if (lane == 0) s_staged[slot][w] = staged ? 1 : 0;
        if (staged) {
            E *stage = reinterpret_cast<E *>(st + kRowBytes);
            for (int t = w; t < ntx; t += kWarps) {
                const int ct = __shfl_sync(0xffffffffu, cnt, t);
                const int et = __shfl_sync(0xffffffffu, e0, t);
                const int bt = __shfl_sync(0xffffffffu, base, t);
                const E *src = static_cast<const E *>(a.data) + (frame_ch + (long long)t * nrx + r) * a.nt + et;
                for (int k = lane * per16; k < ct; k += 32 * per16) cp_async16(stage + bt + et + k, src + k);
            }
        }
        cp_async_arrive(&full[slot]);
    };

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
    for (int it = 0; it < kAhead && it < nitems; ++it) produce(it);

    float acc = 0.f, s1 = 0.f, accr = 0.f;
    bool failed = false;
    for (int it = 0; it < nitems; ++it) {
        const int slot = it % kStages;
        // stage item it + kAhead into the slot item it - 1 used, once every warp left it
        const int p = it + kAhead;
        if (p < nitems) {
            if (it >= 1 && !mbar_wait_bounded(&empty[(it - 1) % kStages], (unsigned)((it - 1) / kStages) & 1u))
                failed = true;
            if (failed || *(volatile int *)&s_failed) {
                failed = true;
                s_failed = 1;
                break;
            }
            produce(p);
        }
        if (!mbar_wait_bounded(&full[slot], (unsigned)(it / kStages) & 1u)) failed = true;
        if (failed || *(volatile int *)&s_failed) {
            failed = true;
            s_failed = 1;
            break;
        }
        const int code = s_code[it];
        const int r = code & 0xffff;
        const int g0 = (code >> 16) & 0xf, g1 = (code >> 20) & 0xf;
        const float *rows = reinterpret_cast<const float *>(smem_raw + (size_t)slot * kStageBytes);
        const float trx = rows[tid], arx = rows[kBlock + tid];  // not copied past the last pixel: unused

        __syncwarp();
        const bool staged = s_staged[slot][w] != 0;
        const bool live = valid && (__fmul_rn(amax, fabsf(arx)) >= a.thresh);
        if (live) {
            const long long ch_first = (frame_ch + r) * a.nt;
            if (staged) {
                const E *stage =
                    reinterpret_cast<const E *>(smem_raw + (size_t)slot * kStageBytes + kRowBytes);
#pragma unroll
                for (int gg = 0; gg < kTxGroups; ++gg) {
                    if (gg >= g0 && gg < g1) {
                        const int g = gg * kTapGroup;
                        const int4 b4 = *reinterpret_cast<const int4 *>(&s_base[slot][w][g]);
                        const int bk[kTapGroup] = {b4.x, b4.y, b4.z, b4.w};
                        accr = staged_group<KIND, T, true>(a, rtau + g, rapod + g, trx, arx, bk,
                                                           stage, ch_first, chs, g, ntx, accr);
                    }
                }
            } else {
#pragma unroll
                for (int gg = 0; gg < kTxGroups; ++gg) {
                    if (gg >= g0 && gg < g1) {
                        const int g = gg * kTapGroup;
                        const int bk[kTapGroup] = {0, 0, 0, 0};
                        accr = staged_group<KIND, T, false>(a, rtau + g, rapod + g, trx, arx, bk,
                                                            nullptr, ch_first, chs, g, ntx, accr);
                    }
                }
            }
        }
        if (code & kItemLast) {  // this receive is complete
            if (SUM == PYCBF_GB_SUM_TX_AND_RX) acc += accr;
            if (SUM == PYCBF_GB_SUM_TX_ONLY && valid) a.out[((long long)f * nrx + r) * np + op] = accr;
            if (SUM == PYCBF_GB_SUM_DMAS_SSR || SUM == PYCBF_GB_SUM_DMAS_POWER) {
                const float sv = (SUM == PYCBF_GB_SUM_DMAS_SSR) ? copysignf(sqrtf(fabsf(accr)), accr) : accr;
                acc = fmaf(sv, s1, acc);
                s1 += sv;
            }
            accr = 0.f;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[slot]);
    }
    // every thread's own copies are complete before the shared memory goes away
    cp_async_wait_all();
    __syncthreads();
    if (s_failed) {
        if (tid == 0 && status) atomicExch(status, 1);
        if (valid) {
            const float nan = __int_as_float(0x7fc00000);
            if (SUM == PYCBF_GB_SUM_TX_ONLY)
                for (int r = 0; r < nrx; ++r) a.out[((long long)f * nrx + r) * np + op] = nan;
            else
                a.out[(long long)f * np + op] = nan;
        }
        return;
    }
    if (valid && SUM != PYCBF_GB_SUM_TX_ONLY) a.out[(long long)f * np + op] = acc;
}

inline size_t staged_smem_bytes(int nrx) {
    return (size_t)kStages * kStageBytes + sizeof(int) * 3 * (size_t)nrx * kTxGroups;
}

template <int KIND, typename T>
cudaError_t launch_plan_one(const DasArgs &a, int *plan, cudaStream_t s) {
    const long long tiles = (a.np + kBlock - 1) / kBlock;
    tabbed_plan_kernel<KIND, T><<<(unsigned)tiles, kBlock, 0, s>>>(a, plan);
    return cudaGetLastError();
}

template <int KIND, int SUM, typename T>
cudaError_t launch_staged_one(const DasArgs &a, const int *plan, int *status, cudaStream_t s) {
    auto kern = das_staged_kernel<KIND, SUM, T>;
    const int smem = (int)staged_smem_bytes(a.nrx);
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (err != cudaSuccess) return err;
    const long long tiles = (a.np + kBlock - 1) / kBlock;
    kern<<<dim3((unsigned)tiles, (unsigned)a.nframes), kBlock, smem, s>>>(a, plan, status);
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

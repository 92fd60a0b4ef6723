// Gradients of the cubic delay-and-sum (no reference counterpart).
//
// Forward (per frame f, pixel p, summed over the taps that contribute):
//   img[p] += w * S_ch(x),  x = tau_tx(p) + tau_rx(p),  ch = (f, tx, rx)
//   S(x) = a y_j + b y_j+1 + (a^3 - a) z_j + (b^3 - b) z_j+1
// with the knot j, fractions a, b and (y, z) of the spline prefilter (whose
// float32 records hold the same cubic as a polynomial in b), z = 1/2 T^-1 D y (T = tridiag(0.5, 2, 0.5) on the interior
// samples, D the second difference; natural ends z_0 = z_nt-1 = 0).
//
// Three kernels, all deterministic (no atomics; every sum has a fixed order):
//   adj_delay_kernel    one thread per pixel: dL/dx = g w S'(x) summed into
//                       dL/dtau_tx (ntx, np) and dL/dtau_rx (nrx, np) for
//                       Tabbed tables, or into dL/ds (np) for the Synthetic
//                       slowness form (x = (D_tx + D_rx) s + t0).
//   adj_scatter_kernel  one CTA per (channel, part of the pixel range): the
//                       transpose of the interpolation into two shared-memory
//                       rows (dL/dy, dL/dz) of the channel, one pair per CTA.
//                       The taps of one warp step are grouped by knot with
//                       match.any and each group's weights are summed in lane
//                       order by its lowest lane, which alone updates the rows
//                       (so no two lanes ever touch one word together); the
//                       warps take turns, in warp order between CTA barriers,
//                       so no two warps do either.
//   adj_finalize_kernel one warp per channel: adds the parts in order, then
//                       the adjoint of the prefilter, dL/drf = dL/dy +
//                       1/2 D^T T^-1 dL/dz (T is symmetric: the same chunked
//                       Thomas recurrences as the forward prefilter).
// Delays are recomputed from the tables or the geometry, never stored per tap;
// the tap decisions (range, threshold, correctly rounded knot) are the forward's.
#include <algorithm>

#include "das_impl.cuh"

namespace pgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarmAdj = 32;  // warm-up of the chunked recurrences (0.268^32 ~ 5e-19)
constexpr size_t kRowSmemMax = 160 * 1024;

// The forward's decisions for one cubic tap; fractions only where it is in range.
__device__ __forceinline__ bool cubic_tap(float x, const DasArgs &a, int &j, float &am, float &b) {
    using K = Kind<PYCBF_GB_INTERP_CUBIC, float>;
    int idx;
    bool fix;
    bool inr = K::index(x, a, idx, fix);
    if (fix) inr = K::index_exact(x, a, idx);
    j = idx;
    am = b = 0.f;
    if (inr) knot_fractions(x, (float)idx, a, am, b);
    return inr;
}

// the upstream gradient of (frame f, receive r) at kernel-order pixel i (g.gk
// holds it in kernel order: gathered through pixel_index when there is one)
__device__ __forceinline__ long long grad_row(int sum, int f, int r, int nrx) {
    return sum == PYCBF_GB_SUM_TX_AND_RX ? (long long)f : (long long)f * nrx + r;
}

__global__ void adj_gather_kernel(const float *__restrict__ gout, const int *__restrict__ pidx,
                                  long long rows, long long np, float *__restrict__ gk) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= rows * np) return;
    const long long row = n / np, i = n - row * np;
    gk[n] = __ldg(gout + row * np + __ldg(pidx + i));
}

// ---------------------------------------------------------------------------
// delays / slowness: gather per pixel
// ---------------------------------------------------------------------------
template <int GEOM, int SUM, typename T>
__global__ void __launch_bounds__(kBlock) adj_delay_kernel(const __grid_constant__ AdjArgs g) {
    using rec = typename CoefRec<T>::raw;
    constexpr int G = 6;  // taps whose record loads are in flight together
    const DasArgs &a = g.d;
    extern __shared__ float sm[];
    const int tid = threadIdx.x;
    const long long i = (long long)blockIdx.x * kBlock + tid;
    if (i >= a.np) return;
    const long long np = a.np;
    const int ntx = a.ntx, nrx = a.nrx, nfr = a.nframes, nt = a.nt;
    const rec *coef = static_cast<const rec *>(a.data);
    // this thread's columns: transmit delay, apodization (Tabbed) or path
    // length (Synthetic), and the dL/dtau_tx accumulator
    float *stau = sm + tid;
    float *sw = stau + (size_t)ntx * kBlock;
    float *sg = sw + (size_t)ntx * kBlock;

    float pnt[3] = {0.f, 0.f, 0.f};
    float slow = 0.f;
    if (GEOM == GEOM_SYNTH_SLOW) {
        for (int k = 0; k < 3; ++k) if (k < a.ndim) pnt[k] = __ldg(a.geo.pnts + i * a.ndim + k);
        slow = __ldg(a.slow + i);
    }
    float amax = 0.f;
    for (int t = 0; t < ntx; ++t) {
        if (GEOM == GEOM_TABBED) {
            stau[(size_t)t * kBlock] = __ldg(a.tautx + (long long)t * np + i);
            const float at = __ldg(a.apodtx + (long long)t * np + i);
            sw[(size_t)t * kBlock] = at;
            sg[(size_t)t * kBlock] = 0.f;
            amax = fmaxf(amax, fabsf(at));
        } else {
            float D, t0add;
            const bool ok = synth_tx_path(a, t, pnt, D, t0add);
            stau[(size_t)t * kBlock] = slow_delay(ok, D, slow, t0add);
            sw[(size_t)t * kBlock] = D;
        }
    }

    float gs = 0.f;
    for (int r = 0; r < nrx; ++r) {
        float trx, arx = 1.f, Drx = 0.f;
        if (GEOM == GEOM_TABBED) {
            trx = __ldg(a.taurx + (long long)r * np + i);
            arx = __ldg(a.apodrx + (long long)r * np + i);
            // the forward's exact reject: no tap of this receive passes the threshold
            if (__fmul_rn(amax, fabsf(arx)) < a.thresh) {
                if (g.grad_taurx) g.grad_taurx[(long long)r * np + i] = 0.f;
                continue;
            }
        } else {
            const bool ok = synth_rx_path(a, r, pnt, Drx);
            if (!ok) continue;
            trx = slow_delay(true, Drx, slow, 0.f);
        }
        float grx = 0.f;
        for (int t0 = 0; t0 < ntx; t0 += G) {
            // the forward's decisions (fast knots, IEEE redo next to a boundary)
            const int nk = min(G, ntx - t0);
            float tt[G], ap[G], sum[G], xs[G], fj[G];
            int jj[G];
#pragma unroll
            for (int k = 0; k < G; ++k) {
                tt[k] = (k < nk) ? stau[(size_t)(t0 + k) * kBlock] : 0.f;
                sum[k] = 0.f;
            }
            unsigned inr, near;
            cubic_knots<G>(a, tt, trx, xs, jj, fj, inr, near);
            unsigned hitm = inr & ((1u << nk) - 1u);
#pragma unroll
            for (int k = 0; k < G; ++k) {
                ap[k] = 1.f;
                if (GEOM == GEOM_TABBED && k < nk) {
                    ap[k] = __fmul_rn(sw[(size_t)(t0 + k) * kBlock], arx);
                    if (!(fabsf(ap[k]) >= a.thresh)) hitm &= ~(1u << k);
                }
            }
            if (!hitm) continue;
            if (hitm & near) cubic_knots_exact<G>(a, xs, jj, fj, hitm & near);
            bool hit[G];
#pragma unroll
            for (int k = 0; k < G; ++k) hit[k] = (hitm >> k) & 1u;
            for (int f = 0; f < nfr; ++f) {
                const float gp = __ldg(g.gk + grad_row(SUM, f, r, nrx) * np + i);
                float4 c[G];
#pragma unroll
                for (int k = 0; k < G; ++k)
                    if (hit[k])
                        c[k] = CoefRec<T>::load(coef + (((long long)f * ntx + t0 + k) * nrx + r) * nt +
                                                jj[k]);
#pragma unroll
                for (int k = 0; k < G; ++k)
                    if (hit[k])
                        sum[k] = fmaf(gp, Kind<PYCBF_GB_INTERP_CUBIC, T>::slope(c[k], xs[k], fj[k], a),
                                      sum[k]);
            }
#pragma unroll
            for (int k = 0; k < G; ++k) {
                if (!hit[k]) continue;
                const int t = t0 + k;
                if (GEOM == GEOM_TABBED) {
                    const float d = ap[k] * sum[k];
                    sg[(size_t)t * kBlock] += d;
                    grx += d;
                } else {
                    gs = fmaf(sum[k], sw[(size_t)t * kBlock] + Drx, gs);  // dx/ds = D_tx + D_rx
                }
            }
        }
        if (GEOM == GEOM_TABBED && g.grad_taurx) g.grad_taurx[(long long)r * np + i] = grx;
    }
    if (GEOM == GEOM_TABBED && g.grad_tautx)
        for (int t = 0; t < ntx; ++t) g.grad_tautx[(long long)t * np + i] = sg[(size_t)t * kBlock];
    if (GEOM == GEOM_SYNTH_SLOW && g.grad_slow) g.grad_slow[i] = gs;
}

// ---------------------------------------------------------------------------
// which receives can contribute to which tiles of kBlock pixels: Tabbed, some
// pixel has fl(max_t |apodtx| * |apodrx|) >= thresh (by monotonic rounding
// every tap of a dead pair fails the threshold); Synthetic, the receive's mask
// accepts some pixel.  One CTA per tile.
// ---------------------------------------------------------------------------
template <int GEOM>
__global__ void __launch_bounds__(kBlock) adj_live_kernel(const __grid_constant__ AdjArgs g) {
    const DasArgs &a = g.d;
    const long long tile = blockIdx.x;
    const long long tiles = gridDim.x;
    const long long i = tile * kBlock + threadIdx.x;
    const bool valid = i < a.np;
    float amax = 0.f;
    float pnt[3] = {0.f, 0.f, 0.f};
    if (valid) {
        if (GEOM == GEOM_TABBED)
            for (int t = 0; t < a.ntx; ++t)
                amax = fmaxf(amax, fabsf(__ldg(a.apodtx + (long long)t * a.np + i)));
        else
            for (int k = 0; k < 3; ++k) if (k < a.ndim) pnt[k] = __ldg(a.geo.pnts + i * a.ndim + k);
    }
    for (int r = 0; r < a.nrx; ++r) {
        bool v = false;
        if (valid) {
            if (GEOM == GEOM_TABBED) {
                v = __fmul_rn(amax, fabsf(__ldg(a.apodrx + (long long)r * a.np + i))) >= a.thresh;
            } else {
                float D;
                v = synth_rx_path(a, r, pnt, D);
            }
        }
        v = __syncthreads_or(v);
        if (threadIdx.x == 0) g.live[(long long)r * tiles + tile] = v ? 1 : 0;
    }
}

// ---------------------------------------------------------------------------
// channel data: transpose of the interpolation, per (channel, part)
// ---------------------------------------------------------------------------
template <int GEOM, int SUM>
__global__ void __launch_bounds__(128) adj_scatter_kernel(const __grid_constant__ AdjArgs g,
                                                          long long part_len, int Lp) {
    const DasArgs &a = g.d;
    extern __shared__ float rows[];  // [2][Lp]: dL/dy, dL/dz
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const long long np = a.np;
    const int ntx = a.ntx, nrx = a.nrx;
    const long long nch = (long long)a.nframes * ntx * nrx;
    const long long c = blockIdx.x;  // channel ((f * ntx + t) * nrx + r)
    const int q = blockIdx.y;        // part
    const int r = (int)(c % nrx);
    const int t = (int)((c / nrx) % ntx);
    const int f = (int)(c / ((long long)nrx * ntx));
    float *ry = rows;
    float *rz = ry + Lp;
    for (int n = threadIdx.x; n < 2 * Lp; n += blockDim.x) ry[n] = 0.f;
    __syncthreads();

    const long long i0 = (long long)q * part_len;
    const long long i1 = min(np, i0 + part_len);
    const float *grow = g.gk + grad_row(SUM, f, r, nrx) * np;
    // this pixel's inputs, fetched one step ahead: Tabbed apodtx, apodrx,
    // tautx, taurx; Synthetic the point and its slowness; the upstream gradient
    struct In {
        float v[4];
        float gp;
    };
    auto fetch = [&](long long i, In &in) {
        if (i >= i1) return;
        if (GEOM == GEOM_TABBED) {
            in.v[0] = __ldg(a.apodtx + (long long)t * np + i);
            in.v[1] = __ldg(a.apodrx + (long long)r * np + i);
            in.v[2] = __ldg(a.tautx + (long long)t * np + i);
            in.v[3] = __ldg(a.taurx + (long long)r * np + i);
        } else {
            for (int k = 0; k < 3; ++k) if (k < a.ndim) in.v[k] = __ldg(a.geo.pnts + i * a.ndim + k);
            in.v[3] = __ldg(a.slow + i);
        }
        in.gp = __ldg(grow + i);
    };
    // steps of blockDim pixels whose tile receive r can contribute to; the
    // others are skipped (the same for every thread of the CTA)
    const unsigned char *rx_live = g.live + (long long)r * ((np + kBlock - 1) / kBlock);
    auto next_live = [&](long long b) {
        while (b < i1 && !rx_live[b / kBlock]) b += blockDim.x;
        return b;
    };
    // one live step's tap of this lane: knot, fractions and the weighted gradient
    struct Tap {
        bool hit;
        int j;
        float am, b, v;
    };
    auto tap_of = [&](long long base, const In &in) {
        Tap tp = {false, 0, 0.f, 0.f, 0.f};
        const long long i = base + threadIdx.x;
        if (base >= i1 || i >= i1) return tp;
        float x = 0.f, apod = 1.f;
        bool live;
        if (GEOM == GEOM_TABBED) {
            apod = __fmul_rn(in.v[0], in.v[1]);
            live = fabsf(apod) >= a.thresh;
            x = __fadd_rn(in.v[2], in.v[3]);
        } else {
            const float pnt[3] = {in.v[0], in.v[1], in.v[2]};
            float Dt, t0add, Dr;
            const bool okt = synth_tx_path(a, t, pnt, Dt, t0add);
            const bool okr = synth_rx_path(a, r, pnt, Dr);
            live = okt && okr;
            x = __fadd_rn(slow_delay(true, Dt, in.v[3], t0add), slow_delay(true, Dr, in.v[3], 0.f));
        }
        if (live && cubic_tap(x, a, tp.j, tp.am, tp.b)) {
            tp.hit = true;
            tp.v = (GEOM == GEOM_TABBED) ? in.gp * apod : in.gp;
        }
        return tp;
    };
    // the warp's taps of one step into its rows: grouped by knot, the lowest
    // lane of a group sums the group's weights in lane order
    auto scatter = [&](const Tap &tp) {
        if (!__any_sync(kFull, tp.hit)) return;
        const unsigned grp = __match_any_sync(kFull, tp.hit ? tp.j : -1);
        const int n = __popc(grp);
        const int nmax = (int)__reduce_max_sync(kFull, tp.hit ? (unsigned)n : 0u);
        const float wa = tp.v * tp.am, wb = tp.v * tp.b;
        const float wc = tp.v * fmaf(tp.am * tp.am, tp.am, -tp.am);
        const float wd = tp.v * fmaf(tp.b * tp.b, tp.b, -tp.b);
        float A = wa, B = wb, C = wc, D = wd;
        unsigned rest = grp & (grp - 1u);
        for (int k = 1; k < nmax; ++k) {
            const int src = rest ? __ffs(rest) - 1 : lane;
            rest &= rest - 1u;
            const float xa = __shfl_sync(kFull, wa, src), xb = __shfl_sync(kFull, wb, src);
            const float xc = __shfl_sync(kFull, wc, src), xd = __shfl_sync(kFull, wd, src);
            if (k < n) {
                A += xa;
                B += xb;
                C += xc;
                D += xd;
            }
        }
        const bool leader = tp.hit && (lane == __ffs(grp) - 1);
        if (leader) {
            ry[tp.j] += A;
            rz[tp.j] += C;
        }
        __syncwarp();
        if (leader) {
            ry[tp.j + 1] += B;
            rz[tp.j + 1] += D;
        }
        __syncwarp();
    };
    // live steps two at a time (their taps computed together; each warp adds
    // its two steps' taps in its turn, warps in order), the next two fetched
    // meanwhile
    In c0 = {{0.f, 0.f, 0.f, 0.f}, 0.f}, c1 = c0, n0 = c0, n1 = c0;
    long long b0 = next_live(i0);
    long long b1 = b0 < i1 ? next_live(b0 + blockDim.x) : i1;
    if (b0 < i1) fetch(b0 + threadIdx.x, c0);
    if (b1 < i1) fetch(b1 + threadIdx.x, c1);
    while (b0 < i1) {
        const long long nb0 = b1 < i1 ? next_live(b1 + blockDim.x) : i1;
        const long long nb1 = nb0 < i1 ? next_live(nb0 + blockDim.x) : i1;
        if (nb0 < i1) fetch(nb0 + threadIdx.x, n0);
        if (nb1 < i1) fetch(nb1 + threadIdx.x, n1);
        const Tap t0 = tap_of(b0, c0);
        const Tap t1 = tap_of(b1, c1);
        for (int turn = 0; turn < nw; ++turn) {  // b0 is the same in every thread
            if (w == turn) {
                scatter(t0);
                scatter(t1);
            }
            __syncthreads();
        }
        b0 = nb0;
        b1 = nb1;
        c0 = n0;
        c1 = n1;
    }
    __syncthreads();
    float *dst = g.partial + ((size_t)q * nch + c) * 2 * Lp;
    for (int m = threadIdx.x; m < 2 * Lp; m += blockDim.x) dst[m] = rows[m];
}

// v = T^-1 dL/dz in place of zv (one warp; u: scratch of nt floats), with v_0 =
// v_nt-1 = 0: the chunked recurrences of the forward prefilter (T symmetric)
__device__ __forceinline__ void prefilter_adjoint_warp(float *zv, float *u, int nt,
                                                       const SplineTable &tab, int lane) {
    if (lane == 0) u[0] = 0.f;
    __syncwarp();
    // T v = dL/dz on the interior samples 1..nt-2 (v_0 = v_nt-1 = 0)
    const int C = ((nt + 31) >> 5) | 1;
    const int s = lane * C;
    const int e = min(s + C, nt);
    {
        const int ib = max(s, 1), ie = min(e, nt - 1);
        if (ib < ie) {
            float up = 0.f;
            for (int k = max(1, ib - kWarmAdj); k < ie; ++k) {
                const float uk = fmaf(-0.5f, up, zv[k]) * tab.invp[min(k, kSplineTab - 1)];
                if (k >= ib) u[k] = uk;
                up = uk;
            }
        }
    }
    __syncwarp();  // every lane is past its reads of dL/dz
    {
        const int kb = max(s, 1), ke = min(e, nt - 1);
        if (kb < ke) {
            float vn = 0.f;
            for (int k = min(nt - 2, ke - 1 + kWarmAdj); k >= kb; --k) {
                const float vk = fmaf(tab.c[min(k, kSplineTab - 1)], vn, u[k]);
                if (k < ke) zv[k] = vk;
                vn = vk;
            }
        }
    }
    __syncwarp();
    if (lane == 0) {
        zv[0] = 0.f;
        zv[nt - 1] = 0.f;
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// adjoint of the prefilter, one warp per channel
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
adj_finalize_kernel(const float *__restrict__ partial, int nparts, long long nch, int nt, int Lp,
                    float *__restrict__ grad_rf, const __grid_constant__ SplineTable tab) {
    extern __shared__ float smem[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const long long ch = (long long)blockIdx.x * wpb + w;
    if (ch >= nch) return;
    const int stride = (nt + 4) & ~3;
    float *zv = smem + (size_t)w * 2 * stride;  // dL/dz, then v = T^-1 dL/dz in place
    float *u = zv + stride;
    const float *p0 = partial + (size_t)ch * 2 * Lp;
    const size_t pstride = (size_t)nch * 2 * Lp;  // between parts
    for (int n = lane; n < nt; n += 32) {
        float sz = 0.f;
        for (int q = 0; q < nparts; ++q) sz += p0[q * pstride + Lp + n];
        zv[n] = sz;
    }
    prefilter_adjoint_warp(zv, u, nt, tab, lane);
    float *dst = grad_rf + ch * (long long)nt;
    for (int n = lane; n < nt; n += 32) {
        float sy = 0.f;
        for (int q = 0; q < nparts; ++q) sy += p0[q * pstride + n];
        const float vm = n >= 1 ? zv[n - 1] : 0.f;
        const float vp = n + 1 < nt ? zv[n + 1] : 0.f;
        dst[n] = fmaf(0.5f, vm - 2.f * zv[n] + vp, sy);
    }
}


size_t delay_smem_bytes(int ntx) { return 3 * (size_t)ntx * kBlock * sizeof(float); }

template <int GEOM, int SUM, typename T>
cudaError_t launch_delay_one(const AdjArgs &g, cudaStream_t s) {
    auto kern = adj_delay_kernel<GEOM, SUM, T>;
    const size_t smem = delay_smem_bytes(g.d.ntx);
    if (smem > 48 * 1024) {
        cudaError_t err =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    const long long bx = (g.d.np + kBlock - 1) / kBlock;
    kern<<<(unsigned)bx, kBlock, smem, s>>>(g);
    return cudaGetLastError();
}

template <int GEOM, int SUM>
cudaError_t launch_scatter_one(const AdjArgs &g, cudaStream_t s) {
    const DasArgs &a = g.d;
    const long long nch = (long long)a.nframes * a.ntx * a.nrx;
    const int nparts = adjoint_parts(nch, a.np);
    const int nw = adjoint_rows_warps(a.nt);
    if (nw == 0) return cudaErrorInvalidValue;
    const int Lp = (a.nt + 1 + 3) & ~3;
    const long long per = (a.np + nparts - 1) / nparts;
    const long long part_len = (per + 127) / 128 * 128;
    const long long tiles = (a.np + kBlock - 1) / kBlock;
    adj_live_kernel<GEOM><<<(unsigned)tiles, kBlock, 0, s>>>(g);
    cudaError_t lerr = cudaGetLastError();
    if (lerr != cudaSuccess) return lerr;
    const size_t smem = (size_t)2 * Lp * sizeof(float);
    auto kern = adj_scatter_kernel<GEOM, SUM>;
    cudaError_t err =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    kern<<<dim3((unsigned)nch, (unsigned)nparts), 32 * nw, smem, s>>>(g, part_len, Lp);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;

    static SplineTable tab = [] {
        SplineTable t;
        make_spline_table(&t);
        return t;
    }();
    const size_t per_warp = sizeof(float) * 2 * (size_t)((a.nt + 4) & ~3);
    const int wpb = (int)std::min<size_t>(8, std::max<size_t>(1, (112 * 1024) / per_warp));
    const size_t fsmem = per_warp * wpb;
    err = cudaFuncSetAttribute(adj_finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)fsmem);
    if (err != cudaSuccess) return err;
    const long long blocks = (nch + wpb - 1) / wpb;
    adj_finalize_kernel<<<(unsigned)blocks, 32 * wpb, fsmem, s>>>(g.partial, nparts, nch, a.nt, Lp,
                                                                  g.grad_rf, tab);
    return cudaGetLastError();
}

template <int GEOM, int SUM, typename T>
cudaError_t launch_adjoint_gs(const AdjArgs &g, cudaStream_t s) {
    if (g.grad_tautx || g.grad_taurx || g.grad_slow) {
        cudaError_t err;
        if (GEOM == GEOM_TABBED && g.plan && CoefRec<T>::kPoly) {
            // the forward's staging plan: the delay gradients gather from staged windows
            DasArgs d = g.d;
            d.gk = g.gk;
            d.gtx = g.grad_tautx;
            d.grx = g.grad_taurx;
            err = launch_das_staged_adj(d, SUM, PYCBF_GB_F32, g.plan, s);
        } else {
            err = launch_delay_one<GEOM, SUM, T>(g, s);
        }
        if (err != cudaSuccess) return err;
    }
    if (g.grad_rf) return launch_scatter_one<GEOM, SUM>(g, s);
    return cudaSuccess;
}

template <typename T>
cudaError_t launch_adjoint_t(const AdjArgs &g0, cudaStream_t s) {
    AdjArgs g = g0;
    const bool both = g.sumtype == PYCBF_GB_SUM_TX_AND_RX;
    g.gk = g.gout;
    if (g.d.pixel_index) {
        const long long rows = (long long)g.d.nframes * (both ? 1 : g.d.nrx);
        const long long n = rows * g.d.np;
        adj_gather_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g.gout, g.d.pixel_index, rows,
                                                                     g.d.np, g.gk_buf);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        g.gk = g.gk_buf;
    }
    if (g.geom == GEOM_TABBED)
        return both ? launch_adjoint_gs<GEOM_TABBED, PYCBF_GB_SUM_TX_AND_RX, T>(g, s)
                    : launch_adjoint_gs<GEOM_TABBED, PYCBF_GB_SUM_TX_ONLY, T>(g, s);
    return both ? launch_adjoint_gs<GEOM_SYNTH_SLOW, PYCBF_GB_SUM_TX_AND_RX, T>(g, s)
                : launch_adjoint_gs<GEOM_SYNTH_SLOW, PYCBF_GB_SUM_TX_ONLY, T>(g, s);
}

}  // namespace

int adjoint_parts(long long nch, long long np) {
    // enough (channel, part) CTAs to fill the GPU several times over (~11,000: the
    // 1408-channel workload measured 1.92 ms forward + adjoint at 8 parts against
    // 2.22 at 2), parts of >= 2048 pixels
    long long p = (11264 + nch - 1) / nch;
    p = std::min<long long>(p, std::max<long long>(1, np / 2048));
    return (int)std::max<long long>(1, std::min<long long>(p, 64));
}

int adjoint_rows_warps(int nt) {
    const size_t row = 2 * (size_t)((nt + 1 + 3) & ~3) * sizeof(float);
    return row <= kRowSmemMax ? 4 : 0;
}

size_t adjoint_grad_bytes(long long nframes, long long nrx, long long np) {
    return ((size_t)nframes * (size_t)nrx * (size_t)np * sizeof(float) + 255) & ~(size_t)255;
}

size_t adjoint_partial_bytes(long long nframes, long long ntx, long long nrx, long long np,
                             int nt) {
    const long long nch = nframes * ntx * nrx;
    const size_t Lp = (size_t)((nt + 1 + 3) & ~3);
    return (size_t)adjoint_parts(nch, np) * (size_t)nch * 2 * Lp * sizeof(float);
}

size_t adjoint_workspace_bytes(long long nframes, long long ntx, long long nrx, long long np,
                               int nt) {
    const size_t tiles = (size_t)((np + kBlock - 1) / kBlock);
    return adjoint_grad_bytes(nframes, nrx, np) + adjoint_partial_bytes(nframes, ntx, nrx, np, nt) +
           (((size_t)nrx * tiles + 255) & ~(size_t)255);
}

cudaError_t launch_adjoint(const AdjArgs &g, int dtype, cudaStream_t s) {
    switch (dtype) {
        case PYCBF_GB_F32: return launch_adjoint_t<float>(g, s);
        case PYCBF_GB_F16: return launch_adjoint_t<__half>(g, s);
        case PYCBF_GB_BF16: return launch_adjoint_t<__nv_bfloat16>(g, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_das_synth_slow(const DasArgs &a, int sumtype, int dtype, cudaStream_t s) {
    constexpr int CU = PYCBF_GB_INTERP_CUBIC;
    const bool both = sumtype == PYCBF_GB_SUM_TX_AND_RX;
    switch (dtype) {
        case PYCBF_GB_F32:
            return both ? launch_das_one<GEOM_SYNTH_SLOW, CU, PYCBF_GB_SUM_TX_AND_RX, float, false>(a, s)
                        : launch_das_one<GEOM_SYNTH_SLOW, CU, PYCBF_GB_SUM_TX_ONLY, float, false>(a, s);
        case PYCBF_GB_F16:
            return both ? launch_das_one<GEOM_SYNTH_SLOW, CU, PYCBF_GB_SUM_TX_AND_RX, __half, false>(a, s)
                        : launch_das_one<GEOM_SYNTH_SLOW, CU, PYCBF_GB_SUM_TX_ONLY, __half, false>(a, s);
        case PYCBF_GB_BF16:
            return both ? launch_das_one<GEOM_SYNTH_SLOW, CU, PYCBF_GB_SUM_TX_AND_RX, __nv_bfloat16, false>(a, s)
                        : launch_das_one<GEOM_SYNTH_SLOW, CU, PYCBF_GB_SUM_TX_ONLY, __nv_bfloat16, false>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace pgb

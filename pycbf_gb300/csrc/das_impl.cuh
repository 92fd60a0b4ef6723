// Delay-and-sum kernel template (Tabbed tables or Synthetic geometry).
//
// One thread per pixel; a CTA covers kBlock consecutive table columns (the
// host may store the tables in a locality-friendly pixel order and pass
// pixel_index to scatter the results back).  Loop order: receive outer,
// transmit inner.  The transmit-side delays and weights of a pixel are loaded
// (Tabbed) or computed (Synthetic) once, into registers when ntx <= kTxReg,
// else into this thread's column of shared memory; receive-side values are
// loaded or computed once per receive.  Each tap gathers one coefficient
// record of its channel (cubic) or one/two samples (nearest/linear) through
// the read-only path and accumulates in registers: no atomics, one store per
// output element.
//
// Tap decisions follow the reference's float32 C path exactly:
//   apod = apodtx*apodrx (one rounding), contributes iff |apod| >= thresh
//   x = tautx + taurx (one rounding); cubic/linear need t0 <= x <= xmax with
//   xmax = t0 + dt*(nt-1) rounded as two operations (pycbf.c:77,84);
//   knot j = (int)((x - t0)/dt) and nearest it = (int)((x - t0)/dt + 0.5)
//   use the correctly rounded quotient: the fast reciprocal product is used
//   unless its fraction lies within eps of the decision boundary, where the
//   IEEE division is taken instead.
#pragma once

#include "common.cuh"

namespace pgb {

constexpr int kBlock = 128;
constexpr int kTxReg = 16;
constexpr float kDxMin = 1e-12f;

__device__ __forceinline__ float quotient_near_int(float d, const DasArgs &a) {
    float q = __fmul_rn(d, a.inv_dt);
    const float f = q - floorf(q);
    if (f < a.eps || f > 1.f - a.eps) q = __fdiv_rn(d, a.dt);
    return q;
}

__device__ __forceinline__ float quotient_near_half(float d, const DasArgs &a) {
    float q = __fmul_rn(d, a.inv_dt);
    const float f = q - floorf(q);
    if (fabsf(f - 0.5f) < a.eps) q = __fdiv_rn(d, a.dt);
    return q;
}

// knot j = (int)((x - t0)/dt) for an in-range x (pycbf.c:81)
__device__ __forceinline__ int knot_index(float x, const DasArgs &a) {
    const float q = quotient_near_int(__fsub_rn(x, a.t0), a);
    return min((int)floorf(q), a.nt - 1);
}

// The interpolation fractions as the reference rounds them (pycbf.c:93-98):
// xhi = t0 + dt*(j+1), xlo = t0 + dt*j, a = (xhi - x)/dt, b = (x - xlo)/dt.
// x carries ~q*2^-24 of rounding relative to dt, so deriving b from the
// quotient instead would differ from the reference by that much.
__device__ __forceinline__ void knot_fractions(float x, int j, const DasArgs &a, float &am,
                                               float &b) {
    const float xlo = __fadd_rn(a.t0, __fmul_rn(a.dt, (float)j));
    const float xhi = __fadd_rn(a.t0, __fmul_rn(a.dt, (float)(j + 1)));
    am = __fmul_rn(__fsub_rn(xhi, x), a.inv_dt);
    b = __fmul_rn(__fsub_rn(x, xlo), a.inv_dt);
}

// ---------------------------------------------------------------------------
// interpolation of one channel at delay x; sets idx (census) and inr
// ---------------------------------------------------------------------------
template <int KIND, typename T> struct Interp;

template <typename T> struct Interp<PYCBF_GB_INTERP_CUBIC, T> {
    template <bool LOAD>
    static __device__ __forceinline__ float eval(const void *data, long long ch, float x,
                                                 const DasArgs &a, int &idx, bool &inr) {
        inr = (x >= a.t0) && (x <= a.xmax);
        if (!inr) return 0.f;
        const int j = knot_index(x, a);
        idx = j;
        if (!LOAD) return 0.f;
        using rec = typename CoefRec<T>::raw;
        const float4 c = CoefRec<T>::load(static_cast<const rec *>(data) + ch + j);
        float am, b;
        knot_fractions(x, j, a, am, b);
        const float wa = fmaf(am * am, am, -am);
        const float wb = fmaf(b * b, b, -b);
        return fmaf(am, c.x, fmaf(b, c.y, fmaf(wa, c.z, wb * c.w)));
    }
};

template <typename T> struct Interp<PYCBF_GB_INTERP_LINEAR, T> {
    template <bool LOAD>
    static __device__ __forceinline__ float eval(const void *data, long long ch, float x,
                                                 const DasArgs &a, int &idx, bool &inr) {
        inr = (x >= a.t0) && (x <= a.xmax);
        if (!inr) return 0.f;
        const int j = knot_index(x, a);
        idx = j;
        if (!LOAD) return 0.f;
        const T *y = static_cast<const T *>(data) + ch;
        const float y0 = load_sample(y + j);
        const float y1 = (j + 1 < a.nt) ? load_sample(y + j + 1) : 0.f;
        float am, b;
        knot_fractions(x, j, a, am, b);
        return fmaf(am, y0, b * y1);
    }
};

template <typename T> struct Interp<PYCBF_GB_INTERP_NEAREST, T> {
    template <bool LOAD>
    static __device__ __forceinline__ float eval(const void *data, long long ch, float x,
                                                 const DasArgs &a, int &idx, bool &inr) {
        const float d = __fsub_rn(x, a.t0);
        const float q = quotient_near_half(d, a);
        const int it = __float2int_rz(q + 0.5f);
        inr = (x == x) && (it >= 0) && (it < a.nt);
        if (!inr) return 0.f;
        idx = it;
        if (!LOAD) return 0.f;
        return load_sample(static_cast<const T *>(data) + ch + it);
    }
};

// The reference CUDA linear_interp as written (__engines__.cu:36-53): the two
// weights multiply the same sample, so it returns (nearly) the floor sample.
template <typename T> struct Interp<PYCBF_GB_INTERP_LINEAR_FLOOR, T> {
    template <bool LOAD>
    static __device__ __forceinline__ float eval(const void *data, long long ch, float x,
                                                 const DasArgs &a, int &idx, bool &inr) {
        const T *y = static_cast<const T *>(data) + ch;
        if (x == a.xend) {
            inr = true;
            idx = a.nt - 1;
            return LOAD ? load_sample(y + a.nt - 1) : 0.f;
        }
        const float d = __fsub_rn(x, a.t0);
        const float q = quotient_near_int(d, a);
        const int ixo = __float2int_rz(q);
        inr = (x == x) && (ixo >= 0) && (ixo < a.nt);
        if (!inr) return 0.f;
        idx = ixo;
        if (!LOAD) return 0.f;
        const float frac =
            __fdiv_rn(__fsub_rn(__fsub_rn(x, __fmul_rn((float)ixo, a.dt)), a.t0), a.dt);
        const float v = load_sample(y + ixo);
        return __fadd_rn(__fmul_rn(v, __fsub_rn(1.0f, frac)), __fmul_rn(v, frac));
    }
};

// ---------------------------------------------------------------------------
// synthetic-point delays (__engines__.cu:382-470, acos tests as cos compares).
// A masked delay is returned as +inf so the range test rejects the tap.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void synth_dist(const float *o, const float *n, const float *p, int nd,
                                           float &mag, float &proj) {
    float m2 = 0.f, pr = 0.f;
    for (int k = 0; k < nd; ++k) {
        const float d = __fsub_rn(p[k], __ldg(o + k));
        m2 = __fadd_rn(m2, __fmul_rn(d, d));
        pr = __fadd_rn(pr, __fmul_rn(d, __ldg(n + k)));
    }
    mag = __fsqrt_rn(m2);
    proj = pr;
}

__device__ __forceinline__ float synth_tx_delay(const DasArgs &a, int t, const float *p) {
    const int nd = a.ndim;
    float mag, proj;
    synth_dist(a.geo.ovectx + t * nd, a.geo.nvectx + t * nd, p, nd, mag, proj);
    const float c0 = a.geo.c0;
    const float ala = __ldg(a.geo.alatx + t);
    const float t0 = __ldg(a.geo.t0tx + t);
    if (ala != 0.f) {
        const float sgn = (proj > 0.f) ? 1.f : -1.f;
        const float cosala = __ldg(a.geo.cosalatx + t);
        if (__ldg(a.geo.doftx + t) != 0.f) {
            if ((fabsf(proj) > kDxMin) && (mag > kDxMin) && (fabsf(__fdiv_rn(proj, mag)) >= cosala))
                return __fadd_rn(sgn * __fdiv_rn(mag, c0), t0);
            const float lat = __fsqrt_rn(fabsf(__fsub_rn(__fmul_rn(mag, mag), __fmul_rn(proj, proj))));
            if (lat < __ldg(a.geo.halfdofsintx + t))
                return __fadd_rn(__fdiv_rn(__fmul_rn(proj, __ldg(a.geo.secalatx + t)), c0), t0);
            return __int_as_float(0x7f800000);
        }
        const float tau = (fabsf(proj) > kDxMin) ? __fadd_rn(sgn * __fdiv_rn(mag, c0), t0) : t0;
        const bool off = (mag > kDxMin) && (fabsf(__fdiv_rn(proj, mag)) < cosala);
        return off ? __int_as_float(0x7f800000) : tau;
    }
    return __fdiv_rn(proj, c0);
}

__device__ __forceinline__ float synth_rx_delay(const DasArgs &a, int r, const float *p) {
    const int nd = a.ndim;
    float mag, proj;
    synth_dist(a.geo.ovecrx + r * nd, a.geo.nvecrx + r * nd, p, nd, mag, proj);
    const bool off = (mag > kDxMin) && (__fdiv_rn(proj, mag) < __ldg(a.geo.cosalarx + r));
    return off ? __int_as_float(0x7f800000) : __fdiv_rn(mag, a.geo.c0);
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
template <int GEOM, int KIND, int SUM, typename T, bool CENSUS>
__global__ void __launch_bounds__(kBlock) das_kernel(const __grid_constant__ DasArgs a) {
    extern __shared__ float sm[];
    const int tid = threadIdx.x;
    const long long i = (long long)blockIdx.x * kBlock + tid;
    if (i >= a.np) return;
    const int f = blockIdx.y;
    const long long np = a.np;
    const int ntx = a.ntx, nrx = a.nrx;
    const long long op = a.pixel_index ? (long long)__ldg(a.pixel_index + i) : i;
    const bool in_regs = ntx <= kTxReg;
    const long long frame_ch = (long long)f * ntx * nrx;

    float pnt[3] = {0.f, 0.f, 0.f};
    if (GEOM == GEOM_SYNTH)
        for (int k = 0; k < a.ndim; ++k) pnt[k] = __ldg(a.geo.pnts + i * a.ndim + k);

    // transmit side: registers or this thread's column of shared memory
    float rtau[kTxReg], rapod[kTxReg], racc[kTxReg];
    float *stau = sm + tid;
    float *sapod = stau + (size_t)ntx * kBlock;
    float *sacc = sapod + (GEOM == GEOM_TABBED ? (size_t)ntx * kBlock : 0);
    auto tx_side = [&](int t, float &tau, float &apod) {
        if (GEOM == GEOM_TABBED) {
            tau = __ldg(a.tautx + (long long)t * np + i);
            apod = __ldg(a.apodtx + (long long)t * np + i);
        } else {
            tau = synth_tx_delay(a, t, pnt);
            apod = 1.f;
        }
    };
    if (in_regs) {
#pragma unroll
        for (int k = 0; k < kTxReg; ++k) {
            rtau[k] = 0.f;
            rapod[k] = 0.f;
            racc[k] = 0.f;
            if (k < ntx) tx_side(k, rtau[k], rapod[k]);
        }
    } else {
        for (int k = 0; k < ntx; ++k) {
            float tau, apod;
            tx_side(k, tau, apod);
            stau[(size_t)k * kBlock] = tau;
            if (GEOM == GEOM_TABBED) sapod[(size_t)k * kBlock] = apod;
            if (SUM == PYCBF_GB_SUM_RX_ONLY) sacc[(size_t)k * kBlock] = 0.f;
        }
    }

    float acc = 0.f, s1 = 0.f;
    int cnt = 0;
    long long isum = 0;

    for (int r = 0; r < nrx; ++r) {
        float trx, arx;
        if (GEOM == GEOM_TABBED) {
            trx = __ldg(a.taurx + (long long)r * np + i);
            arx = __ldg(a.apodrx + (long long)r * np + i);
        } else {
            trx = synth_rx_delay(a, r, pnt);
            arx = 1.f;
        }
        float accr = 0.f;
        auto tap = [&](int t, float ttx, float atx) -> float {
            bool hit;
            float apod;
            if (GEOM == GEOM_TABBED) {
                apod = __fmul_rn(atx, arx);
                hit = fabsf(apod) >= a.thresh;
            } else {
                apod = 1.f;
                hit = true;
            }
            float contrib = 0.f;
            if (hit) {
                const float x = __fadd_rn(ttx, trx);
                int idx = 0;
                bool inr;
                const long long ch = (frame_ch + (long long)t * nrx + r) * a.nt;
                const float v = Interp<KIND, T>::template eval<!CENSUS>(a.data, ch, x, a, idx, inr);
                if (inr) {
                    contrib = (GEOM == GEOM_TABBED) ? apod * v : v;
                    if (CENSUS) {
                        cnt += 1;
                        isum += idx;
                    }
                }
            }
            if (!CENSUS && SUM == PYCBF_GB_SUM_NONE)
                a.out[((long long)(f * ntx + t) * nrx + r) * np + op] = contrib;
            return contrib;
        };
        if (in_regs) {
#pragma unroll
            for (int k = 0; k < kTxReg; ++k) {
                if (k < ntx) {
                    const float c = tap(k, rtau[k], rapod[k]);
                    if (SUM == PYCBF_GB_SUM_RX_ONLY) racc[k] += c;
                    else accr += c;
                }
            }
        } else {
            for (int k = 0; k < ntx; ++k) {
                const float ttx = stau[(size_t)k * kBlock];
                const float atx = (GEOM == GEOM_TABBED) ? sapod[(size_t)k * kBlock] : 1.f;
                const float c = tap(k, ttx, atx);
                if (SUM == PYCBF_GB_SUM_RX_ONLY) sacc[(size_t)k * kBlock] += c;
                else accr += c;
            }
        }
        if (SUM == PYCBF_GB_SUM_TX_AND_RX) acc += accr;
        if (!CENSUS && SUM == PYCBF_GB_SUM_TX_ONLY) a.out[((long long)f * nrx + r) * np + op] = accr;
        if (SUM == PYCBF_GB_SUM_DMAS_SSR || SUM == PYCBF_GB_SUM_DMAS_POWER) {
            // pairwise sum over receives i<j of s_i s_j as sum_j s_j * (sum_{i<j} s_i):
            // no cancellation, two FMAs per receive
            const float s = (SUM == PYCBF_GB_SUM_DMAS_SSR) ? copysignf(sqrtf(fabsf(accr)), accr) : accr;
            acc = fmaf(s, s1, acc);
            s1 += s;
        }
    }

    // census launches carry no image buffer (out is NULL): they store counts only
    if (!CENSUS && (SUM == PYCBF_GB_SUM_TX_AND_RX || SUM == PYCBF_GB_SUM_DMAS_SSR ||
                    SUM == PYCBF_GB_SUM_DMAS_POWER))
        a.out[(long long)f * np + op] = acc;
    if (!CENSUS && SUM == PYCBF_GB_SUM_RX_ONLY) {
        for (int k = 0; k < ntx; ++k) {
            float v;
            if (in_regs) {
                v = 0.f;
#pragma unroll
                for (int kk = 0; kk < kTxReg; ++kk)
                    if (kk == k) v = racc[kk];
            } else {
                v = sacc[(size_t)k * kBlock];
            }
            a.out[((long long)f * ntx + k) * np + op] = v;
        }
    }
    if (CENSUS) {
        a.census_count[i] = cnt;
        a.census_isum[i] = isum;
    }
}

inline size_t das_smem_bytes(int geom, int sum, int ntx) {
    if (ntx <= kTxReg) return 0;
    size_t per = (geom == GEOM_TABBED ? 2 : 1) + (sum == PYCBF_GB_SUM_RX_ONLY ? 1 : 0);
    return per * (size_t)ntx * kBlock * sizeof(float);
}

template <int GEOM, int KIND, int SUM, typename T, bool CENSUS>
cudaError_t launch_das_one(const DasArgs &a, cudaStream_t s) {
    const size_t smem = das_smem_bytes(GEOM, SUM, a.ntx);
    auto kern = das_kernel<GEOM, KIND, SUM, T, CENSUS>;
    if (smem > 48 * 1024) {
        cudaError_t err =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    const long long bx = (a.np + kBlock - 1) / kBlock;
    dim3 grid((unsigned)bx, CENSUS ? 1u : (unsigned)a.nframes);
    kern<<<grid, kBlock, smem, s>>>(a);
    return cudaGetLastError();
}

template <int GEOM, int KIND, typename T>
cudaError_t launch_das_sum(const DasArgs &a, int sum, cudaStream_t s) {
    switch (sum) {
        case PYCBF_GB_SUM_NONE: return launch_das_one<GEOM, KIND, PYCBF_GB_SUM_NONE, T, false>(a, s);
        case PYCBF_GB_SUM_TX_ONLY: return launch_das_one<GEOM, KIND, PYCBF_GB_SUM_TX_ONLY, T, false>(a, s);
        case PYCBF_GB_SUM_RX_ONLY: return launch_das_one<GEOM, KIND, PYCBF_GB_SUM_RX_ONLY, T, false>(a, s);
        case PYCBF_GB_SUM_TX_AND_RX: return launch_das_one<GEOM, KIND, PYCBF_GB_SUM_TX_AND_RX, T, false>(a, s);
        case PYCBF_GB_SUM_DMAS_SSR: return launch_das_one<GEOM, KIND, PYCBF_GB_SUM_DMAS_SSR, T, false>(a, s);
        case PYCBF_GB_SUM_DMAS_POWER: return launch_das_one<GEOM, KIND, PYCBF_GB_SUM_DMAS_POWER, T, false>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

template <int GEOM, typename T>
cudaError_t launch_das_geom_type(const DasArgs &a, int interp, int sum, bool census, cudaStream_t s) {
    if (census) {
        switch (interp) {
            case PYCBF_GB_INTERP_CUBIC: return launch_das_one<GEOM, PYCBF_GB_INTERP_CUBIC, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            case PYCBF_GB_INTERP_LINEAR: return launch_das_one<GEOM, PYCBF_GB_INTERP_LINEAR, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            case PYCBF_GB_INTERP_NEAREST: return launch_das_one<GEOM, PYCBF_GB_INTERP_NEAREST, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            case PYCBF_GB_INTERP_LINEAR_FLOOR: return launch_das_one<GEOM, PYCBF_GB_INTERP_LINEAR_FLOOR, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            default: return cudaErrorInvalidValue;
        }
    }
    switch (interp) {
        case PYCBF_GB_INTERP_CUBIC: return launch_das_sum<GEOM, PYCBF_GB_INTERP_CUBIC, T>(a, sum, s);
        case PYCBF_GB_INTERP_LINEAR: return launch_das_sum<GEOM, PYCBF_GB_INTERP_LINEAR, T>(a, sum, s);
        case PYCBF_GB_INTERP_NEAREST: return launch_das_sum<GEOM, PYCBF_GB_INTERP_NEAREST, T>(a, sum, s);
        case PYCBF_GB_INTERP_LINEAR_FLOOR: return launch_das_sum<GEOM, PYCBF_GB_INTERP_LINEAR_FLOOR, T>(a, sum, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace pgb

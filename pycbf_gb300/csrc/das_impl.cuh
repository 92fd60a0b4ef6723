// Delay-and-sum kernel template (Tabbed tables or Synthetic geometry).
//
// One thread per pixel; a CTA covers kBlock consecutive table columns (the
// host may store the tables in a locality-friendly pixel order and pass
// pixel_index to scatter the results back).  Loop order: receive outer,
// transmit inner.  The transmit-side delays and weights of a pixel are loaded
// (Tabbed) or computed (Synthetic) once, into registers when ntx <= kTxReg;
// beyond, the delays go to this thread's column of shared memory and the
// Tabbed weights are read from the table per receive (L1-resident rows);
// receive-side values are loaded or computed once per receive.  Each tap gathers one coefficient
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

#include <type_traits>

#include "common.cuh"

namespace pgb {

constexpr int kTxReg = 12;
// Over receives, TX_AND_RX images are summed in blocks of kRxBlockSum consecutive
// receive indices: the sum over blocks, in order, of each block's sequential
// sum.  Every kernel (generic, staged, batched) sums this way, so they agree
// bit for bit, and the staged kernel can hand a tile's blocks to different CTAs.
constexpr int kRxBlockSum = 64;
constexpr float kDxMin = 1e-12f;

// (int)fl for an integral float 0 <= fl < 2^23 without a conversion instruction
__device__ __forceinline__ int small_int(float fl) {
    return __float_as_int(__fadd_rn(fl, 8388608.0f)) - 0x4B000000;
}

// The interpolation fractions as the reference rounds them (pycbf.c:93-98):
// xhi = t0 + dt*(j+1), xlo = t0 + dt*j, a = (xhi - x)/dt, b = (x - xlo)/dt.
// x carries ~q*2^-24 of rounding relative to dt, so deriving b from the
// quotient instead would differ from the reference by that much.
__device__ __forceinline__ void knot_fractions(float x, float fj, const DasArgs &a, float &am,
                                               float &b) {
    const float xlo = __fadd_rn(a.t0, __fmul_rn(a.dt, fj));
    const float xhi = __fadd_rn(a.t0, __fmul_rn(a.dt, __fadd_rn(fj, 1.0f)));
    am = __fmul_rn(__fsub_rn(xhi, x), a.inv_dt);
    b = __fmul_rn(__fsub_rn(x, xlo), a.inv_dt);
}

// ---------------------------------------------------------------------------
// Interpolation kinds.  Each tap goes through
//   index(x)        fast: in-range flag, sample index, and whether the
//                   reciprocal quotient sits within eps of a decision boundary
//   index_exact(x)  the same with the IEEE quotient (taken only when flagged)
//   load(idx)       the channel payload (one 16/8-byte record or 1-2 samples)
//   value(payload)  the interpolated sample
// so that a thread can put the gathers of several taps in flight at once.
// ---------------------------------------------------------------------------
template <int KIND, typename T> struct Kind;

template <typename T> struct Kind<PYCBF_GB_INTERP_CUBIC, T> {
    using P = float4;
    static __device__ __forceinline__ bool index(float x, const DasArgs &a, int &idx, bool &fix) {
        const bool inr = (x >= a.t0) && (x <= a.xmax);
        const float q = __fmul_rn(__fsub_rn(x, a.t0), a.inv_dt);
        const float fl = floorf(q);
        const float f = q - fl;
        fix = (f < a.eps) || (f > 1.f - a.eps);
        idx = min(small_int(fl), a.nt - 1);
        return inr;
    }
    static __device__ __forceinline__ bool index_exact(float x, const DasArgs &a, int &idx) {
        idx = min((int)floorf(__fdiv_rn(__fsub_rn(x, a.t0), a.dt)), a.nt - 1);
        return (x >= a.t0) && (x <= a.xmax);
    }
    static __device__ __forceinline__ P load(const void *data, long long ch, int idx,
                                            const DasArgs &a) {
        using rec = typename CoefRec<T>::raw;
        return CoefRec<T>::load(static_cast<const rec *>(data) + ch + idx);
    }
    // fj: the knot index as a float (exact: j < 2^23).
    // float32 records: b = (x - xlo) / dt with xlo = fl(t0 + fl(dt j)) as the
    // reference rounds it (x - xlo is exact), then the interval's polynomial.
    // 16-bit records (y, z): knot positions (xhi, xlo), fractions (a, b) and
    // cubic weights in packed float32 pairs, each lane rounded as
    // knot_fractions rounds it; b comes from (xlo - x) * -1/dt, the same bits
    // as (x - xlo) * 1/dt.
    static __device__ __forceinline__ float value(const P &c, float x, float fj, const DasArgs &a) {
        if constexpr (CoefRec<T>::kPoly) {
            const float xlo = __fadd_rn(a.t0, __fmul_rn(a.dt, fj));
            const float b = __fmul_rn(__fsub_rn(x, xlo), a.inv_dt);
            return fmaf(fmaf(fmaf(c.w, b, c.z), b, c.y), b, c.x);
        } else {
            const float2 K = add2_rn(make_float2(a.t0, a.t0),
                                     make_float2(__fmul_rn(a.dt, __fadd_rn(fj, 1.0f)), __fmul_rn(a.dt, fj)));
            const float2 AB = mul2_rn(add2_rn(K, make_float2(-x, -x)), make_float2(a.inv_dt, -a.inv_dt));
            const float2 W = fma2_rn(mul2_rn(AB, AB), AB, make_float2(-AB.x, -AB.y));
            return fmaf(AB.x, c.x, fmaf(AB.y, c.y, fmaf(W.x, c.z, W.y * c.w)));
        }
    }
    // dS/dx at x (the delay derivative of the adjoint): d(b)/dx = 1/dt, d(a)/dx = -1/dt
    static __device__ __forceinline__ float slope(const P &c, float x, float fj, const DasArgs &a) {
        if constexpr (CoefRec<T>::kPoly) {
            const float xlo = __fadd_rn(a.t0, __fmul_rn(a.dt, fj));
            const float b = __fmul_rn(__fsub_rn(x, xlo), a.inv_dt);
            return fmaf(fmaf(3.f * c.w, b, 2.f * c.z), b, c.y) * a.inv_dt;
        } else {
            float am, b;
            knot_fractions(x, fj, a, am, b);
            const float da = fmaf(3.f * am, am, -1.f);
            const float db = fmaf(3.f * b, b, -1.f);
            return (c.y - c.x + fmaf(db, c.w, -da * c.z)) * a.inv_dt;
        }
    }
};

template <typename T> struct Kind<PYCBF_GB_INTERP_LINEAR, T> {
    using P = float2;
    static __device__ __forceinline__ bool index(float x, const DasArgs &a, int &idx, bool &fix) {
        return Kind<PYCBF_GB_INTERP_CUBIC, T>::index(x, a, idx, fix);
    }
    static __device__ __forceinline__ bool index_exact(float x, const DasArgs &a, int &idx) {
        return Kind<PYCBF_GB_INTERP_CUBIC, T>::index_exact(x, a, idx);
    }
    static __device__ __forceinline__ P load(const void *data, long long ch, int idx,
                                            const DasArgs &a) {
        const T *y = static_cast<const T *>(data) + ch;
        return make_float2(load_sample(y + idx), idx + 1 < a.nt ? load_sample(y + idx + 1) : 0.f);
    }
    static __device__ __forceinline__ float value(const P &c, float x, float fj, const DasArgs &a) {
        float am, b;
        knot_fractions(x, fj, a, am, b);
        return fmaf(am, c.x, b * c.y);
    }
};

template <typename T> struct Kind<PYCBF_GB_INTERP_NEAREST, T> {
    using P = float;
    static __device__ __forceinline__ bool index(float x, const DasArgs &a, int &idx, bool &fix) {
        const float q = __fmul_rn(__fsub_rn(x, a.t0), a.inv_dt);
        const float f = q - floorf(q);
        fix = fabsf(f - 0.5f) < a.eps;
        const int it = __float2int_rz(q + 0.5f);
        idx = it;
        return (x == x) && (it >= 0) && (it < a.nt);
    }
    static __device__ __forceinline__ bool index_exact(float x, const DasArgs &a, int &idx) {
        const int it = __float2int_rz(__fdiv_rn(__fsub_rn(x, a.t0), a.dt) + 0.5f);
        idx = it;
        return (x == x) && (it >= 0) && (it < a.nt);
    }
    static __device__ __forceinline__ P load(const void *data, long long ch, int idx,
                                            const DasArgs &a) {
        return load_sample(static_cast<const T *>(data) + ch + idx);
    }
    static __device__ __forceinline__ float value(const P &c, float, float, const DasArgs &) {
        return c;
    }
};

// The reference CUDA linear_interp as written (__engines__.cu:36-53): the two
// weights multiply the same sample, so it returns (nearly) the floor sample.
template <typename T> struct Kind<PYCBF_GB_INTERP_LINEAR_FLOOR, T> {
    using P = float;
    static __device__ __forceinline__ bool index(float x, const DasArgs &a, int &idx, bool &fix) {
        const float q = __fmul_rn(__fsub_rn(x, a.t0), a.inv_dt);
        const float f = q - floorf(q);
        fix = (f < a.eps) || (f > 1.f - a.eps);
        return floor_in_range(x, __float2int_rz(q), a, idx);
    }
    static __device__ __forceinline__ bool index_exact(float x, const DasArgs &a, int &idx) {
        return floor_in_range(x, __float2int_rz(__fdiv_rn(__fsub_rn(x, a.t0), a.dt)), a, idx);
    }
    static __device__ __forceinline__ bool floor_in_range(float x, int ixo, const DasArgs &a,
                                                          int &idx) {
        if (x == a.xend) {
            idx = a.nt - 1;
            return true;
        }
        idx = ixo;
        return (x == x) && (ixo >= 0) && (ixo < a.nt);
    }
    static __device__ __forceinline__ P load(const void *data, long long ch, int idx,
                                            const DasArgs &a) {
        return load_sample(static_cast<const T *>(data) + ch + idx);
    }
    static __device__ __forceinline__ float value(const P &v, float x, float fixo, const DasArgs &a) {
        if (x == a.xend) return v;
        const float frac =
            __fdiv_rn(__fsub_rn(__fsub_rn(x, __fmul_rn(fixo, a.dt)), a.t0), a.dt);
        return __fadd_rn(__fmul_rn(v, __fsub_rn(1.0f, frac)), __fmul_rn(v, frac));
    }
};

// ---------------------------------------------------------------------------
// korder / akima / makima: one float32 record of cubic coefficients per
// interval (poly.cu), whatever the storage type.  Knot ixo = (int)((x-t0)/dt)
// with the correctly rounded quotient; korder fills outside [t0, xfma] or
// past the last knot, akima/makima outside [t0, xfma] and take the last knot
// at x == xfma (__engines__.cu:181-187, 266-269, 318-322).
// ---------------------------------------------------------------------------
template <int KIND, typename T> struct KindPoly {
    using P = float4;
    static __device__ __forceinline__ bool index(float x, const DasArgs &a, int &idx, bool &fix) {
        const float q = __fmul_rn(__fsub_rn(x, a.t0), a.inv_dt);
        const float fl = floorf(q);
        const float f = q - fl;
        fix = (f < a.eps) || (f > 1.f - a.eps);
        return finish(x, fl, a, idx);
    }
    static __device__ __forceinline__ bool index_exact(float x, const DasArgs &a, int &idx) {
        return finish(x, floorf(__fdiv_rn(__fsub_rn(x, a.t0), a.dt)), a, idx);
    }
    static __device__ __forceinline__ bool finish(float x, float fl, const DasArgs &a, int &idx) {
        const float last = (float)(a.nt - 1);
        bool inr = (x >= a.t0) && (x <= a.xfma);
        if (KIND == KIND_POLY_NORM) inr = inr && (fl <= last);
        float j = fminf(fl, last);
        if (KIND == KIND_POLY_DELTA && x == a.xfma) j = last;
        idx = inr ? (int)j : 0;
        return inr;
    }
    static __device__ __forceinline__ P load(const void *data, long long ch, int idx,
                                            const DasArgs &) {
        return __ldg(static_cast<const float4 *>(data) + ch + idx);
    }
    static __device__ __forceinline__ float value(const P &c, float x, float fj, const DasArgs &a) {
        float u;
        if (KIND == KIND_POLY_NORM)
            u = __fdiv_rn(fmaf(-a.dt, fj, __fsub_rn(x, a.t0)), a.dt);
        else
            u = __fsub_rn(x, fmaf(a.dt, fj, a.t0));
        const float s1 = __fadd_rn(c.x, __fmul_rn(c.y, u));
        const float s2 = __fadd_rn(s1, __fmul_rn(__fmul_rn(c.z, u), u));
        return __fadd_rn(s2, __fmul_rn(__fmul_rn(__fmul_rn(c.w, u), u), u));
    }
};
template <typename T> struct Kind<KIND_POLY_NORM, T> : KindPoly<KIND_POLY_NORM, T> {};
template <typename T> struct Kind<KIND_POLY_DELTA, T> : KindPoly<KIND_POLY_DELTA, T> {};

// ---------------------------------------------------------------------------
// synthetic-point delays (__engines__.cu:382-470, acos tests as cos compares).
// A masked delay is returned as +inf so the range test rejects the tap.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void synth_dist(const float *o, const float *n, const float *p, int nd,
                                           float &mag, float &proj) {
    float m2 = 0.f, pr = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // nd <= 3: constant indices keep p in registers
        if (k < nd) {
            const float d = __fsub_rn(p[k], __ldg(o + k));
            m2 = __fadd_rn(m2, __fmul_rn(d, d));
            pr = __fadd_rn(pr, __fmul_rn(d, __ldg(n + k)));
        }
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

// The same geometry as path lengths for the slowness form: a transmit delay
// is D*s + t0add, a receive delay D*s; false where the element masks the point.
__device__ __forceinline__ bool synth_tx_path(const DasArgs &a, int t, const float *p, float &D,
                                              float &t0add) {
    const int nd = a.ndim;
    float mag, proj;
    synth_dist(a.geo.ovectx + t * nd, a.geo.nvectx + t * nd, p, nd, mag, proj);
    const float ala = __ldg(a.geo.alatx + t);
    t0add = 0.f;
    D = proj;
    if (ala == 0.f) return true;
    t0add = __ldg(a.geo.t0tx + t);
    const float sgn = (proj > 0.f) ? 1.f : -1.f;
    const float cosala = __ldg(a.geo.cosalatx + t);
    if (__ldg(a.geo.doftx + t) != 0.f) {
        if ((fabsf(proj) > kDxMin) && (mag > kDxMin) && (fabsf(__fdiv_rn(proj, mag)) >= cosala)) {
            D = sgn * mag;
            return true;
        }
        const float lat = __fsqrt_rn(fabsf(__fsub_rn(__fmul_rn(mag, mag), __fmul_rn(proj, proj))));
        D = __fmul_rn(proj, __ldg(a.geo.secalatx + t));
        return lat < __ldg(a.geo.halfdofsintx + t);
    }
    D = (fabsf(proj) > kDxMin) ? sgn * mag : 0.f;
    return !((mag > kDxMin) && (fabsf(__fdiv_rn(proj, mag)) < cosala));
}

__device__ __forceinline__ bool synth_rx_path(const DasArgs &a, int r, const float *p, float &D) {
    const int nd = a.ndim;
    float mag, proj;
    synth_dist(a.geo.ovecrx + r * nd, a.geo.nvecrx + r * nd, p, nd, mag, proj);
    D = mag;
    return !((mag > kDxMin) && (__fdiv_rn(proj, mag) < __ldg(a.geo.cosalarx + r)));
}

__device__ __forceinline__ float slow_delay(bool ok, float D, float s, float t0add) {
    return ok ? __fadd_rn(__fmul_rn(D, s), t0add) : __int_as_float(0x7f800000);
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
constexpr int kGroup = 6;  // taps whose gathers a thread keeps in flight together
// the same for the fast cubic group over transmits in shared memory: six
// for float32 records; four for 16-bit records, whose (y, z) interpolation
// needs more registers (groups of six cost the 3-D 25-transmit launch 11 %
// in occupancy)
template <typename T> constexpr int kGroupSmem = CoefRec<T>::kPoly ? 6 : 4;

// Fast knots of N cubic taps x_k = fl(tt_k + trx), decided as the staged
// kernel decides them: delay sums and quotients q = fl(fl(x - t0) * fl(1/dt))
// two taps per instruction; s = q - 1/2 plus 1.5 * 2^23 rounds to the knot j
// in the sum's low bits, and where |s - j| <= 1/2 - eps_fast the fast
// quotient and the reference's correctly rounded one floor to the same j.
// Bit k of inr: t0 <= x_k <= xmax; of near: the quotient is closer to an
// integer (or NaN), so the caller redoes the taps it keeps with
// cubic_knots_exact.  For a tap in range and not near, jj[k] <= nt - 1.
template <int N>
__device__ __forceinline__ void cubic_knots(const DasArgs &a, const float *tt, float trx,
                                            float *xs, int *jj, float *fj, unsigned &inr,
                                            unsigned &near) {
    constexpr int NP = (N + 1) / 2;
    const float2 trx2 = make_float2(trx, trx);
    const float2 t02 = make_float2(a.t0, a.t0), inv2 = make_float2(a.inv_dt, a.inv_dt);
    const float2 half2 = make_float2(0.5f, 0.5f), mag2 = make_float2(12582912.f, 12582912.f);
    const float hmax = 0.5f - a.eps_fast;
    inr = near = 0u;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const int k1 = (2 * p + 1 < N) ? 2 * p + 1 : 2 * p;
        const float2 x2 = add2_rn(make_float2(tt[2 * p], tt[k1]), trx2);
        const float2 q2 = mul2_rn(sub2_rn(x2, t02), inv2);
        const float2 s2 = sub2_rn(q2, half2);
        const float2 r2 = add2_rn(s2, mag2);
        const float2 f2 = sub2_rn(r2, mag2);
        const float2 h2 = sub2_rn(s2, f2);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * p + h;
            if (k < N) {
                const float x = h ? x2.y : x2.x;
                xs[k] = x;
                fj[k] = h ? f2.y : f2.x;
                jj[k] = __float_as_int(h ? r2.y : r2.x) - 0x4B400000;
                inr |= (unsigned)((x >= a.t0) && (x <= a.xmax)) << k;
                near |= (unsigned)!(fabsf(h ? h2.y : h2.x) <= hmax) << k;
            }
        }
    }
}

// the knots of the taps in `redo` from the IEEE quotient (the reference's rule)
template <int N>
__device__ __forceinline__ void cubic_knots_exact(const DasArgs &a, const float *xs, int *jj,
                                                  float *fj, unsigned redo) {
    using K = Kind<PYCBF_GB_INTERP_CUBIC, float>;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if ((redo >> k) & 1u) {
            int idx;
            K::index_exact(xs[k], a, idx);
            jj[k] = idx;
            fj[k] = (float)idx;
        }
    }
}

// Cubic taps of up to N transmits k0.. k0+nk-1 of one receive (trx, arx)
// for the generic kernel, the decisions made as the staged kernel makes them:
// delay sums, weights and fast quotients q = fl(fl(x - t0) * fl(1/dt)) two
// taps per instruction; s = q - 1/2 plus 1.5 * 2^23 rounds to the knot j in
// the sum's low bits, and where |s - j| <= 1/2 - eps_fast the fast quotient
// and the reference's correctly rounded one floor to the same j.  A tap that
// contributes (in range, weight past the threshold) with its quotient closer
// to an integer is redone with the IEEE division.  Records are gathered from
// global memory (rec: the receive's channel of transmit k0, chs elements
// between transmits); values and the running sum are those of the generic
// group (Kind::value, one fma per contributing tap, in transmit order), so
// the image bits do not change.
template <int GEOM, typename T, int N>
__device__ __forceinline__ float generic_cubic_group(const DasArgs &a, const float *tt,
                                                     const float *at, int nk, float trx, float arx,
                                                     const typename CoefRec<T>::raw *rec,
                                                     long long chs, float accr) {
    using K = Kind<PYCBF_GB_INTERP_CUBIC, T>;
    constexpr int NP = (N + 1) / 2;
    const float2 trx2 = make_float2(trx, trx), arx2 = make_float2(arx, arx);
    const float2 t02 = make_float2(a.t0, a.t0), inv2 = make_float2(a.inv_dt, a.inv_dt);
    const float2 half2 = make_float2(0.5f, 0.5f), mag2 = make_float2(12582912.f, 12582912.f);
    const float hmax = 0.5f - a.eps_fast;
    float xs[N], ap[N], fj[N];
    int jj[N];
    unsigned hit = 0u, fix = 0u;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const int k1 = (2 * p + 1 < N) ? 2 * p + 1 : 2 * p;
        const float2 x2 = add2_rn(make_float2(tt[2 * p], tt[k1]), trx2);
        const float2 ap2 = (GEOM == GEOM_TABBED) ? mul2_rn(make_float2(at[2 * p], at[k1]), arx2)
                                                 : make_float2(1.f, 1.f);
        const float2 q2 = mul2_rn(sub2_rn(x2, t02), inv2);
        const float2 s2 = sub2_rn(q2, half2);
        const float2 r2 = add2_rn(s2, mag2);
        const float2 f2 = sub2_rn(r2, mag2);
        const float2 h2 = sub2_rn(s2, f2);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * p + h;
            if (k < N) {
                const float x = h ? x2.y : x2.x;
                const float apod = h ? ap2.y : ap2.x;
                const bool contrib = (k < nk) && (x >= a.t0) && (x <= a.xmax) &&
                                     (GEOM != GEOM_TABBED || fabsf(apod) >= a.thresh);
                const bool near = !(fabsf(h ? h2.y : h2.x) <= hmax);
                xs[k] = x;
                ap[k] = apod;
                fj[k] = h ? f2.y : f2.x;
                // a contributing tap has x <= xmax, so its fast knot is <= nt - 1
                jj[k] = __float_as_int(h ? r2.y : r2.x) - 0x4B400000;
                hit |= (unsigned)contrib << k;
                fix |= (unsigned)(contrib && near) << k;
            }
        }
    }
    if (fix) {  // rare: a quotient next to a rounding boundary, redo it exactly
#pragma unroll
        for (int k = 0; k < N; ++k) {
            if ((fix >> k) & 1u) {
                int idx;
                K::index_exact(xs[k], a, idx);
                jj[k] = idx;
                fj[k] = (float)idx;
            }
        }
    }
    typename K::P pv[N];
#pragma unroll
    for (int k = 0; k < N; ++k)
        if ((hit >> k) & 1u) pv[k] = CoefRec<T>::load(rec + (long long)k * chs + jj[k]);
#pragma unroll
    for (int k = 0; k < N; ++k)
        if ((hit >> k) & 1u) accr = fmaf(ap[k], K::value(pv[k], xs[k], fj[k], a), accr);
    return accr;
}

// Where the transmit side of a pixel lives: decided per launch from ntx
// (kTxAuto, one kernel for both), or fixed at compile time so that a kernel
// carries the registers of one form only (kTxRegs: ntx <= kTxReg in
// registers; kTxSmem: the thread's column of shared memory).
constexpr int kTxAuto = 0, kTxRegs = 1, kTxSmem = 2;

// One pixel (table column i of frame f) of the generic delay-and-sum: the
// body of das_kernel, also run by the batched kernel for each of its jobs.
// sm: the CTA's dynamic shared memory (das_smem_bytes), a column per thread.
template <int GEOM, int KIND, int SUM, typename T, bool CENSUS, int TXM = kTxAuto>
__device__ __forceinline__ void das_pixel(const DasArgs &a, long long i, int f, float *sm) {
    using K = Kind<KIND, T>;
    const int tid = threadIdx.x;
    if (i >= a.np) return;
    const long long np = a.np;
    const int ntx = a.ntx, nrx = a.nrx;
    const long long op = a.pixel_index ? (long long)__ldg(a.pixel_index + i) : i;
    const bool in_regs = TXM == kTxAuto ? ntx <= kTxReg : TXM == kTxRegs;
    const long long frame_ch = (long long)f * ntx * nrx;
    const long long chs = (long long)nrx * a.nt;  // channel stride between transmits

    float pnt[3] = {0.f, 0.f, 0.f};
    if (GEOM != GEOM_TABBED)
        for (int k = 0; k < 3; ++k) if (k < a.ndim) pnt[k] = __ldg(a.geo.pnts + i * a.ndim + k);
    const float slow = (GEOM == GEOM_SYNTH_SLOW) ? __ldg(a.slow + i) : 0.f;

    // transmit side: registers (ntx <= kTxReg) or this thread's column of shared memory.
    // Synthetic masks travel as +inf delays, which the range test rejects.
    float rtau[kTxReg], rapod[kTxReg], racc[kTxReg];
    float *stau = sm + tid;
    // Tabbed transmit weights beyond kTxReg are read from the table per
    // receive (L1-resident: a tile's rows), which halves the shared memory of
    // the column form and so raises the CTAs per SM (two -> five at 75 transmits)
    float *sacc = stau + (size_t)ntx * kBlock;
    float amax = 0.f;  // max |apodtx| of this pixel, for the exact receive-level reject
    auto tx_side = [&](int t, float &tau, float &apod) {
        if (GEOM == GEOM_TABBED) {
            tau = __ldg(a.tautx + (long long)t * np + i);
            apod = __ldg(a.apodtx + (long long)t * np + i);
            amax = fmaxf(amax, fabsf(apod));
        } else if (GEOM == GEOM_SYNTH) {
            tau = synth_tx_delay(a, t, pnt);
            apod = 1.f;
        } else {
            float D, t0add;
            const bool ok = synth_tx_path(a, t, pnt, D, t0add);
            tau = slow_delay(ok, D, slow, t0add);
            apod = 1.f;
        }
    };
#pragma unroll
    for (int k = 0; k < kTxReg; ++k) {
        rtau[k] = 0.f;
        rapod[k] = 0.f;
        racc[k] = 0.f;
    }
    if (in_regs) {
#pragma unroll
        for (int k = 0; k < kTxReg; ++k)
            if (k < ntx) tx_side(k, rtau[k], rapod[k]);
    } else {
        for (int k = 0; k < ntx; ++k) {
            float tau, apod;
            tx_side(k, tau, apod);
            stau[(size_t)k * kBlock] = tau;
            if (SUM == PYCBF_GB_SUM_RX_ONLY) sacc[(size_t)k * kBlock] = 0.f;
        }
    }

    float acc = 0.f, s1 = 0.f;
    float bacc = 0.f;  // TX_AND_RX: sequential sum of the current block of kRxBlockSum receives
    int cnt = 0;
    long long isum = 0;

    // receive-side values, fetched one receive ahead
    auto rx_side = [&](int r, float &trx, float &arx) {
        if (GEOM == GEOM_TABBED) {
            trx = __ldg(a.taurx + (long long)r * np + i);
            arx = __ldg(a.apodrx + (long long)r * np + i);
        } else if (GEOM == GEOM_SYNTH) {
            trx = synth_rx_delay(a, r, pnt);
            arx = 1.f;
        } else {
            float D;
            const bool ok = synth_rx_path(a, r, pnt, D);
            trx = slow_delay(ok, D, slow, 0.f);
            arx = 1.f;
        }
    };
    float trx_next = 0.f, arx_next = 0.f;
    if (GEOM == GEOM_TABBED && nrx > 0) rx_side(0, trx_next, arx_next);

    for (int r = 0; r < nrx; ++r) {
        if (SUM == PYCBF_GB_SUM_TX_AND_RX && r > 0 && r % kRxBlockSum == 0) {
            acc += bacc;  // the image is the sum of the blocks' sums, in block order
            bacc = 0.f;
        }
        float trx, arx;
        if (GEOM == GEOM_TABBED) {
            trx = trx_next;
            arx = arx_next;
            if (r + 1 < nrx) rx_side(r + 1, trx_next, arx_next);
        } else {
            rx_side(r, trx, arx);
        }
        // Exact reject of the whole receive: rounding is monotonic, so
        // fl(amax*|arx|) < thresh implies fl(|apodtx*apodrx|) < thresh for every
        // transmit.  A masked synthetic receive has an infinite delay.
        bool live;
        if (GEOM == GEOM_TABBED) live = __fmul_rn(amax, fabsf(arx)) >= a.thresh;
        else live = trx != __int_as_float(0x7f800000);
        if (!live && SUM != PYCBF_GB_SUM_NONE) {
            if (!CENSUS && SUM == PYCBF_GB_SUM_TX_ONLY) a.out[((long long)f * nrx + r) * np + op] = 0.f;
            continue;
        }
        const long long ch0 = (frame_ch + r) * a.nt;  // channel (tx 0, rx r)
        float accr = 0.f;

        // one group of up to kGroup transmits taken from registers or shared memory
        auto group = [&](int k0, int nk, const float *tt, const float *at) {
            float xs[kGroup], ap[kGroup];
            int ix[kGroup];
            unsigned hit = 0u, fix = 0u;
#pragma unroll
            for (int k = 0; k < kGroup; ++k) {
                xs[k] = 0.f;
                ap[k] = 0.f;
                ix[k] = 0;
                if (k < nk) {
                    const float x = __fadd_rn(tt[k], trx);
                    float apod = 1.f;
                    bool h = true;
                    if (GEOM == GEOM_TABBED) {
                        apod = __fmul_rn(at[k], arx);
                        h = fabsf(apod) >= a.thresh;
                    }
                    bool fx;
                    int idx;
                    const bool inr = K::index(x, a, idx, fx);
                    xs[k] = x;
                    ap[k] = apod;
                    ix[k] = idx;
                    hit |= (unsigned)(h && inr) << k;
                    fix |= (unsigned)(h && fx) << k;
                }
            }
            if (fix) {  // rare: a quotient next to a rounding boundary, redo it exactly
#pragma unroll
                for (int k = 0; k < kGroup; ++k) {
                    if ((fix >> k) & 1u) {
                        int idx;
                        const bool inr = K::index_exact(xs[k], a, idx);
                        ix[k] = idx;
                        hit = inr ? (hit | (1u << k)) : (hit & ~(1u << k));
                    }
                }
            }
            typename K::P pv[kGroup];
#pragma unroll
            for (int k = 0; k < kGroup; ++k)
                if ((hit >> k) & 1u) pv[k] = K::load(a.data, ch0 + (long long)(k0 + k) * chs, ix[k], a);
#pragma unroll
            for (int k = 0; k < kGroup; ++k) {
                if (k < nk) {
                    // per-receive sums accumulate with one fma per tap (the staged
                    // kernel does the same, so both give identical bits)
                    constexpr bool kPerTap = SUM == PYCBF_GB_SUM_NONE || SUM == PYCBF_GB_SUM_RX_ONLY;
                    float c = 0.f;
                    if ((hit >> k) & 1u) {
                        if (!CENSUS) {
                            const float v = K::value(pv[k], xs[k], (float)ix[k], a);
                            if (kPerTap) c = (GEOM == GEOM_TABBED) ? ap[k] * v : v;
                            else accr = fmaf(ap[k], v, accr);
                        } else {
                            cnt += 1;
                            isum += ix[k];
                        }
                    }
                    const int t = k0 + k;
                    if (!CENSUS && SUM == PYCBF_GB_SUM_NONE)
                        a.out[(((long long)f * ntx + t) * nrx + r) * np + op] = c;
                    if (SUM == PYCBF_GB_SUM_RX_ONLY) {
                        if (in_regs) {
#pragma unroll
                            for (int kk = 0; kk < kTxReg; ++kk)
                                if (kk == t) racc[kk] += c;
                        } else {
                            sacc[(size_t)t * kBlock] += c;
                        }
                    }
                }
            }
        };

        // cubic sums per receive: the fast-decision groups; the rest (census,
        // per-tap outputs, other kinds) the general group
        constexpr bool kFastCubic = KIND == PYCBF_GB_INTERP_CUBIC && !CENSUS &&
                                    SUM != PYCBF_GB_SUM_NONE && SUM != PYCBF_GB_SUM_RX_ONLY;
        using Rec = typename CoefRec<T>::raw;
        const Rec *rec_r = static_cast<const Rec *>(a.data) + ch0;
        if (in_regs) {
#pragma unroll
            for (int g = 0; g < kTxReg; g += kGroup) {
                if (g < ntx) {
                    if constexpr (kFastCubic)
                        accr = generic_cubic_group<GEOM, T, kGroup>(
                            a, rtau + g, rapod + g, min(kGroup, ntx - g), trx, arx,
                            rec_r + (long long)g * chs, chs, accr);
                    else
                        group(g, min(kGroup, ntx - g), rtau + g, rapod + g);
                }
            }
        } else {
            if constexpr (kFastCubic) {
                for (int g = 0; g < ntx; g += kGroupSmem<T>) {
                    const int nk = min(kGroupSmem<T>, ntx - g);
                    float tt[kGroupSmem<T>], at[kGroupSmem<T>];
#pragma unroll
                    for (int k = 0; k < kGroupSmem<T>; ++k) {
                        tt[k] = (k < nk) ? stau[(size_t)(g + k) * kBlock] : 0.f;
                        at[k] = (GEOM == GEOM_TABBED && k < nk)
                                    ? __ldg(a.apodtx + (long long)(g + k) * np + i)
                                    : 1.f;
                    }
                    accr = generic_cubic_group<GEOM, T, kGroupSmem<T>>(
                        a, tt, at, nk, trx, arx, rec_r + (long long)g * chs, chs, accr);
                }
            } else {
                for (int g = 0; g < ntx; g += kGroup) {
                    const int nk = min(kGroup, ntx - g);
                    float tt[kGroup], at[kGroup];
#pragma unroll
                    for (int k = 0; k < kGroup; ++k) {
                        tt[k] = (k < nk) ? stau[(size_t)(g + k) * kBlock] : 0.f;
                        at[k] = (GEOM == GEOM_TABBED && k < nk)
                                    ? __ldg(a.apodtx + (long long)(g + k) * np + i)
                                    : 1.f;
                    }
                    group(g, nk, tt, at);
                }
            }
        }

        if (SUM == PYCBF_GB_SUM_TX_AND_RX) bacc += accr;
        if (!CENSUS && SUM == PYCBF_GB_SUM_TX_ONLY) a.out[((long long)f * nrx + r) * np + op] = accr;
        if (SUM == PYCBF_GB_SUM_DMAS_SSR || SUM == PYCBF_GB_SUM_DMAS_POWER) {
            // pairwise sum over receives i<j of s_i s_j as sum_j s_j * (sum_{i<j} s_i):
            // no cancellation, two FMAs per receive
            const float s = (SUM == PYCBF_GB_SUM_DMAS_SSR) ? copysignf(sqrtf(fabsf(accr)), accr) : accr;
            acc = fmaf(s, s1, acc);
            s1 += s;
        }
    }

    if (SUM == PYCBF_GB_SUM_TX_AND_RX) acc += bacc;
    // census launches carry no image buffer (out is NULL): they store counts only
    if (!CENSUS && (SUM == PYCBF_GB_SUM_TX_AND_RX || SUM == PYCBF_GB_SUM_DMAS_SSR ||
                    SUM == PYCBF_GB_SUM_DMAS_POWER))
        a.out[(long long)f * np + op] = acc;
    if (!CENSUS && SUM == PYCBF_GB_SUM_RX_ONLY) {
        if (in_regs) {
#pragma unroll
            for (int k = 0; k < kTxReg; ++k)
                if (k < ntx) a.out[((long long)f * ntx + k) * np + op] = racc[k];
        } else {
            for (int k = 0; k < ntx; ++k) a.out[((long long)f * ntx + k) * np + op] = sacc[(size_t)k * kBlock];
        }
    }
    if (CENSUS) {
        a.census_count[i] = cnt;
        a.census_isum[i] = isum;
    }
}

// Five CTAs per SM for the shared-memory form (its registers fit 96 per
// thread; 3-D 25-transmit launches measured 5 % faster than at four).
template <int GEOM, int KIND, int SUM, typename T, bool CENSUS, int TXM>
__global__ void __launch_bounds__(kBlock, TXM == kTxSmem ? 5 : 4) das_kernel(const __grid_constant__ DasArgs a) {
    extern __shared__ float sm[];
    das_pixel<GEOM, KIND, SUM, T, CENSUS, TXM>(a, (long long)blockIdx.x * kBlock + threadIdx.x,
                                          (int)blockIdx.y, sm);
}

// the column form: per transmit the delay (and the RX_ONLY accumulator)
inline size_t das_smem_bytes(int geom, int sum, int ntx) {
    (void)geom;
    if (ntx <= kTxReg) return 0;
    const size_t per = 1 + (sum == PYCBF_GB_SUM_RX_ONLY ? 1 : 0);
    return per * (size_t)ntx * kBlock * sizeof(float);
}

template <int GEOM, int KIND, int SUM, typename T, bool CENSUS, int TXM>
cudaError_t launch_das_txm(const DasArgs &a, cudaStream_t s) {
    const size_t smem = das_smem_bytes(GEOM, SUM, a.ntx);
    auto kern = das_kernel<GEOM, KIND, SUM, T, CENSUS, TXM>;
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

// cubic images: a kernel per transmit-side form (fewer registers each);
// census launches and the other kinds: one kernel for both
template <int GEOM, int KIND, int SUM, typename T, bool CENSUS>
cudaError_t launch_das_one(const DasArgs &a, cudaStream_t s) {
    if constexpr (KIND == PYCBF_GB_INTERP_CUBIC && !CENSUS) {
        if (a.ntx <= kTxReg) return launch_das_txm<GEOM, KIND, SUM, T, CENSUS, kTxRegs>(a, s);
        return launch_das_txm<GEOM, KIND, SUM, T, CENSUS, kTxSmem>(a, s);
    } else {
        return launch_das_txm<GEOM, KIND, SUM, T, CENSUS, kTxAuto>(a, s);
    }
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
        if constexpr (std::is_same<T, float>::value) {
            if (interp == KIND_POLY_NORM)
                return launch_das_one<GEOM, KIND_POLY_NORM, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            if (interp == KIND_POLY_DELTA)
                return launch_das_one<GEOM, KIND_POLY_DELTA, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
        }
        switch (interp) {
            case PYCBF_GB_INTERP_CUBIC: return launch_das_one<GEOM, PYCBF_GB_INTERP_CUBIC, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            case PYCBF_GB_INTERP_LINEAR: return launch_das_one<GEOM, PYCBF_GB_INTERP_LINEAR, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            case PYCBF_GB_INTERP_NEAREST: return launch_das_one<GEOM, PYCBF_GB_INTERP_NEAREST, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            case PYCBF_GB_INTERP_LINEAR_FLOOR: return launch_das_one<GEOM, PYCBF_GB_INTERP_LINEAR_FLOOR, PYCBF_GB_SUM_TX_AND_RX, T, true>(a, s);
            default: return cudaErrorInvalidValue;
        }
    }
    if constexpr (std::is_same<T, float>::value) {  // polynomial records are float32 always
        if (interp == KIND_POLY_NORM) return launch_das_sum<GEOM, KIND_POLY_NORM, T>(a, sum, s);
        if (interp == KIND_POLY_DELTA) return launch_das_sum<GEOM, KIND_POLY_DELTA, T>(a, sum, s);
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

/*
 * pycbf_oracle.c -- CPU oracle for the pycbf beamforming hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py load this library, and only as the checker or as
 * the timed CPU baseline; the product (pycbf_gb300) never links or calls it.
 *
 * What it is: a float32 restatement, in this project's own code, of
 *   - the reference's C path, pycbf/cpu/pycbf.c (natural cubic spline knots,
 *     cubic point evaluation, beamform_cubic, beamform_nearest), and
 *   - the formulas the reference's CUDA kernels and notebooks use for the
 *     paths that have no C code: synthetic-point delays and masks
 *     (pycbf/gpu/__engines__.cu:382-470), linear interpolation
 *     (__engines__.cu:36-53), DMAS (pycbf/gpu/__advanced_engines__.cu:17-61)
 *     and short-lag spatial coherence (examples/advanced_beamforming.ipynb,
 *     cells 2 and 6).
 *
 * Build rule: compiled with -ffp-contract=off so every float operation is
 * rounded on its own, as gcc does for the reference on x86-64.  Where the
 * reference reads one element past a channel (pycbf.c:103 at x == xmax) the
 * oracle reads a zero pad instead; the coefficient there is exactly zero, so
 * the value is the same whenever the reference's stray read is finite.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* natural cubic spline second derivatives: pycbf.c:114-141                 */
/* y has n samples; y2 receives n values; u is scratch of n floats          */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_spline_y2(const float *y, int n, float dx, float *y2, float *u)
{
    if (n <= 0) return;
    const float half = 0.5f;
    y2[0] = 0.0f;
    u[0] = 0.0f;
    for (int i = 1; i < n - 1; ++i) {
        float p = half * y2[i - 1] + 2.0f;
        y2[i] = (half - 1.0f) / p;
        float curv = (y[i + 1] - y[i]) / dx - (y[i] - y[i - 1]) / dx;
        u[i] = (6.0f * curv / (2.0f * dx) - half * u[i - 1]) / p;
    }
    y2[n - 1] = 0.0f;
    for (int k = n - 2; k >= 0; --k) y2[k] = y2[k] * y2[k + 1] + u[k];
}

/* upper end of the sampled interval, pycbf.c:77 (no fused multiply-add)    */
ORC_EXPORT float orc_xmax(float xstart, float dx, int n)
{
    float span = dx * (float)(n - 1);
    return xstart + span;
}

/* ------------------------------------------------------------------------ */
/* cubic evaluation at one point: pycbf.c:68-105                            */
/* y and y2 must hold n+1 values, the last one a zero pad                   */
/* ------------------------------------------------------------------------ */
ORC_EXPORT float orc_cubic_point(float x, const float *y, const float *y2, int n,
                                 float xstart, float dx, float fill)
{
    float xmax = orc_xmax(xstart, dx, n);
    if ((x < xstart) || (x > xmax)) return fill;
    int j = (int)((x - xstart) / dx);
    float xhi = xstart + dx * (float)(j + 1);
    float xlo = xstart + dx * (float)j;
    float a = (xhi - x) / dx;
    float b = (x - xlo) / dx;
    float dx2 = powf(dx, 2.0f);
    float c = (1.0f / 6.0f) * (powf(a, 3.0f) - a) * dx2;
    float d = (1.0f / 6.0f) * (powf(b, 3.0f) - b) * dx2;
    return a * y[j] + b * y[j + 1] + c * y2[j] + d * y2[j + 1];
}

/* knot index of a point that is in range (the j of pycbf.c:81) */
static int orc_cubic_index(float x, float xstart, float dx)
{
    return (int)((x - xstart) / dx);
}

/* padded copy of one channel plus its spline: buffers of n+1 floats */
static void orc_prepare_channel(const float *sig, int nt, float dt,
                                float *ypad, float *y2pad, float *scratch)
{
    memcpy(ypad, sig, sizeof(float) * (size_t)nt);
    ypad[nt] = 0.0f;
    orc_spline_y2(sig, nt, dt, y2pad, scratch);
    y2pad[nt] = 0.0f;
}

/* ------------------------------------------------------------------------ */
/* one (tx, rx) channel, cubic: pycbf.c:179-207 (out is accumulated)        */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_beamform_cubic(float t0, float dt, int nt, const float *sig, int nout,
                                   float thresh, const float *tautx, const float *apodtx,
                                   const float *taurx, const float *apodrx, float *out)
{
    float *buf = (float *)malloc(sizeof(float) * (size_t)(3 * (nt + 1)));
    float *ypad = buf, *y2pad = buf + (nt + 1), *scr = buf + 2 * (nt + 1);
    orc_prepare_channel(sig, nt, dt, ypad, y2pad, scr);
    for (int i = 0; i < nout; ++i) {
        float apod = apodtx[i] * apodrx[i];
        if (fabsf(apod) >= thresh) {
            float x = tautx[i] + taurx[i];
            out[i] += apod * orc_cubic_point(x, ypad, y2pad, nt, t0, dt, 0.0f);
        }
    }
    free(buf);
}

/* time index of nearest-neighbour lookup: pycbf.c:264, the +0.5 is double.  */
/* Values that do not fit an int are reported as -1 (out of range), which is */
/* the decision the reference reaches on both x86-64 and aarch64.            */
static int orc_nearest_index(float x, float t0, float dtu)
{
    float q = (x - t0) / dtu;
    double v = (double)q + 0.5;
    if (!(v > -2147483648.0 && v < 2147483647.0)) return -1;
    return (int)v;
}

/* cubic upsampling of one channel onto usf*(nt-1)+1 samples: pycbf.c:234-253 */
static void orc_upsample(const float *sig, int nt, float t0, float dt, int usf, float *out)
{
    int ntu = usf * (nt - 1) + 1;
    float dtu = dt / (float)usf;
    float *buf = (float *)malloc(sizeof(float) * (size_t)(3 * (nt + 1)));
    float *ypad = buf, *y2pad = buf + (nt + 1), *scr = buf + 2 * (nt + 1);
    orc_prepare_channel(sig, nt, dt, ypad, y2pad, scr);
    for (int it = 0; it < ntu; ++it) {
        float tq = t0 + (float)it * dtu;
        out[it] = orc_cubic_point(tq, ypad, y2pad, nt, t0, dt, 0.0f);
    }
    free(buf);
}

/* ------------------------------------------------------------------------ */
/* one (tx, rx) channel, nearest with optional upsampling: pycbf.c:209-271  */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_beamform_nearest(float t0, float dt, int nt, const float *sig, int nout,
                                     float thresh, const float *tautx, const float *apodtx,
                                     const float *taurx, const float *apodrx, float *out, int usf)
{
    const float *s = sig;
    float *up = NULL;
    int ntu = nt;
    float dtu = dt;
    if (usf != 1) {
        ntu = usf * (nt - 1) + 1;
        dtu = dt / (float)usf;
        up = (float *)malloc(sizeof(float) * (size_t)ntu);
        orc_upsample(sig, nt, t0, dt, usf, up);
        s = up;
    }
    for (int i = 0; i < nout; ++i) {
        float apod = apodtx[i] * apodrx[i];
        int it = orc_nearest_index(tautx[i] + taurx[i], t0, dtu);
        if ((fabsf(apod) >= thresh) && (it >= 0) && (it < ntu)) out[i] += apod * s[it];
    }
    free(up);
}

/* ------------------------------------------------------------------------ */
/* linear interpolation                                                     */
/*   kind 0: the two-point part of the cubic formula, in range [t0, tmax]   */
/*   kind 1: the reference CUDA linear_interp as written                    */
/*           (__engines__.cu:36-53), which returns the floor sample         */
/* ------------------------------------------------------------------------ */
static float orc_linear_point(float x, const float *ypad, int n, float x0, float dx)
{
    float xmax = orc_xmax(x0, dx, n);
    if ((x < x0) || (x > xmax)) return 0.0f;
    int j = (int)((x - x0) / dx);
    float xhi = x0 + dx * (float)(j + 1);
    float xlo = x0 + dx * (float)j;
    float a = (xhi - x) / dx;
    float b = (x - xlo) / dx;
    return a * ypad[j] + b * ypad[j + 1];
}

static float orc_linear_floor_point(float x, const float *y, int n, float x0, float dx)
{
    int ixo = (int)((x - x0) / dx);
    if (x == x0 + dx * (float)n) return y[n - 1];
    if ((ixo < 0) || (ixo >= n)) return 0.0f;
    float frac = (x - (float)ixo * dx - x0) / dx;
    return y[ixo] * (1.0f - frac) + y[ixo] * frac;
}

ORC_EXPORT void orc_beamform_linear(float t0, float dt, int nt, const float *sig, int nout,
                                    float thresh, const float *tautx, const float *apodtx,
                                    const float *taurx, const float *apodrx, float *out, int kind)
{
    float *ypad = (float *)malloc(sizeof(float) * (size_t)(nt + 1));
    memcpy(ypad, sig, sizeof(float) * (size_t)nt);
    ypad[nt] = 0.0f;
    for (int i = 0; i < nout; ++i) {
        float apod = apodtx[i] * apodrx[i];
        if (fabsf(apod) >= thresh) {
            float x = tautx[i] + taurx[i];
            float v = kind ? orc_linear_floor_point(x, ypad, nt, t0, dt)
                           : orc_linear_point(x, ypad, nt, t0, dt);
            out[i] += apod * v;
        }
    }
    free(ypad);
}

/* ------------------------------------------------------------------------ */
/* whole frame, Tabbed: the (tx-major, rx-minor) loop of                    */
/* pycbf/cpu/__core_bf_classes__.py:240-245 with the output offsets of      */
/* :49-61.  interp: 0 cubic, 1 nearest, 2 linear, 3 linear (floor quirk).   */
/* sumtype: 0 none, 1 tx_only, 2 rx_only, 3 tx_and_rx.  out is accumulated. */
/* tx range [tx0, tx1) lets callers split the work across threads.          */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_das_tabbed(int interp, int usf, float t0, float dt, int nt,
                               const float *rf, int ntx, int nrx, long long np, float thresh,
                               const float *tautx, const float *apodtx,
                               const float *taurx, const float *apodrx,
                               int sumtype, float *out, int tx0, int tx1)
{
    for (int itx = tx0; itx < tx1; ++itx) {
        for (int irx = 0; irx < nrx; ++irx) {
            long long off;
            if (sumtype == 0) off = np * ((long long)irx + (long long)itx * nrx);
            else if (sumtype == 1) off = np * irx;
            else if (sumtype == 2) off = np * itx;
            else off = 0;
            const float *sig = rf + ((long long)itx * nrx + irx) * nt;
            const float *ttx = tautx + (long long)itx * np, *atx = apodtx + (long long)itx * np;
            const float *trx = taurx + (long long)irx * np, *arx = apodrx + (long long)irx * np;
            if (interp == 0)
                orc_beamform_cubic(t0, dt, nt, sig, (int)np, thresh, ttx, atx, trx, arx, out + off);
            else if (interp == 1)
                orc_beamform_nearest(t0, dt, nt, sig, (int)np, thresh, ttx, atx, trx, arx, out + off, usf);
            else
                orc_beamform_linear(t0, dt, nt, sig, (int)np, thresh, ttx, atx, trx, arx, out + off,
                                    interp == 3);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* The interpolators the reference has only in its CUDA file: korder cubic  */
/* (__engines__.cu:292-355, S from gpu/__core_bf_classes__.py:366-395),     */
/* akima (:188-269) and makima (:58-183).  The reference compiles them with */
/* NVRTC, whose default contracts x0 + dx*n, x - x0 - dx*n and the korder  */
/* derivative sums into fused multiply-adds; those are fused here          */
/* (orc_madd), every other operation as in the source, one rounding each.   */
/* Out-of-range values are                                                  */
/* the fill 0.  Two reads past the channel in the reference are given       */
/* defined values: an akima/makima index at or past nx-1 (x a hair below    */
/* the last knot with the quotient rounded up) returns y[nx-1].             */
/* orc_set_poly_fusion(0) rounds those multiply-adds in two steps instead,  */
/* as a host build of the reference's kernels does (tests only).            */
/* ------------------------------------------------------------------------ */
static int orc_poly_fused = 1;

ORC_EXPORT void orc_set_poly_fusion(int on) { orc_poly_fused = on != 0; }

/* a * b + c: one rounding (the device contraction) or two */
static inline float orc_madd(float a, float b, float c)
{
    return orc_poly_fused ? fmaf(a, b, c) : a * b + c;
}

ORC_EXPORT int orc_poly_index(int kind, float x, float x0, float dx, int nx)
{
    /* knot index of a tap, or -1 when the fill applies */
    float xn = orc_madd(dx, (float)(nx - 1), x0);
    if (kind == 4) {
        int ixin = (int)((x - x0) / dx);
        if ((x < x0) || (ixin > nx - 1) || (x > xn)) return -1;
        return ixin;
    }
    if (x == xn) return nx - 1;
    if ((x < x0) || (x > xn)) return -1;
    int ixo = (int)((x - x0) / dx);
    return ixo > nx - 1 ? nx - 1 : ixo;
}

static float orc_korder_point(float x, const float *y, int nx, float x0, float dx,
                              const float *S, int k)
{
    int ixin = orc_poly_index(4, x, x0, dx, nx);
    if (ixin < 0) return 0.0f;
    if (ixin == nx - 1) return y[nx - 1];
    int ik0, iy0;
    if (ixin < k / 2) {
        ik0 = ixin;
        iy0 = 0;
    } else if (ixin > nx - k / 2 - 1) {
        ik0 = k - nx + ixin;
        iy0 = nx - k;
    } else {
        ik0 = (k - 1) / 2;
        iy0 = ixin - (k - 1) / 2;
    }
    float y0 = y[ixin], y1 = y[ixin + 1], yp0 = 0.0f, yp1 = 0.0f;
    for (int i = 0; i < k; ++i) {
        yp0 = orc_madd(S[ik0 * k + i], y[iy0 + i], yp0);
        yp1 = orc_madd(S[ik0 * k + k + i], y[iy0 + i], yp1);
    }
    float xnorm = orc_madd(-dx, (float)ixin, x - x0) / dx;
    float a0 = y0, a1 = yp0;
    float a2 = 3.0f * (y1 - y0) - 2.0f * yp0 - yp1;
    float a3 = 2.0f * (y0 - y1) + yp0 + yp1;
    return a0 + a1 * xnorm + a2 * xnorm * xnorm + a3 * xnorm * xnorm * xnorm;
}

/* the one-sided slopes (sp0, sp1) and secant mp0 of interval ixo */
ORC_EXPORT void orc_akima_slopes(const float *y, int nx, int ixo, int makima, float *sp0_,
                                 float *sp1_, float *mp0_)
{
    float mm2 = 0, mm1 = 0, mp0 = 0, mp1 = 0, mp2 = 0, w0, w1, sp0, sp1;
#define ORC_W(p, q) (fabsf((p) - (q)) + (makima ? fabsf((p) + (q)) / 2 : 0.0f))
    if (ixo == 0) {
        mp0 = y[ixo + 1] - y[ixo + 0];
        mp1 = y[ixo + 2] - y[ixo + 1];
        sp0 = mp0;
        sp1 = (mp0 + mp1) / 2;
    } else if (ixo == 1) {
        mm1 = y[ixo + 0] - y[ixo - 1];
        mp0 = y[ixo + 1] - y[ixo - 0];
        mp1 = y[ixo + 2] - y[ixo + 1];
        mp2 = y[ixo + 3] - y[ixo + 2];
        sp0 = (mp0 + mm1) / 2;
        if ((mm1 == mp0) && (mp0 == mp1) && (mp1 == mp2)) sp1 = 0;
        else {
            w0 = ORC_W(mp2, mp1);
            w1 = ORC_W(mp0, mm1);
            sp1 = (w0 * mp0 + w1 * mp1) / (w0 + w1);
        }
    } else if (ixo == nx - 3) {
        mm2 = y[ixo - 1] - y[ixo - 2];
        mm1 = y[ixo + 0] - y[ixo - 1];
        mp0 = y[ixo + 1] - y[ixo - 0];
        mp1 = y[ixo + 2] - y[ixo + 1];
        if ((mm2 == mm1) && (mm1 == mp0) && (mp0 == mp1)) sp0 = 0;
        else {
            w0 = ORC_W(mp1, mp0);
            w1 = ORC_W(mm1, mm2);
            sp0 = (w0 * mm1 + w1 * mp0) / (w0 + w1);
        }
        sp1 = (mp0 + mp1) / 2;
    } else if (ixo == nx - 2) {
        mm1 = y[ixo + 0] - y[ixo - 1];
        mp0 = y[ixo + 1] - y[ixo + 0];
        sp0 = (mm1 + mp0) / 2;
        sp1 = mp0;
    } else {
        mm2 = y[ixo - 1] - y[ixo - 2];
        mm1 = y[ixo + 0] - y[ixo - 1];
        mp0 = y[ixo + 1] - y[ixo + 0];
        mp1 = y[ixo + 2] - y[ixo + 1];
        mp2 = y[ixo + 3] - y[ixo + 2];
        if ((mm2 == mm1) && (mm1 == mp0) && (mp0 == mp1)) sp0 = 0;
        else {
            w0 = ORC_W(mp1, mp0);
            w1 = ORC_W(mm1, mm2);
            sp0 = (w0 * mm1 + w1 * mp0) / (w0 + w1);
        }
        if ((mm1 == mp0) && (mp0 == mp1) && (mp1 == mp2)) sp1 = 0;
        else {
            w0 = ORC_W(mp2, mp1);
            w1 = ORC_W(mp0, mm1);
            sp1 = (w0 * mp0 + w1 * mp1) / (w0 + w1);
        }
    }
#undef ORC_W
    *sp0_ = sp0;
    *sp1_ = sp1;
    *mp0_ = mp0;
}

static float orc_akima_point(float x, const float *y, int nx, float x0, float dx, int makima)
{
    int ixo = orc_poly_index(5, x, x0, dx, nx);
    if (ixo < 0) return 0.0f;
    if (ixo == nx - 1) return y[nx - 1];
    float sp0, sp1, mp0;
    orc_akima_slopes(y, nx, ixo, makima, &sp0, &sp1, &mp0);
    float a = y[ixo];
    float b = sp0;
    float c = (3 * mp0 - 2 * sp0 - sp1) / dx;
    float d = (sp0 + sp1 - 2 * mp0) / (dx * dx);
    float delta = x - orc_madd(dx, (float)ixo, x0);
    return a + b * delta + c * delta * delta + d * delta * delta * delta;
}

/* Tabbed image with kind 4 (korder, S k x k), 5 (akima), 6 (makima); a tap
 * contributes when |apodtx*apodrx| >= thresh and it is in range; sumtype
 * codes as orc_das_tabbed. */
ORC_EXPORT void orc_das_poly(int kind, int k, const float *S, float t0, float dt, int nt,
                             const float *rf, int ntx, int nrx, long long np, float thresh,
                             const float *tautx, const float *apodtx, const float *taurx,
                             const float *apodrx, int sumtype, float *out)
{
    for (int itx = 0; itx < ntx; ++itx)
        for (int irx = 0; irx < nrx; ++irx) {
            long long off;
            if (sumtype == 0) off = np * ((long long)irx + (long long)itx * nrx);
            else if (sumtype == 1) off = np * irx;
            else if (sumtype == 2) off = np * itx;
            else off = 0;
            const float *sig = rf + ((long long)itx * nrx + irx) * nt;
            for (long long i = 0; i < np; ++i) {
                float apod = apodtx[itx * np + i] * apodrx[irx * np + i];
                if (!(fabsf(apod) >= thresh)) continue;
                float x = tautx[itx * np + i] + taurx[irx * np + i];
                if (orc_poly_index(kind, x, t0, dt, nt) < 0) continue;
                float v = kind == 4 ? orc_korder_point(x, sig, nt, t0, dt, S, k)
                                    : orc_akima_point(x, sig, nt, t0, dt, kind == 6);
                out[off + i] += apod * v;
            }
        }
}

/* ------------------------------------------------------------------------ */
/* tap census: per pixel, the number of contributing (tx, rx) taps and the  */
/* sum of their sample indices (knot j for cubic/linear, it for nearest).   */
/* A tap contributes when |apodtx*apodrx| >= thresh and it is in range.     */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_tap_census(int interp, int usf, float t0, float dt, int nt,
                               int ntx, int nrx, long long np, float thresh,
                               const float *tautx, const float *apodtx,
                               const float *taurx, const float *apodrx,
                               int32_t *count, int64_t *isum)
{
    float xmax = orc_xmax(t0, dt, nt);
    int ntu = (interp == 1 && usf != 1) ? usf * (nt - 1) + 1 : nt;
    float dtu = (interp == 1 && usf != 1) ? dt / (float)usf : dt;
    for (int itx = 0; itx < ntx; ++itx)
        for (int irx = 0; irx < nrx; ++irx)
            for (long long i = 0; i < np; ++i) {
                float apod = apodtx[itx * np + i] * apodrx[irx * np + i];
                if (!(fabsf(apod) >= thresh)) continue;
                float x = tautx[itx * np + i] + taurx[irx * np + i];
                int idx;
                if (interp == 1) {
                    idx = orc_nearest_index(x, t0, dtu);
                    if (idx < 0 || idx >= ntu) continue;
                } else if (interp >= 4) {
                    idx = orc_poly_index(interp, x, t0, dt, nt);
                    if (idx < 0) continue;
                } else {
                    if ((x < t0) || (x > xmax)) continue;
                    idx = orc_cubic_index(x, t0, dt);
                }
                count[i] += 1;
                isum[i] += idx;
            }
}

/* ------------------------------------------------------------------------ */
/* synthetic-point delays and masks, restated from                          */
/* pycbf/gpu/__engines__.cu:382-470.  The acos(u) > ala tests are written   */
/* as u < cos(ala) with cos(ala) given per element (cosala), and the        */
/* per-transmit constants sec(ala) = sqrt(1 + tan^2 ala) and                */
/* dof*sin(ala)/2 are given too; the 1e-12 guards are float compares.       */
/* ------------------------------------------------------------------------ */
#define ORC_DX_MIN 1e-12f

ORC_EXPORT void orc_synth_tx(int ndim, const float *foc, const float *nvec, float c0, float t0,
                             float ala, float cosala, float secala, float halfdofsin, float dof,
                             const float *p, float *tau, float *apod)
{
    float mag2 = 0.0f, proj = 0.0f;
    for (int k = 0; k < ndim; ++k) {
        float d = p[k] - foc[k];
        mag2 = mag2 + d * d;
        proj = proj + d * nvec[k];
    }
    float mag = sqrtf(mag2);
    if (ala != 0.0f) {
        float sgn = (proj > 0.0f) ? 1.0f : -1.0f;
        if (dof != 0.0f) {
            if ((fabsf(proj) > ORC_DX_MIN) && (mag > ORC_DX_MIN) && (fabsf(proj / mag) >= cosala)) {
                *tau = sgn * (mag / c0) + t0;
                *apod = 1.0f;
            } else if (sqrtf(fabsf(mag * mag - proj * proj)) < halfdofsin) {
                *tau = proj * secala / c0 + t0;
                *apod = 1.0f;
            } else {
                *tau = 0.0f;
                *apod = 0.0f;
            }
        } else {
            *tau = (fabsf(proj) > ORC_DX_MIN) ? sgn * (mag / c0) + t0 : t0;
            *apod = ((mag > ORC_DX_MIN) && (fabsf(proj / mag) < cosala)) ? 0.0f : 1.0f;
        }
    } else {
        *tau = proj / c0;
        *apod = 1.0f;
    }
}

ORC_EXPORT void orc_synth_rx(int ndim, const float *orig, const float *nvec, float c0,
                             float cosala, const float *p, float *tau, float *apod)
{
    float mag2 = 0.0f, proj = 0.0f;
    for (int k = 0; k < ndim; ++k) {
        float d = p[k] - orig[k];
        mag2 = mag2 + d * d;
        proj = proj + d * nvec[k];
    }
    float mag = sqrtf(mag2);
    *tau = mag / c0;
    *apod = ((mag > ORC_DX_MIN) && (proj / mag < cosala)) ? 0.0f : 1.0f;
}

/* tables for a synthetic geometry: tau/apod (ntx, np) and (nrx, np) */
ORC_EXPORT void orc_synth_tables(int ndim, long long np, const float *pnts, float c0,
                                 int ntx, const float *ovectx, const float *nvectx,
                                 const float *t0tx, const float *alatx, const float *cosalatx,
                                 const float *secalatx, const float *halfdofsintx,
                                 const float *doftx,
                                 int nrx, const float *ovecrx, const float *nvecrx,
                                 const float *cosalarx,
                                 float *tautx, float *apodtx, float *taurx, float *apodrx)
{
    for (int t = 0; t < ntx; ++t)
        for (long long i = 0; i < np; ++i)
            orc_synth_tx(ndim, ovectx + t * ndim, nvectx + t * ndim, c0, t0tx[t], alatx[t],
                         cosalatx[t], secalatx[t], halfdofsintx[t], doftx[t], pnts + i * ndim,
                         tautx + t * np + i, apodtx + t * np + i);
    for (int r = 0; r < nrx; ++r)
        for (long long i = 0; i < np; ++i)
            orc_synth_rx(ndim, ovecrx + r * ndim, nvecrx + r * ndim, c0, cosalarx[r],
                         pnts + i * ndim, taurx + r * np + i, apodrx + r * np + i);
}

/* ------------------------------------------------------------------------ */
/* DMAS over separated images im (nsep, np): for each listed lag L, the     */
/* pairs (i, i+L) with i+L < nsep; ssr adds sign(a*b)*sqrt|a*b|, power adds */
/* a*b (__advanced_engines__.cu:55-60, notebook cell 9 of                   */
/* advanced_beamforming.ipynb).  Sums in double.  out is (np) when sumlags, */
/* else (nlag, np); it is overwritten.                                      */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_dmas(const float *im, long long nsep, long long np, const int *lags, int nlag,
                         int power, int sumlags, float *out)
{
    long long nout = sumlags ? np : (long long)nlag * np;
    for (long long i = 0; i < nout; ++i) out[i] = 0.0f;
    for (long long ip = 0; ip < np; ++ip) {
        double tot = 0.0;
        for (int l = 0; l < nlag; ++l) {
            long long lag = lags[l];
            double acc = 0.0;
            for (long long s = 0; s + lag < nsep; ++s) {
                if (lag < 0) break;
                float prod = im[s * np + ip] * im[(s + lag) * np + ip];
                if (power) acc += (double)prod;
                else {
                    double sg = (prod > 0.0f) ? 1.0 : ((prod < 0.0f) ? -1.0 : 0.0);
                    acc += sg * sqrt(fabs((double)prod));
                }
            }
            if (sumlags) tot += acc;
            else out[(long long)l * np + ip] = (float)acc;
        }
        if (sumlags) out[ip] = (float)tot;
    }
}

/* ------------------------------------------------------------------------ */
/* short-lag spatial coherence, restated from advanced_beamforming.ipynb    */
/* (calc_lagn_coherence, cell 2; pixel loop, cell 6) without decimation.    */
/* im: (nrx, nx, nz) tx-summed per-element image; mask: (nrx, nx, nz)      */
/* receive mask (nonzero = on).  For pixel (ix, iz) the axial kernel is     */
/* rows [max(0, iz-nkern), min(nz, iz+nkern+1)); elements whose mask is on  */
/* for every kernel row are kept, in order; with fewer than nlag+1 kept the */
/* pixel is 0.  For lag m = 1..nlag, R_m = nanmean over kept pairs (e,e+m)  */
/* of mean_z(d_e d_{e+m}) / (s_e s_{e+m}), d = value - kernel mean,         */
/* s = population std (s < 1e-10 -> excluded); out = sum_m R_m / nlag, NaN */
/* when some lag has no valid pair.  Double arithmetic.                     */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_slsc(const float *im, const uint8_t *mask, int nrx, int nx, int nz,
                         int nlag, int nkern, double *out)
{
    int kmax = 2 * nkern + 1;
    double *dev = (double *)malloc(sizeof(double) * (size_t)nrx * (size_t)kmax);
    double *sd = (double *)malloc(sizeof(double) * (size_t)nrx);
    int *sel = (int *)malloc(sizeof(int) * (size_t)nrx);
    for (int ix = 0; ix < nx; ++ix) {
        for (int iz = 0; iz < nz; ++iz) {
            int z0 = iz - nkern < 0 ? 0 : iz - nkern;
            int z1 = iz + nkern + 1 > nz ? nz : iz + nkern + 1;
            int L = z1 - z0;
            int nsel = 0;
            for (int e = 0; e < nrx; ++e) {
                int on = 1;
                for (int z = z0; z < z1; ++z)
                    if (!mask[((long long)e * nx + ix) * nz + z]) { on = 0; break; }
                if (on) sel[nsel++] = e;
            }
            double res = 0.0;
            if (nsel >= nlag + 1) {
                for (int k = 0; k < nsel; ++k) {
                    const float *row = im + ((long long)sel[k] * nx + ix) * nz + z0;
                    double mu = 0.0;
                    for (int z = 0; z < L; ++z) mu += row[z];
                    mu /= L;
                    double var = 0.0;
                    for (int z = 0; z < L; ++z) {
                        double d = row[z] - mu;
                        dev[k * kmax + z] = d;
                        var += d * d;
                    }
                    double s = sqrt(var / L);
                    sd[k] = (s < 1e-10) ? NAN : s;
                }
                for (int m = 1; m <= nlag; ++m) {
                    double acc = 0.0;
                    int cnt = 0;
                    for (int k = 0; k + m < nsel; ++k) {
                        double c = 0.0;
                        for (int z = 0; z < L; ++z) c += dev[k * kmax + z] * dev[(k + m) * kmax + z];
                        c /= L;
                        double r = c / (sd[k] * sd[k + m]);
                        if (!isnan(r)) { acc += r; ++cnt; }
                    }
                    res += (cnt ? acc / cnt : NAN) / nlag;
                }
            }
            out[(long long)ix * nz + iz] = res;
        }
    }
    free(dev);
    free(sd);
    free(sel);
}

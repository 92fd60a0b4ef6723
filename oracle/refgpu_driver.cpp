/*
 * The reference's CUDA delay-and-sum and DMAS kernels run on the CPU (test
 * infrastructure only).  pycbf/gpu/__engines__.cu and __advanced_engines__.cu
 * are compiled from where they lie (their paths arrive as REF_ENGINES and
 * REF_ADVANCED), with refgpu_shim.h standing in for the CUDA built-ins;
 * nothing of them is copied here.  Each entry point below emulates the
 * reference's launch of one kernel: blocks of one thread, run in thread
 * order (one per (frame, transmit, receive, pixel) tap for delay-and-sum),
 * each atomicAdd a plain add.  The launch arguments are the ones
 * the reference's Python classes pass (pycbf/gpu/__core_bf_classes__.py:
 * 176-243 Synthetic, 291-354 Tabbed), including the int32 k that the
 * Synthetic korder kernel receives in a float parameter.
 *
 * What differs from a device run: no fused multiply-adds (built with
 * -ffp-contract=off), the host's sin/tan/acos, and a fixed summation order
 * where the device's atomics add in any order.
 */
#include <string.h>

#include "refgpu_shim.h"
#include REF_ENGINES
#include REF_ADVANCED

namespace {

template <class Kernel>
void launch_taps(long long ntaps, Kernel kernel)
{
    threadIdx = {0u, 0u, 0u};
    blockDim = {1u, 1u, 1u};
    gridDim = {(unsigned int)ntaps, 1u, 1u};
    for (long long b = 0; b < ntaps; ++b) {
        blockIdx = {(unsigned int)b, 0u, 0u};
        kernel();
    }
}

RFInfo rf_info(long long ntx, long long nrx, int ndim, float t0, float dt, int nt)
{
    RFInfo info;
    info.ntx = ntx;
    info.nrx = nrx;
    info.ndim = ndim;
    info.tInfo.x0 = t0;
    info.tInfo.dx = dt;
    info.tInfo.nx = nt;
    return info;
}

}  // namespace

extern "C" {

/* Tabbed: interp 0 nearest, 1 linear, 2 akima, 3 makima (the reference's
 * jumpTable order), or -1 for korder cubic with (k, S).  flag: the
 * reference's sum flag (0 none, 1 tx only, 2 rx only, 3 tx and rx).  out is
 * accumulated into, as the reference's zeroed output is. */
int rgd_tabbed(int interp, int k, const float *S, float t0, float dt, int nt, const float *rf,
               long long ntx, long long nrx, long long np, long long nfr, const float *tautx,
               const float *apodtx, const float *taurx, const float *apodrx, int flag, float *out)
{
    if (interp < -1 || interp > 3 || ntx * nrx * np * nfr >= (1LL << 32)) return 1;
    const RFInfo info = rf_info(ntx, nrx, 0, t0, dt, nt);
    const long long n = nfr * ntx * nrx * np;
    if (interp < 0)
        launch_taps(n, [&] {
            das_bmode_tabbed_korder_cubic(info, rf, tautx, apodtx, taurx, apodrx, k, S, np, out,
                                          nfr, flag);
        });
    else
        launch_taps(n, [&] {
            das_bmode_tabbed_multi_interp(info, rf, tautx, apodtx, taurx, apodrx, interp, np, out,
                                          nfr, flag);
        });
    return 0;
}

/* Synthetic: geometry arrays as the reference's float32 copies (ovec/nvec
 * (n, ndim), t0tx / alatx / doftx / alarx (n)); pnts (np, ndim).  interp as
 * rgd_tabbed; for korder, k is passed as the reference passes it, an int32
 * in the kernel's float parameter. */
int rgd_synthetic(int interp, int k, const float *S, float t0, float dt, int nt, int ndim,
                  const float *rf, long long ntx, long long nrx, long long np, long long nfr,
                  const float *ovectx, const float *nvectx, const float *t0tx, const float *alatx,
                  const float *doftx, const float *ovecrx, const float *nvecrx,
                  const float *alarx, float c0, const float *pnts, int flag, float *out)
{
    if (interp < -1 || interp > 3 || ntx * nrx * np * nfr >= (1LL << 32)) return 1;
    if (ndim != 2 && ndim != 3) return 1;
    const RFInfo info = rf_info(ntx, nrx, ndim, t0, dt, nt);
    const long long n = nfr * ntx * nrx * np;
    if (interp < 0) {
        float k_bits;
        memcpy(&k_bits, &k, sizeof k_bits);
        launch_taps(n, [&] {
            das_bmode_synthetic_korder_cubic(info, rf, ovectx, nvectx, t0tx, alatx, doftx, ovecrx,
                                             nvecrx, alarx, k_bits, S, c0, np, pnts, out, nfr,
                                             flag);
        });
    } else {
        launch_taps(n, [&] {
            das_bmode_synthetic_multi_interp(info, rf, ovectx, nvectx, t0tx, alatx, doftx, ovecrx,
                                             nvecrx, alarx, interp, c0, np, pnts, out, nfr, flag);
        });
    }
    return 0;
}

/* DMAS (calc_dmas, pycbf/gpu/__advanced_engines__.cu:17-61) as the
 * reference's classes launch it (gpu/__advanced_bf_classes__.py:51-63):
 * nthreads emulated threads (their ceil(ntx*nrx*nop/nthread) blocks of
 * nthread), each handling tid < nlag*nsep*np, lag = the lag's position.
 * imout is accumulated into. */
int rgd_dmas(const float *imsep, long long nsep, long long np, const int *lags, int nlag,
             int sumtype, int sumlags, float *imout, long long nthreads)
{
    if (nthreads < 0 || nthreads >= (1LL << 32)) return 1;
    launch_taps(nthreads, [&] {
        calc_dmas(imsep, nsep, np, lags, nlag, sumtype, sumlags, imout);
    });
    return 0;
}

}  /* extern "C" */

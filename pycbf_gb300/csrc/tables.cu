// Delay tables and apodizations of a linear array on a pixel grid, built on
// the GPU (the caller-side step before the Tabbed path).
//
// Restates pycbf/helpers/__full_aperture_2D__.py make_tabs_and_apods_2D
// (:170-203) and the functions it calls: plane-wave (:129-168), diverging
// (:37-84) and focused (:86-127) transmits, receive (:3-35).  The per
// transmit constants (origins, normals, time offsets, acceptance angles) are
// computed by the caller on the host exactly as those functions compute them;
// every per-pixel value is computed here in float64 with one rounding per
// operation, in the order numpy evaluates it (no fused multiply-adds), then
// rounded once to float32 -- what the reference classes do with the float64
// tables (`__core_bf_classes__.py` casts them to float32).
//
// Pixel p is (xout[p / nz], zout[p % nz]): meshgrid(xout, zout, indexing='ij')
// flattened.  One thread per pixel; each writes its column of every table.
#include "common.cuh"

namespace pgb {

namespace {

__device__ __forceinline__ double hyp(double dx, double dz) {
    // numpy's norm of a 2-vector: sqrt(dx*dx + dz*dz), each step rounded
    return __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dz, dz)));
}

__global__ void __launch_bounds__(256) tables_2d_kernel(const __grid_constant__ Tables2D p,
                                                        const double *__restrict__ xele,
                                                        const double *__restrict__ xout,
                                                        const double *__restrict__ zout,
                                                        float *__restrict__ tautx,
                                                        float *__restrict__ apodtx,
                                                        float *__restrict__ taurx,
                                                        float *__restrict__ apodrx) {
    const long long np = (long long)p.nx * p.nz;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const double px = __ldg(xout + i / p.nz), pz = __ldg(zout + i % p.nz);
    const double xneg = __ldg(xele), xpos = __ldg(xele + p.nele - 1);
    const double pi_2 = 1.5707963267948966;  // 0.5 * pi, as numpy forms it

    for (int t = 0; t < p.ntx; ++t) {
        const double *c = p.tx[t];
        double tau, apod = 1.0;
        if (p.txkind == 0) {  // plane wave: (P - O) . N / cm; apod inside the projected aperture
            const double dx = __dsub_rn(px, c[0]), dz = __dsub_rn(pz, c[1]);
            tau = __ddiv_rn(__dadd_rn(__dmul_rn(dx, c[2]), __dmul_rn(dz, c[3])), p.cm);
            // Nperp = (-cos, sin) = (-N.z, N.x); origins (xele[0], 0) and (xele[-1], 0)
            const double nx = -c[3], nz = c[2];
            const double dneg = __dadd_rn(__dmul_rn(__dsub_rn(px, xneg), nx), __dmul_rn(pz, nz));
            const double dpos = __dadd_rn(__dmul_rn(__dsub_rn(px, xpos), nx), __dmul_rn(pz, nz));
            apod = (dneg <= 0.0 && dpos >= 0.0) ? 1.0 : 0.0;
        } else if (p.txkind == 1) {  // diverging: |P - O| / cm - tau0
            tau = __dsub_rn(__ddiv_rn(hyp(__dsub_rn(px, c[0]), __dsub_rn(pz, c[1])), p.cm), c[4]);
        } else {  // focused: sign(proj) |P - O| / cm + t0; apod acos(|proj| / |P - O|) < ala
            const double dx = __dsub_rn(px, c[0]), dz = __dsub_rn(pz, c[1]);
            const double proj = __dadd_rn(__dmul_rn(dx, c[2]), __dmul_rn(dz, c[3]));
            double mag = hyp(dx, dz);
            const double sgn = proj > 0.0 ? 1.0 : (proj < 0.0 ? -1.0 : 0.0);
            tau = __dadd_rn(__ddiv_rn(__dmul_rn(sgn, mag), p.cm), c[4]);
            if (mag < 1e-12) mag = 1e-12;
            apod = (acos(__ddiv_rn(fabs(proj), mag)) < c[5]) ? 1.0 : 0.0;
        }
        tautx[(long long)t * np + i] = __double2float_rn(tau);
        apodtx[(long long)t * np + i] = __double2float_rn(apod);
    }
    // |dx| - dz / (2 fnum) < 0 (the caller passes 2 fnum); dz = pz for every element
    const double half = __ddiv_rn(pz, p.fnum2);
    for (int r = 0; r < p.nele; ++r) {
        const double dx = __dsub_rn(px, __ldg(xele + r)), dz = pz;  // elements at z = 0
        taurx[(long long)r * np + i] = __double2float_rn(__ddiv_rn(hyp(dx, dz), p.cm));
        const bool inside = __dsub_rn(fabs(dx), half) < 0.0;
        double w = inside ? 1.0 : 0.0;
        if (p.hann && inside) {  // Hann weight across the active aperture (an extension)
            const double u = fmin(fmax(__ddiv_rn(dx, fmax(half, 1e-30)), -1.0), 1.0);
            const double cv = cos(__dmul_rn(pi_2, u));
            w = __dmul_rn(cv, cv);
        }
        apodrx[(long long)r * np + i] = __double2float_rn(w);
    }
}

}  // namespace

cudaError_t launch_tables_2d(const Tables2D &p, const double *xele, const double *xout,
                             const double *zout, float *tautx, float *apodtx, float *taurx,
                             float *apodrx, cudaStream_t s) {
    const long long np = (long long)p.nx * p.nz;
    const long long blocks = (np + 255) / 256;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    tables_2d_kernel<<<(unsigned)blocks, 256, 0, s>>>(p, xele, xout, zout, tautx, apodtx, taurx,
                                                      apodrx);
    return cudaGetLastError();
}

}  // namespace pgb

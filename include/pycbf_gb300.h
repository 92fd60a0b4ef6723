/*
 * pycbf_gb300.h -- C ABI of the GB300 (sm_103a) beamforming kernels.
 *
 * Plain C types only: device pointers are `void *` / `float *`, sizes are
 * integers, streams are passed as `void *` (a cudaStream_t; NULL = the legacy
 * default stream).  Every entry point:
 *   - validates its arguments on the host first and returns a status code
 *     (never aborts, never prints);
 *   - allocates no device memory: scratch comes from the caller's workspace
 *     (size from pycbf_gb_workspace_bytes);
 *   - is stream-ordered and does not synchronise;
 *   - keeps no mutable global state, so it is safe to call from several
 *     host threads on distinct outputs.
 * The exception is pycbf_gb_das_tabbed_cubic_noalloc: it takes no
 * workspace, because its scratch is a device array that the library itself
 * holds (a fixed PYCBF_GB_NOALLOC_SCRATCH_BYTES on every GPU that loads the
 * library), and that array is mutable global state shared by all its calls:
 * calls that overlap on the GPU race on it.
 *
 * All arithmetic is float32.  Channel data may be stored as float32, float16,
 * bfloat16 or int16; delays, weights and sums stay float32.
 */
#ifndef PYCBF_GB300_H
#define PYCBF_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PYCBF_GB_ABI_VERSION 1

/* status codes */
enum {
    PYCBF_GB_OK = 0,
    PYCBF_GB_EINVAL = 1,       /* null pointer, negative size or unknown code       */
    PYCBF_GB_ERANGE = 2,       /* sizes beyond what the kernels index                */
    PYCBF_GB_EWORKSPACE = 3,   /* workspace missing or smaller than required         */
    PYCBF_GB_EUNSUPPORTED = 4, /* combination this path does not implement           */
    PYCBF_GB_ECUDA = 5         /* a CUDA call failed: see pycbf_gb_last_cuda_error() */
};

/* Channel-data storage types.  PYCBF_GB_I16: int16 samples (raw converter */
/* counts, as acquisition systems deliver them), converted exactly to      */
/* float32 by the first kernel that reads them -- inside the spline        */
/* prefilter for cubic, one conversion pass into the workspace for         */
/* nearest/linear -- so the host-to-device copy moves 2 bytes a sample.    */
/* Accepted by pycbf_gb_das_tabbed, pycbf_gb_das_synthetic,                */
/* pycbf_gb_spline_coefficients (float32 records) and the plan and census  */
/* calls; other entry points return PYCBF_GB_EUNSUPPORTED (convert first   */
/* with pycbf_gb_convert_i16).                                             */
enum { PYCBF_GB_F32 = 0, PYCBF_GB_F16 = 1, PYCBF_GB_BF16 = 2, PYCBF_GB_I16 = 3 };

/* interpolation kinds */
enum {
    PYCBF_GB_INTERP_NEAREST = 0,      /* pycbf.c:264-267 (usf = 1)                          */
    PYCBF_GB_INTERP_LINEAR = 1,       /* two-point part of the cubic formula, cubic's range */
    PYCBF_GB_INTERP_CUBIC = 2,        /* natural cubic spline, pycbf.c:68-166               */
    PYCBF_GB_INTERP_LINEAR_FLOOR = 3, /* __engines__.cu:36-53 as written (floor sample)     */
    PYCBF_GB_INTERP_KORDER = 4,       /* k-point cubic, __engines__.cu:292-355: _poly calls  */
    PYCBF_GB_INTERP_AKIMA = 5,        /* __engines__.cu:188-269: _poly calls                 */
    PYCBF_GB_INTERP_MAKIMA = 6        /* __engines__.cu:58-183: _poly calls                  */
};

/* how taps are summed; 0..3 are the reference's flag values (__engines__.cu:500-504) */
enum {
    PYCBF_GB_SUM_NONE = 0,        /* out (nframes, ntx, nrx, np)                         */
    PYCBF_GB_SUM_TX_ONLY = 1,     /* out (nframes, nrx, np): summed over transmits       */
    PYCBF_GB_SUM_RX_ONLY = 2,     /* out (nframes, ntx, np): summed over receives        */
    PYCBF_GB_SUM_TX_AND_RX = 3,   /* out (nframes, np)                                   */
    PYCBF_GB_SUM_DMAS_SSR = 4,    /* out (nframes, np): sum over all receive pairs i<j of
                                     sign(a_i a_j) sqrt|a_i a_j|, a = transmit sums       */
    PYCBF_GB_SUM_DMAS_POWER = 5   /* out (nframes, np): sum over all pairs i<j of a_i a_j */
};

/* Channel-data description; mirrors RFInfo of pycbf/gpu/__engines__.cu:369-374
 * plus the frame count and the storage type.  rfdata is (nframes, ntx, nrx, nt),
 * C-contiguous. */
typedef struct pycbf_gb_rfinfo {
    long long ntx;
    long long nrx;
    int ndim;            /* 0 for Tabbed; 2 or 3 for Synthetic                   */
    float t0;            /* time of sample 0 (tInfo.x0)                            */
    float dt;            /* sample period (tInfo.dx)                               */
    int nt;              /* samples per channel (tInfo.nx)                         */
    long long nframes;
    int dtype;           /* PYCBF_GB_F32 / _F16 / _BF16 / _I16                     */
} pycbf_gb_rfinfo;

/* Size limits; beyond them a call returns PYCBF_GB_ERANGE before any CUDA
 * call:
 *   ntx, nrx <= 2^20; nt < 2^22; nframes <= 65535; np < 2^31;
 *   cubic interpolation (the spline prefilter): nt <= 18000;
 *   delay-and-sum: ntx <= 454 (227 with PYCBF_GB_SUM_RX_ONLY), the per-pixel
 *   transmit delays living in shared memory. */

/* Synthetic-point geometry, all device pointers (float32).  The fields follow
 * the Synthetic dataclass (pycbf/__bf_base_classes__.py:166-178).  The acos
 * tests of __engines__.cu:412,427,468 are evaluated as cosine compares, so
 * the caller passes cos(ala) per element, and per transmit sec(ala) =
 * sqrt(1 + tan^2 ala) and dof*sin(ala)/2 (each computed in double, rounded to
 * float). */
typedef struct pycbf_gb_synthetic {
    const float *ovectx;       /* (ntx, ndim) */
    const float *nvectx;       /* (ntx, ndim) */
    const float *t0tx;         /* (ntx)       */
    const float *alatx;        /* (ntx)       */
    const float *doftx;        /* (ntx)       */
    const float *cosalatx;     /* (ntx)       */
    const float *secalatx;     /* (ntx)       */
    const float *halfdofsintx; /* (ntx)       */
    const float *ovecrx;       /* (nrx, ndim) */
    const float *nvecrx;       /* (nrx, ndim) */
    const float *cosalarx;     /* (nrx)       */
    const float *pnts;         /* (np, ndim)  */
    long long np;
    float c0;
} pycbf_gb_synthetic;

/* ---------------------------------------------------------------------- */
/* housekeeping                                                            */
/* ---------------------------------------------------------------------- */
int pycbf_gb_abi_version(void);
const char *pycbf_gb_status_string(int status);
/* cudaError_t of the last failed CUDA call made by this thread (0 if none) */
int pycbf_gb_last_cuda_error(void);

/* Bytes of workspace a Tabbed or Synthetic call with this channel data and
 * interpolation kind needs: the spline coefficients for cubic; for
 * nearest/linear 0, or nframes*ntx*nrx*nt float32 samples for int16 data. */
size_t pycbf_gb_workspace_bytes(const pycbf_gb_rfinfo *rf, int interp);

/* ---------------------------------------------------------------------- */
/* Natural cubic spline coefficients of every channel.                     */
/* Replaces tie_knots1D_fixed (pycbf/cpu/pycbf.c:114-166), which the      */
/* reference runs per channel inside beamform_cubic (pycbf.c:194).        */
/* coef receives, per channel and sample j, one record of the interval    */
/* [t_j, t_j+1] with z = y'' dt^2 / 6 and y_nt = z_nt = 0.  F32 and I16    */
/* channel data: float32 x4, the interval's cubic as a polynomial in the   */
/* fraction b = (x - xlo_j) / dt, (p0, p1, p2, p3) with c_j = (xhi_j -     */
/* xlo_j) / dt for the knots as the reference rounds them:                 */
/*   p0 = c y_j + (c^3 - c) z_j,  p1 = y_j+1 - y_j + (1 - 3c^2) z_j - z_j+1, */
/*   p2 = 3c z_j,  p3 = z_j+1 - z_j;                                       */
/* F16/BF16: (y_j, y_j+1, z_j, z_j+1) in the storage type.  coef must hold */
/* pycbf_gb_workspace_bytes(rf, PYCBF_GB_INTERP_CUBIC) bytes.              */
/* ---------------------------------------------------------------------- */
int pycbf_gb_spline_coefficients(const pycbf_gb_rfinfo *rf, const void *rfdata, void *coef,
                                 size_t coef_bytes, void *stream);

/* ---------------------------------------------------------------------- */
/* Tabbed delay-and-sum.                                                   */
/* Replaces the per-channel C call beamform_cubic / beamform_nearest       */
/* (pycbf/cpu/pycbf.h:27-54, driven by cpu/__core_bf_classes__.py:149-192) */
/* and the CuPy kernels das_bmode_tabbed_korder_cubic /                    */
/* das_bmode_tabbed_multi_interp (pycbf/gpu/__engines__.cu:726-864,        */
/* launched by gpu/__core_bf_classes__.py:291-354).                        */
/*                                                                          */
/* tautx, apodtx: (ntx, np); taurx, apodrx: (nrx, np), float32, device.    */
/* A tap (pixel, tx, rx) contributes when |apodtx*apodrx| >= thresh and    */
/* the delay tautx+taurx is in range (pycbf.c:200-203, 84-87, 264-267).    */
/* pixel_index: NULL, or int32[np]: table column i is written to output    */
/* pixel pixel_index[i] (lets callers store the tables in a                */
/* locality-friendly order).  plan: NULL, or a staging plan built by       */
/* pycbf_gb_tabbed_plan for these tables, this thresh and this interp;     */
/* with it, ntx <= 12 and sumtype tx_only / tx_and_rx / dmas, the kernel   */
/* stages channel windows in shared memory by TMA (same results).  out is  */
/* written, not accumulated.                                               */
/* ---------------------------------------------------------------------- */
int pycbf_gb_das_tabbed(const pycbf_gb_rfinfo *rf, const void *rfdata, const float *tautx,
                        const float *apodtx, const float *taurx, const float *apodrx,
                        long long np, const int *pixel_index, int interp, float thresh,
                        int sumtype, const void *plan, float *out, void *workspace,
                        size_t workspace_bytes, void *stream);

/* Staging plan of a Tabbed table set (no counterpart in the reference: it  */
/* precomputes, per tile of 128 table columns, the receives that can        */
/* contribute and the delay bounds that size each channel window, the tile  */
/* order, and the (tile, block of 64 receives) work items of single-frame   */
/* calls).  plan needs pycbf_gb_tabbed_plan_bytes bytes, 16-byte aligned;   */
/* ntx <= 12.  Its first int32 is a status word: 0, or 1 after a kernel     */
/* gave up a bounded wait (its outputs are then NaN).  Its second is the    */
/* work-queue head of the staged kernel; the plan also holds per-tile       */
/* counters and one frame's block partial sums, all reset or rewritten by   */
/* every call that uses the plan: calls sharing one plan must not overlap   */
/* on the GPU.  Images are sums over blocks of 64 receives (in order) of    */
/* each block's sequential sum, with or without a plan.                     */
size_t pycbf_gb_tabbed_plan_bytes(long long np, int ntx, int nrx);
int pycbf_gb_tabbed_plan(const pycbf_gb_rfinfo *rf, const float *tautx, const float *apodtx,
                         const float *taurx, const float *apodrx, long long np, int interp,
                         float thresh, void *plan, size_t plan_bytes, void *stream);

/* The cubic Tabbed delay-and-sum on coefficients already produced by      */
/* pycbf_gb_spline_coefficients (prefilter once, beamform with several     */
/* table sets or sum types).  Same arguments as pycbf_gb_das_tabbed with   */
/* interp = cubic; coef must be 16-byte aligned.                           */
int pycbf_gb_das_tabbed_prefiltered(const pycbf_gb_rfinfo *rf, const void *coef,
                                    const float *tautx, const float *apodtx, const float *taurx,
                                    const float *apodrx, long long np, const int *pixel_index,
                                    float thresh, int sumtype, const void *plan, float *out,
                                    void *stream);

/* ---------------------------------------------------------------------- */
/* Cubic upsampling for nearest-neighbour interpolation with usf > 1.      */
/* Replaces the upsampling inside beamform_nearest (pycbf/cpu/pycbf.c:     */
/* 223-253): out (nframes, ntx, nrx, usf*(nt-1)+1) float32, sample it the  */
/* natural cubic spline of the channel at t0 + it*fl(dt/usf) (0 outside    */
/* [t0, t0 + dt*(nt-1)]).  workspace: pycbf_gb_workspace_bytes(rf, CUBIC)  */
/* bytes for the spline coefficients; out: pycbf_gb_upsampled_bytes.      */
/* Beamform the result with interp = nearest and an rfinfo whose nt is     */
/* usf*(nt-1)+1, dt is the float32 quotient dt/usf and dtype is F32; the   */
/* taps are then those of beamform_nearest with that usf.                  */
/* ---------------------------------------------------------------------- */
size_t pycbf_gb_upsampled_bytes(const pycbf_gb_rfinfo *rf, int usf);
int pycbf_gb_upsample(const pycbf_gb_rfinfo *rf, const void *rfdata, int usf, void *workspace,
                      size_t workspace_bytes, float *out, size_t out_bytes, void *stream);

/* ---------------------------------------------------------------------- */
/* The interpolators the reference has only on the GPU: korder cubic (the  */
/* default of pycbf.gpu, k-point derivative estimate with the k x k matrix */
/* S of gpu/__core_bf_classes__.py:366-395), akima and makima              */
/* (__engines__.cu:58-355).  A prefilter turns every interval of every     */
/* channel into the float32 coefficients of its cubic (float32 records     */
/* whatever the storage type); the delay-and-sum then gathers one record   */
/* per tap like the cubic spline path.                                     */
/*   pycbf_gb_poly_coefficients: interp KORDER (k even, 0..128, k <= nt;   */
/*     S: host float32 k*k row-major; k = 0 gives zero derivatives, what   */
/*     the reference's Synthetic korder kernel computes, its k arriving as */
/*     0), AKIMA or MAKIMA (nt >= 5; k, S ignored).  coef: 16-byte aligned,*/
/*     pycbf_gb_poly_workspace_bytes bytes.                                */
/*   pycbf_gb_das_tabbed_poly / _synthetic_poly: as pycbf_gb_das_tabbed /  */
/*     _synthetic without plan and workspace, on those coefficients.       */
/* Range rules of the reference's kernels: korder fills outside            */
/* [t0, t0 + dt*(nt-1)] (that bound one fused multiply-add, as NVRTC       */
/* compiles it); akima/makima return y[nt-1] at the last knot.  A tap      */
/* contributes when |apodtx*apodrx| >= thresh and it is in range.          */
/* ---------------------------------------------------------------------- */
size_t pycbf_gb_poly_workspace_bytes(const pycbf_gb_rfinfo *rf, int interp, int k);
int pycbf_gb_poly_coefficients(const pycbf_gb_rfinfo *rf, const void *rfdata, int interp, int k,
                               const float *S, void *coef, size_t coef_bytes, void *stream);
int pycbf_gb_das_tabbed_poly(const pycbf_gb_rfinfo *rf, const void *coef, int interp,
                             const float *tautx, const float *apodtx, const float *taurx,
                             const float *apodrx, long long np, const int *pixel_index,
                             float thresh, int sumtype, float *out, void *stream);
int pycbf_gb_das_synthetic_poly(const pycbf_gb_rfinfo *rf, const void *coef, int interp,
                                const pycbf_gb_synthetic *geo, const int *pixel_index,
                                int sumtype, float *out, void *stream);

/* ---------------------------------------------------------------------- */
/* Delay tables and apodizations of a linear array on a pixel grid, built  */
/* on the GPU.  Replaces make_tabs_and_apods_2D                            */
/* (pycbf/helpers/__full_aperture_2D__.py:170-203) and the table functions */
/* it calls (:3-168), whose float64 NumPy result the reference classes     */
/* cast to float32.  Pixels: meshgrid(xout, zout, indexing='ij')           */
/* flattened (z fastest), np = nx*nz.  txkind 0 plane wave, 1 diverging,   */
/* 2 focused; tx_params (host, ntx <= 256 rows of 6 doubles), computed as  */
/* those functions compute them:                                           */
/*   plane wave  (ox, oz, sin s', cos s', -, -): origin, steering after    */
/*               the speed-of-sound correction s' = asin(cm sin s / ctx)   */
/*   diverging   (ox, oz, -, -, tau0, -): source and its reference delay   */
/*   focused     (ox, oz, nx, nz, t0tx, alatx): the synthetic-point fields */
/* xele (nele), xout (nx), zout (nz): device float64.  Outputs (device     */
/* float32): tautx, apodtx (ntx, np); taurx, apodrx (nele, np).  Every     */
/* value is computed in float64 in NumPy's order of operations, without    */
/* fused multiply-adds, then rounded to float32.  hann = 1 weights the     */
/* receive F-number mask by cos^2(pi/2 dx/a), a = z/(2 fnum) (an           */
/* extension; 0 gives the reference's 0/1 mask).                           */
/* ---------------------------------------------------------------------- */
int pycbf_gb_tables_2d(int txkind, int ntx, const double *tx_params, int nele,
                       const double *xele, int nx, const double *xout, int nz,
                       const double *zout, double cm, double fnum, int hann, float *tautx,
                       float *apodtx, float *taurx, float *apodrx, void *stream);

/* Failure-path test hook (no counterpart in the reference): the cubic     */
/* staged delay-and-sum of pycbf_gb_das_tabbed_prefiltered (sum over tx    */
/* and rx) with the first receive of every tile announcing its bytes      */
/* without issuing its copies, so that receive's mbarrier wait runs out    */
/* (nothing is in flight for it) after                                     */
/* wait_cycles SM cycles (1e3 .. 2^31).  Each CTA that gives up writes NaN */
/* to its pixels, drains its copies (bounded), sets the plan's status word */
/* (int32 word 0 of the plan, sticky until the caller clears it) and       */
/* returns; the context stays usable.  No fault, trap or unbounded wait is */
/* involved.  Requires a plan; PYCBF_GB_EUNSUPPORTED if the staged kernel  */
/* does not apply.                                                         */
int pycbf_gb_das_tabbed_stall_test(const pycbf_gb_rfinfo *rf, const void *coef,
                                   const float *tautx, const float *apodtx, const float *taurx,
                                   const float *apodrx, long long np, const int *pixel_index,
                                   float thresh, const void *plan, float *out,
                                   long long wait_cycles, void *stream);

/* ---------------------------------------------------------------------- */
/* Synthetic-point delay-and-sum: delays and masks computed per pixel on   */
/* the fly.  Replaces das_bmode_synthetic_korder_cubic /                   */
/* das_bmode_synthetic_multi_interp (pycbf/gpu/__engines__.cu:506-694,     */
/* launched by gpu/__core_bf_classes__.py:167-243) and their delay         */
/* functions calc_tautx_apodtx / calc_taurx_apodrx (:382-470).  A tap      */
/* contributes when both masks are on (|apodtx*apodrx| > 0.01, :564) and   */
/* the delay is in range.                                                  */
/* ---------------------------------------------------------------------- */
int pycbf_gb_das_synthetic(const pycbf_gb_rfinfo *rf, const void *rfdata,
                           const pycbf_gb_synthetic *geo, const int *pixel_index, int interp,
                           int sumtype, float *out, void *workspace, size_t workspace_bytes,
                           void *stream);

/* ---------------------------------------------------------------------- */
/* Tap census (test and debug aid): per table column, the number of        */
/* contributing (tx, rx) taps and the sum of their sample indices (knot j  */
/* for cubic/linear, nearest sample for nearest).  Frame 0 only.           */
/* count: int32[np], index_sum: int64[np], both overwritten.               */
/* ---------------------------------------------------------------------- */
int pycbf_gb_tap_census_tabbed(const pycbf_gb_rfinfo *rf, const float *tautx,
                               const float *apodtx, const float *taurx, const float *apodrx,
                               long long np, int interp, float thresh, int *count,
                               long long *index_sum, void *stream);
int pycbf_gb_tap_census_synthetic(const pycbf_gb_rfinfo *rf, const pycbf_gb_synthetic *geo,
                                  int interp, int *count, long long *index_sum, void *stream);

/* Receive masks of a synthetic geometry, the apodrx of calc_taurx_apodrx  */
/* (pycbf/gpu/__engines__.cu:444-470): mask (nrx, np) uint8, 1 = accepted. */
/* Used to select SLSC elements for Synthetic beamformers.                 */
int pycbf_gb_synthetic_rx_mask(const pycbf_gb_rfinfo *rf, const pycbf_gb_synthetic *geo,
                               unsigned char *mask, void *stream);

/* ---------------------------------------------------------------------- */
/* DMAS over separated images.  Replaces calc_dmas                         */
/* (pycbf/gpu/__advanced_engines__.cu:17-61, launched by                   */
/* gpu/__advanced_bf_classes__.py:30-67).  imsep: (nframes, nsep, np);     */
/* lags: device int32[nlag], the lag values (the reference kernel uses the */
/* lag's position 0..nlag-1 instead; both agree when lags = 0..nlag-1).    */
/* dmastype 0 = signed square root, 1 = power.  out: (nframes, np) if      */
/* sumlags else (nframes, nlag, np); written, not accumulated.             */
/* ---------------------------------------------------------------------- */
int pycbf_gb_dmas(const float *imsep, long long nframes, long long nsep, long long np,
                  const int *lags, int nlag, int dmastype, int sumlags, float *out,
                  void *stream);

/* ---------------------------------------------------------------------- */
/* Short-lag spatial coherence.  The reference has it only as notebook     */
/* NumPy (examples/advanced_beamforming.ipynb, calc_lagn_coherence in      */
/* cell 2, pixel loop in cell 6).  im: (nframes, nrx, nx, nz) tx-summed    */
/* per-element images (z fastest); mask: (nrx, nx, nz) uint8 receive mask. */
/* For pixel (ix, iz) the axial kernel is rows [iz-nkern, iz+nkern]        */
/* clipped to the grid; elements whose mask is on for all of it are kept;  */
/* fewer than nlag+1 kept gives 0; otherwise the mean over lags 1..nlag of */
/* the nan-mean over kept element pairs of the normalised axial            */
/* correlation (NaN when a lag has no pair with both deviations >= 1e-10). */
/* out: (nframes, nx, nz) float32, written.                                */
/* ---------------------------------------------------------------------- */
int pycbf_gb_slsc(const float *im, const unsigned char *mask, long long nframes, int nrx, int nx,
                  int nz, int nlag, int nkern, float *out, void *stream);

/* ---------------------------------------------------------------------- */
/* The same coherence with the kept-element sets computed once per mask    */
/* (no counterpart in the reference, whose notebook loop re-derives them   */
/* per pixel).  pycbf_gb_slsc_kept writes, for the axial kernel half-width */
/* nkern, bit e % 32 of word e / 32 of each pixel (word q of pixel p at    */
/* kept[q * nx * nz + p]) when element e's mask is on over the pixel's     */
/* whole kernel; kept_bytes >= pycbf_gb_slsc_kept_bytes(nrx, nx, nz).      */
/* pycbf_gb_slsc_with_kept then gives pycbf_gb_slsc's output bit for bit   */
/* for the same nkern.  Both need nlag <= 16, nkern <= 3 and nrx <= 256    */
/* (PYCBF_GB_ERANGE otherwise: use pycbf_gb_slsc).                          */
/* ---------------------------------------------------------------------- */
size_t pycbf_gb_slsc_kept_bytes(int nrx, int nx, int nz);
int pycbf_gb_slsc_kept(const unsigned char *mask, int nrx, int nx, int nz, int nlag, int nkern,
                       unsigned *kept, size_t kept_bytes, void *stream);
int pycbf_gb_slsc_with_kept(const float *im, const unsigned *kept, long long nframes, int nrx,
                            int nx, int nz, int nlag, int nkern, float *out, void *stream);

/* ---------------------------------------------------------------------- */
/* Cubic Tabbed delay-and-sum that allocates nothing (no counterpart in    */
/* the reference).  For callers that cannot call cudaMalloc -- a language  */
/* runtime reaching CUDA only through this C ABI, a service whose device   */
/* memory is fixed at start-up, code that must not trigger the implicit    */
/* synchronisation of an allocation -- and so cannot provide the workspace */
/* pycbf_gb_das_tabbed needs for cubic interpolation.  The spline          */
/* coefficients live in a device array of PYCBF_GB_NOALLOC_SCRATCH_BYTES   */
/* inside this library, held by every GPU that loads it until the process */
/* exits.  Channel data whose coefficients                                 */
/* (pycbf_gb_workspace_bytes(rf, PYCBF_GB_INTERP_CUBIC)) exceed it are      */
/* rejected with PYCBF_GB_ERANGE; every check runs before any work is      */
/* queued.  The first call on a device looks up the array's address on     */
/* that device and keeps it (valid until a cudaDeviceReset); make it       */
/* before any stream capture.                                              */
/* All calls share the array: calls whose work overlaps on the GPU (other  */
/* streams, other host threads) race on it.  Other arguments and results   */
/* are those of pycbf_gb_das_tabbed with interp = cubic and no plan.       */
/* ---------------------------------------------------------------------- */
#define PYCBF_GB_NOALLOC_SCRATCH_BYTES (64u << 20)
int pycbf_gb_das_tabbed_cubic_noalloc(const pycbf_gb_rfinfo *rf, const void *rfdata,
                                      const float *tautx, const float *apodtx,
                                      const float *taurx, const float *apodrx, long long np,
                                      const int *pixel_index, float thresh, int sumtype,
                                      float *out, void *stream);

/* ---------------------------------------------------------------------- */
/* Differentiable cubic delay-and-sum (no counterpart in the reference,   */
/* whose beamformers are forward-only).  Inputs are spline coefficients    */
/* from pycbf_gb_spline_coefficients; sumtype is PYCBF_GB_SUM_TX_AND_RX    */
/* (gradient and image (nframes, np)) or PYCBF_GB_SUM_TX_ONLY ((nframes,   */
/* nrx, np)); ntx <= 128.                                                  */
/*                                                                        */
/* The Synthetic form replaces 1/c0 by a slowness per pixel s[i] (s/m, in  */
/* table-column order): every delay is its path length times s[i] (plus    */
/* t0tx for the focused transmits), with the masks of                      */
/* pycbf_gb_das_synthetic.  geo->c0 is not used.                           */
/*                                                                        */
/* The adjoints take the upstream gradient grad_out (shaped like the       */
/* image, indexed through pixel_index like it) and write, each only when   */
/* its pointer is not NULL:                                                */
/*   grad_rf     (nframes, ntx, nrx, nt) float32 whatever the storage      */
/*   grad_tautx  (ntx, np), grad_taurx (nrx, np): Tabbed, summed over      */
/*               frames, table-column order                                */
/*   grad_slow   (np): Synthetic, summed over frames                       */
/* All outputs are overwritten; every sum has a fixed order, so results    */
/* are bitwise reproducible.  Apodization is not differentiated.           */
/* workspace: pycbf_gb_adjoint_workspace_bytes bytes, 16-byte aligned;     */
/* it may be NULL only when grad_rf and pixel_index are both NULL.         */
/* ---------------------------------------------------------------------- */
int pycbf_gb_das_synthetic_slowness(const pycbf_gb_rfinfo *rf, const void *coef,
                                    const pycbf_gb_synthetic *geo, const float *slowness,
                                    const int *pixel_index, int sumtype, float *out,
                                    void *stream);
size_t pycbf_gb_adjoint_workspace_bytes(const pycbf_gb_rfinfo *rf, long long np);
int pycbf_gb_das_tabbed_adjoint(const pycbf_gb_rfinfo *rf, const void *coef,
                                const float *tautx, const float *apodtx, const float *taurx,
                                const float *apodrx, long long np, const int *pixel_index,
                                float thresh, int sumtype, const float *grad_out,
                                float *grad_rf, float *grad_tautx, float *grad_taurx,
                                void *workspace, size_t workspace_bytes, void *stream);
/* The same with the forward's staging plan (pycbf_gb_tabbed_plan of these   */
/* tables, or NULL): where the plan's staged path applies (cubic, float32   */
/* channel data, one frame, ntx <= 12), the delay gradients gather the      */
/* records from its staged windows.  The plan's queue head is reused, so it */
/* must not be in use by another call at the same time.  No counterpart in  */
/* the reference, whose beamformers are forward-only.                       */
int pycbf_gb_das_tabbed_adjoint_planned(const pycbf_gb_rfinfo *rf, const void *coef,
                                        const float *tautx, const float *apodtx,
                                        const float *taurx, const float *apodrx, long long np,
                                        const int *pixel_index, float thresh, int sumtype,
                                        const void *plan, const float *grad_out, float *grad_rf,
                                        float *grad_tautx, float *grad_taurx, void *workspace,
                                        size_t workspace_bytes, void *stream);
int pycbf_gb_das_synthetic_adjoint(const pycbf_gb_rfinfo *rf, const void *coef,
                                   const pycbf_gb_synthetic *geo, const float *slowness,
                                   const int *pixel_index, int sumtype, const float *grad_out,
                                   float *grad_rf, float *grad_slow, void *workspace,
                                   size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------- */
/* Uneven batches (no counterpart in the reference): many frames of        */
/* Tabbed and Synthetic beamformers of any size and storage type,          */
/* prefiltered and beamformed (cubic, summed over transmits and receives)  */
/* by two launches -- one batched prefilter, one persistent delay-and-sum  */
/* that takes (frame, pixel tile) work items from a queue -- so the whole  */
/* batch can be captured in one CUDA graph.                                */
/*                                                                        */
/* Each job is one frame: rf.nframes = 1, rfdata (ntx, nrx, nt) stored as  */
/* float32, float16 or bfloat16 (PYCBF_GB_I16: PYCBF_GB_EUNSUPPORTED); coef its */
/* own pycbf_gb_workspace_bytes(&rf, PYCBF_GB_INTERP_CUBIC) bytes          */
/* (16-byte aligned); out (np) float32.  Tabbed jobs give the tables, np   */
/* and thresh (geo NULL); Synthetic jobs give geo (np from geo->np; delays */
/* and masks of pycbf_gb_das_synthetic).  Several jobs may share tables,   */
/* geometry or pixel_index.                                                */
/*                                                                        */
/* pycbf_gb_batch_plan validates every job and writes, into the caller's   */
/* device buffer plan (pycbf_gb_batch_plan_bytes, 16-byte aligned), the    */
/* job descriptors and the work items: runs of tiles_per_item (1..8) tiles */
/* of 128 pixels, in job order (order 0) or largest estimated cost first   */
/* (order 1).  It fills *info, which pycbf_gb_batch_run needs.             */
/* pycbf_gb_batch_run queues the prefilter and the delay-and-sum on the   */
/* stream: tx_chunk (4, 8 or 12) transmits are held in registers at a      */
/* time, or (tx_chunk 0) each pixel runs the single-frame kernel's own     */
/* body (transmits in registers up to 12, in shared memory beyond:         */
/* info->max_ntx sizes it); ctas CTAs of 128 threads serve the queue.      */
/* With tx_chunk 0, or ntx <= tx_chunk, a job's image is bitwise the one   */
/* pycbf_gb_das_tabbed / pycbf_gb_das_synthetic give for its frame.  run   */
/* allocates nothing and                                                   */
/* makes no host-blocking call, so it can be captured in a CUDA graph once */
/* plan has run; rerunning it (or the graph) reuses the plan's buffers.    */
/* ---------------------------------------------------------------------- */
typedef struct pycbf_gb_batch_job {
    int geom;                       /* 0 Tabbed, 1 Synthetic                          */
    pycbf_gb_rfinfo rf;
    const void *rfdata;
    void *coef;
    const float *tautx, *apodtx, *taurx, *apodrx;   /* Tabbed                      */
    long long np;                   /* Tabbed                                         */
    float thresh;                   /* Tabbed                                         */
    const pycbf_gb_synthetic *geo;  /* Synthetic (host pointer, copied by plan)       */
    const int *pixel_index;
    float *out;
} pycbf_gb_batch_job;

typedef struct pycbf_gb_batch_info {
    long long nitems;
    long long nchannels;
    int njobs;
    int max_nt;
    int tiles_per_item;
    int max_ntx;
    int dtypes;                     /* bit 1 << dtype for every storage type present  */
} pycbf_gb_batch_info;

size_t pycbf_gb_batch_plan_bytes(const pycbf_gb_batch_job *jobs, int njobs, int tiles_per_item);
int pycbf_gb_batch_plan(const pycbf_gb_batch_job *jobs, int njobs, int tiles_per_item, int order,
                        void *plan, size_t plan_bytes, pycbf_gb_batch_info *info, void *stream);
int pycbf_gb_batch_run(const void *plan, const pycbf_gb_batch_info *info, int tx_chunk, int ctas,
                       void *stream);

/* ---------------------------------------------------------------------- */
/* Measurement utility (no counterpart in the reference): blocks x 256    */
/* threads each run iters rounds of 8 independent float32 FMAs and store  */
/* one float to out[blocks*256].  FLOPs = blocks*256*iters*16.  Gives the */
/* FP32 peak that the benchmark's FP32 roofline fraction divides by.      */
/* ---------------------------------------------------------------------- */
int pycbf_gb_fp32_probe(float *out, int blocks, int iters, void *stream);

/* int16 -> float32 on the device (n samples, exact): the conversion the  */
/* PYCBF_GB_I16 paths fuse, for the entry points that take float data.    */
int pycbf_gb_convert_i16(const short *src, long long n, float *dst, void *stream);

/* ---------------------------------------------------------------------- */
/* IQ demodulation, envelope and log compression of beamformed images (the */
/* step after the path).  Replaces the examples' fft_tukey_demod           */
/* (examples/SyntheticPointBeamforming.ipynb cell 1; the same function in  */
/* SyntheticVsTabbed.ipynb cell 1, develop_dmas_class.ipynb cell 7), a     */
/* CuPy rfft -> band slice -> Tukey window -> ifftshift -> ifft chain, and */
/* their display line 20*log10(env/np.percentile(env, 99) + 1e-10)         */
/* (SyntheticPointBeamforming.ipynb cell 11).                              */
/*                                                                         */
/* pycbf_gb_demod: iq[c][m] = sum_k x[c][k] * W[k][m] for ncols lines of n */
/* samples (x row-major, device float32); W (n, M) complex, interleaved    */
/* float32 pairs, the whole FFT chain as one matrix (pycbf_gb300.demod     */
/* builds it).  iq (ncols, M) complex interleaved and/or env (ncols, M)    */
/* = |iq|; either may be NULL, not both.                                   */
/*                                                                         */
/* pycbf_gb_percentile: out[s] = NumPy's percentile (method 'linear') of   */
/* segment s of v (nseg segments of n contiguous floats), q in [0, 100];   */
/* NaN in a segment gives NaN.  The two order statistics are selected      */
/* exactly.  Workspace: pycbf_gb_percentile_workspace_bytes(nseg) device   */
/* bytes.  out is device memory.                                            */
/*                                                                         */
/* pycbf_gb_log_compress: out[s*n + i] = 20 log10(env[s*n + i] / ref[s] +  */
/* floor_add), ref in device memory (the percentile's output).  out may    */
/* alias env.                                                              */
/*                                                                         */
/* pycbf_gb_log_compress_percentile: both -- ref[s] = the q-th percentile  */
/* of segment s, out its log compression -- in one launch for segments of */
/* up to 425,984 values (a cluster of 8 CTAs per segment holds it in       */
/* shared memory).  Workspace as for pycbf_gb_percentile; out may alias    */
/* env.                                                                    */
/* ---------------------------------------------------------------------- */
int pycbf_gb_demod(const float *x, long long ncols, int n, const float *W, int M, float *iq,
                   float *env, void *stream);
size_t pycbf_gb_percentile_workspace_bytes(long long nseg);
int pycbf_gb_percentile(const float *v, long long nseg, long long n, double q, float *out,
                        void *workspace, size_t workspace_bytes, void *stream);
int pycbf_gb_log_compress(const float *env, long long nseg, long long n, const float *ref,
                          float floor_add, float *out, void *stream);
int pycbf_gb_log_compress_percentile(const float *env, long long nseg, long long n, double q,
                                     float floor_add, float *out, float *ref, void *workspace,
                                     size_t workspace_bytes, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PYCBF_GB300_H */

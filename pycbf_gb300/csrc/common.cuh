// Shared device helpers and the launch interface between the kernel files and
// the C ABI (abi.cu).  Internal to libpycbf_gb300.so.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "pycbf_gb300.h"

namespace pgb {

// ---------------------------------------------------------------------------
// storage types
// ---------------------------------------------------------------------------
__device__ __forceinline__ float load_sample(const float *p) { return __ldg(p); }
__device__ __forceinline__ float load_sample(const __half *p) { return __half2float(__ldg(p)); }
__device__ __forceinline__ float load_sample(const __nv_bfloat16 *p) {
    return __bfloat162float(__ldg(p));
}

__device__ __forceinline__ float load_sample_reg(float v) { return v; }
__device__ __forceinline__ float load_sample_reg(__half v) { return __half2float(v); }
__device__ __forceinline__ float load_sample_reg(__nv_bfloat16 v) { return __bfloat162float(v); }
// int16 channel data (raw converter counts): exact in float32
__device__ __forceinline__ float load_sample(const short *p) { return (float)__ldg(p); }
__device__ __forceinline__ float load_sample_reg(short v) { return (float)v; }

// A spline coefficient record of interval j of a channel.
//
// float32 (and int16) channel data: the interval's cubic as a polynomial in
// the fraction b = (x - xlo_j) / dt, v(b) = p0 + p1 b + p2 b^2 + p3 b^3, one
// float4.  It equals the reference's evaluation (pycbf.c:93-98)
//   a y_j + b y_j+1 + (a^3 - a) z_j + (b^3 - b) z_j+1,  a = (xhi_j - x) / dt
// rewritten with a = c_j - b, c_j = (xhi_j - xlo_j) / dt, where xlo_j =
// fl(t0 + fl(dt j)) and xhi_j = fl(t0 + fl(dt (j+1))) are the knots as the
// reference rounds them (c_j differs from 1 by up to ~ulp(x)/dt):
//   p0 = c y_j + (c^3 - c) z_j        p1 = y_j+1 - y_j + (1 - 3c^2) z_j - z_j+1
//   p2 = 3c z_j                       p3 = z_j+1 - z_j
// so a tap needs only b (from x and xlo_j) and three multiply-adds.
// 16-bit channel data: (y_j, y_j+1, z_j, z_j+1) packed in a uint2 (the
// polynomial's coefficients would lose more to 16-bit rounding).
template <typename T> struct CoefRec;
template <> struct CoefRec<float> {
    using raw = float4;
    static constexpr bool kPoly = true;
    static __device__ __forceinline__ float4 load(const raw *p) { return __ldg(p); }
    static __device__ __forceinline__ float4 unpack(const raw &r) { return r; }
    // the record of interval j from the samples and second-derivative terms
    static __device__ __forceinline__ raw make(float y0, float y1, float z0, float z1, int j,
                                               float t0, float dt) {
        const float xlo = __fadd_rn(t0, __fmul_rn(dt, (float)j));
        const float xhi = __fadd_rn(t0, __fmul_rn(dt, (float)(j + 1)));
        const float c = __fdiv_rn(__fsub_rn(xhi, xlo), dt);
        const float c2 = c * c;
        return make_float4(fmaf(c2 * c - c, z0, c * y0), fmaf(1.f - 3.f * c2, z0, y1 - y0) - z1,
                           3.f * c * z0, z1 - z0);
    }
};
// int16 channels are prefiltered into float32 records
template <> struct CoefRec<short> : CoefRec<float> {};
template <> struct CoefRec<__half> {
    using raw = uint2;
    static constexpr bool kPoly = false;
    static __device__ __forceinline__ raw make(float y0, float y1, float z0, float z1, int, float,
                                               float) {
        return pack(y0, y1, z0, z1);
    }
    static __device__ __forceinline__ float4 load(const raw *p) { return unpack(__ldg(p)); }
    static __device__ __forceinline__ float4 unpack(raw r) {
        __half2 h0 = *reinterpret_cast<__half2 *>(&r.x);
        __half2 h1 = *reinterpret_cast<__half2 *>(&r.y);
        float2 a = __half22float2(h0), b = __half22float2(h1);
        return make_float4(a.x, a.y, b.x, b.y);
    }
    static __device__ __forceinline__ raw pack(float a, float b, float c, float d) {
        __half2 h0 = __floats2half2_rn(a, b), h1 = __floats2half2_rn(c, d);
        uint2 r;
        r.x = *reinterpret_cast<unsigned *>(&h0);
        r.y = *reinterpret_cast<unsigned *>(&h1);
        return r;
    }
};
template <> struct CoefRec<__nv_bfloat16> {
    using raw = uint2;
    static constexpr bool kPoly = false;
    static __device__ __forceinline__ raw make(float y0, float y1, float z0, float z1, int, float,
                                               float) {
        return pack(y0, y1, z0, z1);
    }
    static __device__ __forceinline__ float4 load(const raw *p) { return unpack(__ldg(p)); }
    static __device__ __forceinline__ float4 unpack(raw r) {
        __nv_bfloat162 h0 = *reinterpret_cast<__nv_bfloat162 *>(&r.x);
        __nv_bfloat162 h1 = *reinterpret_cast<__nv_bfloat162 *>(&r.y);
        float2 a = __bfloat1622float2(h0), b = __bfloat1622float2(h1);
        return make_float4(a.x, a.y, b.x, b.y);
    }
    static __device__ __forceinline__ raw pack(float a, float b, float c, float d) {
        __nv_bfloat162 h0 = __floats2bfloat162_rn(a, b), h1 = __floats2bfloat162_rn(c, d);
        uint2 r;
        r.x = *reinterpret_cast<unsigned *>(&h0);
        r.y = *reinterpret_cast<unsigned *>(&h1);
        return r;
    }
};

// ---------------------------------------------------------------------------
// packed float32 pairs (sm_100+ f32x2 arithmetic, one instruction for two
// lanes, each rounded to nearest as the scalar operation).  A packed multiply
// whose result feeds a packed add was observed to come out with one rounding,
// as a fused multiply-add -- with the float2 intrinsics and with this PTX
// alike -- so code here never feeds a packed product into a packed add; a
// product that must be rounded on its own is formed with __fmul_rn.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long pack2(float2 v) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}
__device__ __forceinline__ float2 unpack2(unsigned long long r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}
__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}
__device__ __forceinline__ float2 fma2_rn(float2 a, float2 b, float2 c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)), "l"(pack2(c)));
    return unpack2(r);
}

// ---------------------------------------------------------------------------
// spline prefilter
// ---------------------------------------------------------------------------
// The forward sweep of the natural-spline tridiagonal solve (pycbf.c:126-133)
// has data-independent pivots p_i = 0.5*y2f_{i-1} + 2; they converge to
// 2 - (2 - sqrt 3)/2 within ~10 steps.  The host tabulates 1/p_i and the
// back-substitution factors c_i = y2f_i = -0.5/p_i for i < kSplineTab; larger
// i use the last entry.
constexpr int kSplineTab = 64;
struct SplineTable {
    float invp[kSplineTab];
    float c[kSplineTab];
};
void make_spline_table(SplineTable *t);

struct SplineArgs {
    const void *rf;          // (nch, nt) storage type
    void *coef;              // (nch, nt) coefficient records
    long long nch;
    int nt;
    float t0, dt;            // the time axis (the float32 records depend on the knots)
};
cudaError_t launch_spline(const SplineArgs &a, int dtype, cudaStream_t s);

// ---------------------------------------------------------------------------
// delay-and-sum
// ---------------------------------------------------------------------------
// pixels (threads) per CTA of the delay-and-sum kernels: one table column each
constexpr int kBlock = 128;

// GEOM_SYNTH_SLOW: synthetic geometry whose delays are path length x a
// per-pixel slowness (the differentiable form) instead of path length / c0
enum Geom { GEOM_TABBED = 0, GEOM_SYNTH = 1, GEOM_SYNTH_SLOW = 2 };

struct DasArgs {
    // channel data (or spline coefficients for cubic), (nframes, ntx, nrx, nt)
    const void *data;
    // Tabbed tables (device, float32)
    const float *tautx, *apodtx, *taurx, *apodrx;
    // Synthetic geometry (device, float32)
    pycbf_gb_synthetic geo;
    const int *pixel_index;
    float *out;
    int *census_count;
    long long *census_isum;
    long long np;
    int ntx, nrx, nt, ndim, nframes;
    float t0, dt, inv_dt, xmax, xend, thresh, eps;
    // the staged cubic taps' floor test: 1.25 x the largest gap 1.5 |q| 2^-23
    // between the reciprocal quotient and the IEEE quotient for |q| < nt
    float eps_fast;
    const float *slow;  // GEOM_SYNTH_SLOW: slowness per pixel (s/m), kernel pixel order
    float xfma;         // fma(dt, nt-1, t0): the last knot as the reference's CUDA kernels round it
    // staged kernel: SM cycles after which an mbarrier wait gives up (0: 2^31,
    // about a second); stall_test: the first receive of every tile announces
    // its bytes and issues no copy, so its wait runs out (the failure path,
    // exercised without a fault)
    long long wait_cycles;
    int stall_test;
    // staged delay gradients: the upstream gradient (kernel pixel order) and
    // dL/dtautx (ntx, np), dL/dtaurx (nrx, np), either may be null
    const float *gk;
    float *gtx, *grx;
};

// gather kinds of the polynomial-record interpolators (records from poly.cu)
constexpr int KIND_POLY_NORM = 4;   // korder: a0 + a1 u + a2 u^2 + a3 u^3, u in [0, 1)
constexpr int KIND_POLY_DELTA = 5;  // akima / makima: a + b d + c d^2 + d d^3, d in seconds
cudaError_t launch_poly_records(const DasArgs &a, const void *rf, int dtype, int interp, int k,
                                const float *S, float4 *rec, long long nch, cudaStream_t s);
cudaError_t launch_das(const DasArgs &a, int geom, int interp, int sumtype, int dtype, bool census,
                       cudaStream_t s);
cudaError_t launch_synth_rx_mask(const DasArgs &a, unsigned char *mask, cudaStream_t s);
// TMA-staged Tabbed path (ntx <= 12; sums over transmits per receive)
long long tabbed_plan_words(long long np, int ntx, int nrx);
cudaError_t launch_tabbed_plan(const DasArgs &a, int interp, int dtype, int *plan, cudaStream_t s);
cudaError_t launch_das_staged(const DasArgs &a, int interp, int sumtype, int dtype, const int *plan,
                              int *status, cudaStream_t s);
// the delay gradients on the staging plan (cubic, float32 records, one frame)
cudaError_t launch_das_staged_adj(const DasArgs &a, int sumtype, int dtype, const int *plan,
                                  cudaStream_t s);

// cubic upsampling for nearest with usf > 1: out (nch, ntu) float32 from the
// spline records in a.data (time axis of the original channel data in a)
cudaError_t launch_upsample(const DasArgs &a, int dtype, float *out, long long nch, int ntu,
                            float dtu, cudaStream_t s);

// ---------------------------------------------------------------------------
// delay tables of a linear array on a grid (tables.cu)
// ---------------------------------------------------------------------------
constexpr int kTables2DMaxTx = 256;
struct Tables2D {
    int txkind;                      // 0 plane wave, 1 diverging, 2 focused
    int ntx, nele, nx, nz, hann;
    double cm, fnum2;                // speed of sound, 2 * f-number
    double tx[kTables2DMaxTx][6];    // per transmit: ox, oz, nx, nz, t0 (tau0 / t0tx), ala
};
cudaError_t launch_tables_2d(const Tables2D &p, const double *xele, const double *xout,
                             const double *zout, float *tautx, float *apodtx, float *taurx,
                             float *apodrx, cudaStream_t s);

// ---------------------------------------------------------------------------
// uneven batches: one frame of one beamformer per job, all in one launch
// ---------------------------------------------------------------------------
struct BatchJob {
    DasArgs a;            // a.data: this frame's coefficient records; a.out: its image (np)
    const void *rf;       // this frame's channel data (ntx, nrx, nt), storage type
    long long ch0;        // first channel of this job in the batch's channel numbering
    int geom;             // GEOM_TABBED or GEOM_SYNTH
    int dtype;            // storage type
};
cudaError_t launch_batch_spline(const BatchJob *jobs, int njobs, long long nch_total, int max_nt,
                                cudaStream_t s, bool set_attr);
// items: (job, first tile / tiles_per_item) pairs in processing order; counter:
// the work-queue head (zero before the launch)
// tx_chunk 0: the single-frame kernel's per-pixel body (dynamic shared memory for
// max_ntx transmits, its limit set by prepare_batch_das outside any capture);
// dtypes: bit 1 << dtype of each storage type in the batch (one type: a kernel
// with that type's paths only)
cudaError_t launch_batch_das(const BatchJob *jobs, const int2 *items, long long nitems,
                             int tiles_per_item, unsigned long long *counter, int tx_chunk,
                             int ctas, cudaStream_t s, int max_ntx, int dtypes);
cudaError_t prepare_batch_das(int max_ntx);

// ---------------------------------------------------------------------------
// adjoint (gradients of the cubic delay-and-sum; no reference counterpart)
// ---------------------------------------------------------------------------
struct AdjArgs {
    DasArgs d;            // the forward's arguments (d.data = coefficient records)
    int geom;             // GEOM_TABBED or GEOM_SYNTH_SLOW
    int sumtype;          // PYCBF_GB_SUM_TX_AND_RX or PYCBF_GB_SUM_TX_ONLY
    const float *gout;    // upstream gradient, shaped like the forward's output
    float *grad_rf;       // (nframes, ntx, nrx, nt) float32, or NULL
    float *grad_tautx;    // Tabbed (ntx, np), or NULL
    float *grad_taurx;    // Tabbed (nrx, np), or NULL
    float *grad_slow;     // Synthetic (np), or NULL
    float *gk_buf;        // workspace: grad_out gathered into kernel pixel order
    float *partial;       // workspace: per-part sums of the spline-record adjoints
    unsigned char *live;  // workspace: live[r * tiles + tile] = receive r can contribute to the tile
    const float *gk;      // set by launch_adjoint: gk_buf, or grad_out without pixel_index
    const int *plan;      // Tabbed: the forward's staging plan when its staged path applies, or NULL
};
// parts of the pixel range whose channel adjoints are summed separately, and
// the workspace: [gathered gradient (nframes * nrx * np floats, 256-byte
// rounded)][partial sums (parts * nch * 2 * Lp floats)][receive-tile liveness
// (nrx * tiles bytes, 256-byte rounded)]
int adjoint_parts(long long nch, long long np);
size_t adjoint_grad_bytes(long long nframes, long long nrx, long long np);
size_t adjoint_partial_bytes(long long nframes, long long ntx, long long nrx, long long np, int nt);
size_t adjoint_workspace_bytes(long long nframes, long long ntx, long long nrx, long long np,
                               int nt);
int adjoint_rows_warps(int nt);  // warps per scatter CTA (they share its rows), 0 = nt too large
cudaError_t launch_adjoint(const AdjArgs &a, int dtype, cudaStream_t s);
cudaError_t launch_das_synth_slow(const DasArgs &a, int sumtype, int dtype, cudaStream_t s);

// ---------------------------------------------------------------------------
// coherence
// ---------------------------------------------------------------------------
cudaError_t launch_dmas(const float *im, long long nframes, long long nsep, long long np,
                        const int *lags, int nlag, int power, int sumlags, float *out,
                        cudaStream_t s);
// kept: the per-pixel kept-element bit sets of launch_slsc_kept, or null to
// derive them from mask (which may then be null only when kept is given)
cudaError_t launch_slsc(const float *im, const unsigned char *mask, const unsigned *kept,
                        long long nframes, int nrx, int nx, int nz, int nlag, int nkern, float *out,
                        cudaStream_t s);
bool slsc_kept_supported(int nrx, int nlag, int nkern);
cudaError_t launch_slsc_kept(const unsigned char *mask, int nrx, int nx, int nz, int nkern,
                             unsigned *kept, cudaStream_t s);

// argument checks of the cubic Tabbed delay-and-sum on prefiltered records (abi.cu)
int check_tabbed_prefiltered(const pycbf_gb_rfinfo *rf, const void *coef, const float *tautx,
                             const float *apodtx, const float *taurx, const float *apodrx,
                             long long np, float thresh, int sumtype, const float *out);

// int16 channel data -> float32 (spline.cu)
cudaError_t launch_convert_i16(const short *src, long long n, float *dst, cudaStream_t s);

// ---------------------------------------------------------------------------
// demodulation, percentile, log compression (demod.cu)
// ---------------------------------------------------------------------------
// iq / env: (ncols, M) complex / float, either may be null
cudaError_t launch_demod(const float *x, long long ncols, int n, const float2 *W, int M,
                         float2 *iq, float *env, cudaStream_t s);
size_t percentile_workspace_bytes(long long nseg);
// out (nseg, device): the percentiles; logout (optional): the log compression of v with them
cudaError_t launch_percentile(const float *v, long long nseg, long long n, double q, float *out,
                              void *ws, cudaStream_t s, float floor_add = 0.f,
                              float *logout = nullptr);
cudaError_t launch_log_compress(const float *env, long long nseg, long long n, const float *ref,
                                float floor_add, float *out, cudaStream_t s);

}  // namespace pgb

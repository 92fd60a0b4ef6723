// Prefilter of the interpolators the reference has only in its CUDA file:
// every interval j of every channel becomes one float32 record of cubic
// coefficients, so that a tap gathers one 16-byte record (as for the cubic
// spline) instead of k + 2 samples (korder) or six samples and three
// divisions (akima, makima).
//
//   korder (__engines__.cu:292-355): derivative estimates yp0, yp1 at the
//     ends of interval j from a k-sample window and two rows of S
//     (gpu/__core_bf_classes__.py:366-395); record (a0, a1, a2, a3) of
//     a0 + a1 u + a2 u^2 + a3 u^3, u = (x - t0 - dt j)/dt.
//   akima / makima (:188-269 / :58-183): one-sided slopes sp0, sp1 of the
//     interval from the secants around it (the boundary cases of the
//     source, makima adding |m_a + m_b|/2 to each weight); record
//     (y_j, sp0, (3 mp0 - 2 sp0 - sp1)/dt, (sp0 + sp1 - 2 mp0)/dt^2) of a +
//     b d + c d^2 + d d^3, d = x - (t0 + dt j) in seconds, as the source
//     evaluates it.
// The last sample's record is (y_nt-1, 0, 0, 0): both kernels return
// y_nt-1 there.  Every operation is one IEEE rounding, in the order of the
// source (the S products fused, as NVRTC compiles the accumulation).
// One thread per (channel, interval); S in shared memory.
#include "das_impl.cuh"

namespace pgb {

namespace {

template <typename T>
__device__ __forceinline__ float ld(const T *y, int i) {
    return load_sample(y + i);
}

__device__ __forceinline__ float half_of(float v) { return __fdiv_rn(v, 2.0f); }

__device__ __forceinline__ float weight(float p, float q, bool makima) {
    const float w = fabsf(__fsub_rn(p, q));
    return makima ? __fadd_rn(w, half_of(fabsf(__fadd_rn(p, q)))) : w;
}

__device__ __forceinline__ float blend(float w0, float m0, float w1, float m1) {
    return __fdiv_rn(__fadd_rn(__fmul_rn(w0, m0), __fmul_rn(w1, m1)), __fadd_rn(w0, w1));
}

template <typename T>
__device__ float4 akima_record(const T *y, int nx, int ixo, float dt, bool makima) {
    float mm2, mm1, mp0, mp1, mp2, sp0, sp1;
    const float y0 = ld(y, ixo);
    if (ixo == 0) {
        mp0 = __fsub_rn(ld(y, 1), y0);
        mp1 = __fsub_rn(ld(y, 2), ld(y, 1));
        sp0 = mp0;
        sp1 = half_of(__fadd_rn(mp0, mp1));
    } else if (ixo == 1) {
        mm1 = __fsub_rn(y0, ld(y, 0));
        mp0 = __fsub_rn(ld(y, 2), y0);
        mp1 = __fsub_rn(ld(y, 3), ld(y, 2));
        mp2 = __fsub_rn(ld(y, 4), ld(y, 3));
        sp0 = half_of(__fadd_rn(mp0, mm1));
        if ((mm1 == mp0) && (mp0 == mp1) && (mp1 == mp2)) sp1 = 0.f;
        else sp1 = blend(weight(mp2, mp1, makima), mp0, weight(mp0, mm1, makima), mp1);
    } else if (ixo == nx - 3) {
        mm2 = __fsub_rn(ld(y, ixo - 1), ld(y, ixo - 2));
        mm1 = __fsub_rn(y0, ld(y, ixo - 1));
        mp0 = __fsub_rn(ld(y, ixo + 1), y0);
        mp1 = __fsub_rn(ld(y, ixo + 2), ld(y, ixo + 1));
        if ((mm2 == mm1) && (mm1 == mp0) && (mp0 == mp1)) sp0 = 0.f;
        else sp0 = blend(weight(mp1, mp0, makima), mm1, weight(mm1, mm2, makima), mp0);
        sp1 = half_of(__fadd_rn(mp0, mp1));
    } else if (ixo == nx - 2) {
        mm1 = __fsub_rn(y0, ld(y, ixo - 1));
        mp0 = __fsub_rn(ld(y, ixo + 1), y0);
        sp0 = half_of(__fadd_rn(mm1, mp0));
        sp1 = mp0;
    } else {
        mm2 = __fsub_rn(ld(y, ixo - 1), ld(y, ixo - 2));
        mm1 = __fsub_rn(y0, ld(y, ixo - 1));
        mp0 = __fsub_rn(ld(y, ixo + 1), y0);
        mp1 = __fsub_rn(ld(y, ixo + 2), ld(y, ixo + 1));
        mp2 = __fsub_rn(ld(y, ixo + 3), ld(y, ixo + 2));
        if ((mm2 == mm1) && (mm1 == mp0) && (mp0 == mp1)) sp0 = 0.f;
        else sp0 = blend(weight(mp1, mp0, makima), mm1, weight(mm1, mm2, makima), mp0);
        if ((mm1 == mp0) && (mp0 == mp1) && (mp1 == mp2)) sp1 = 0.f;
        else sp1 = blend(weight(mp2, mp1, makima), mp0, weight(mp0, mm1, makima), mp1);
    }
    const float c = __fdiv_rn(__fsub_rn(__fsub_rn(__fmul_rn(3.f, mp0), __fmul_rn(2.f, sp0)), sp1), dt);
    const float d = __fdiv_rn(__fsub_rn(__fadd_rn(sp0, sp1), __fmul_rn(2.f, mp0)), __fmul_rn(dt, dt));
    return make_float4(y0, sp0, c, d);
}

template <typename T>
__device__ float4 korder_record(const T *y, int nx, int ixin, int k, const float *S) {
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
    const float y0 = ld(y, ixin), y1 = ld(y, ixin + 1);
    float yp0 = 0.f, yp1 = 0.f;
    for (int i = 0; i < k; ++i) {
        const float v = ld(y, iy0 + i);
        yp0 = fmaf(S[ik0 * k + i], v, yp0);
        yp1 = fmaf(S[ik0 * k + k + i], v, yp1);
    }
    const float a2 = __fsub_rn(__fsub_rn(__fmul_rn(3.f, __fsub_rn(y1, y0)), __fmul_rn(2.f, yp0)), yp1);
    const float a3 = __fadd_rn(__fadd_rn(__fmul_rn(2.f, __fsub_rn(y0, y1)), yp0), yp1);
    return make_float4(y0, yp0, a2, a3);
}

template <typename T>
__global__ void __launch_bounds__(256)
poly_records_kernel(const T *__restrict__ rf, float4 *__restrict__ rec, long long nch, int nt,
                    float dt, int interp, int k, const float *__restrict__ S) {
    extern __shared__ float sS[];
    if (interp == PYCBF_GB_INTERP_KORDER) {
        for (int i = threadIdx.x; i < k * k; i += blockDim.x) sS[i] = S[i];
        __syncthreads();
    }
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nch * (long long)nt) return;
    const long long ch = n / nt;
    const int j = (int)(n - ch * nt);
    const T *y = rf + ch * (long long)nt;
    float4 r;
    if (j == nt - 1) r = make_float4(ld(y, j), 0.f, 0.f, 0.f);
    else if (interp == PYCBF_GB_INTERP_KORDER) r = korder_record(y, nt, j, k, sS);
    else r = akima_record(y, nt, j, dt, interp == PYCBF_GB_INTERP_MAKIMA);
    rec[n] = r;
}

template <typename T>
cudaError_t launch_poly_t(const DasArgs &a, const void *rf, int interp, int k, const float *S,
                          float4 *rec, long long nch, cudaStream_t s) {
    const long long total = nch * (long long)a.nt;
    const long long blocks = (total + 255) / 256;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    const size_t smem = interp == PYCBF_GB_INTERP_KORDER ? sizeof(float) * (size_t)k * k : 0;
    auto kern = poly_records_kernel<T>;
    if (smem > 48 * 1024) {
        cudaError_t err =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    kern<<<(unsigned)blocks, 256, smem, s>>>(static_cast<const T *>(rf), rec, nch, a.nt, a.dt,
                                             interp, k, S);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_poly_records(const DasArgs &a, const void *rf, int dtype, int interp, int k,
                                const float *S, float4 *rec, long long nch, cudaStream_t s) {
    switch (dtype) {
        case PYCBF_GB_F32: return launch_poly_t<float>(a, rf, interp, k, S, rec, nch, s);
        case PYCBF_GB_F16: return launch_poly_t<__half>(a, rf, interp, k, S, rec, nch, s);
        case PYCBF_GB_BF16: return launch_poly_t<__nv_bfloat16>(a, rf, interp, k, S, rec, nch, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace pgb

// Natural cubic spline coefficients for every channel, one pair of warps per
// channel.
//
// The reference builds the knots of each channel with a serial Thomas solve
// (tie_knots1D_fixed, pycbf/cpu/pycbf.c:114-166): a forward sweep
//   u_i = (6 (y_{i+1} - 2 y_i + y_{i-1}) / (2 dx^2) - 0.5 u_{i-1}) / p_i
// and a back-substitution y2_k = c_k y2_{k+1} + u_k.  Both recurrences
// contract by |0.5/p| -> 2 - sqrt(3) = 0.268 per step, so a lane can start
// either sweep kWarm = 16 samples before its chunk from zero: the start error
// has shrunk by 0.268^16 ~ 7e-10 when the chunk begins.  Each of the 64 lanes
// owns a contiguous chunk of the channel (of odd length, so that the lanes'
// sequential sweeps fall in distinct shared-memory banks; 33 samples at nt =
// 2048, so each lane's serial chain is 49 steps); the channel, u and y2 sit in
// shared memory.  Output per sample j: one record of interval j (CoefRec: the
// interval's cubic as a polynomial in the fraction for float32 records,
// (y_j, y_j+1, z_j, z_j+1) for 16-bit ones), z = y2 dx^2 / 6, with y_nt =
// z_nt = 0, so the forward kernel does one 16-byte (or 8-byte) load per tap.
#include <algorithm>

#include "common.cuh"

namespace pgb {

// warm-up of each lane's sweeps: 0.268^16 = 7e-10 of the start error is left,
// below float32 rounding
constexpr int kWarm = 16;

void make_spline_table(SplineTable *t) {
    float y2f = 0.0f;
    t->invp[0] = 0.5f;
    t->c[0] = 0.0f;
    for (int i = 1; i < kSplineTab; ++i) {
        float p = 0.5f * y2f + 2.0f;
        float y2 = (0.5f - 1.0f) / p;
        t->invp[i] = 1.0f / p;
        t->c[i] = y2;
        y2f = y2;
    }
}

// One channel by LANES threads (one warp, or a pair of warps: 64 lanes halve
// each lane's serial recurrences): src (nt samples) -> dst (nt records); smem
// holds two arrays of (nt + 4) & ~3 floats: the channel, and u overwritten in
// place by z (each lane first runs its back-substitution warm-up over the next
// lanes' u, then all lanes overwrite their own chunks).  A pair synchronises on
// named barrier `bar` (1..15).
template <int LANES>
__device__ __forceinline__ void lanes_sync(int bar) {
    if (LANES == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(LANES) : "memory");
}
template <typename T, int LANES = 32>
__device__ __forceinline__ void spline_channel(const T *__restrict__ src,
                                               typename CoefRec<T>::raw *__restrict__ dst, int nt,
                                               float t0, float dt, const SplineTable &tab,
                                               float *smem, int bar = 0) {
    const int lane = threadIdx.x & (LANES - 1);
    const int stride = (nt + 4) & ~3;  // >= nt+1, keeps every array 16-byte aligned
    float *y = smem;
    float *uz = y + stride;  // u, then z

    // stage the channel: 16-byte vector loads, several in flight per lane
    constexpr int V = 16 / sizeof(T);
    if ((nt % V) == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
#pragma unroll 8
        for (int k = lane; k < nt / V; k += LANES) {
            const uint4 v = __ldg(s4 + k);
            const T *e = reinterpret_cast<const T *>(&v);
#pragma unroll
            for (int m = 0; m < V; ++m) y[k * V + m] = load_sample_reg(e[m]);
        }
    } else {
        for (int k = lane; k < nt; k += LANES) y[k] = load_sample(src + k);
    }
    if (lane == 0) {
        y[nt] = 0.f;
        uz[0] = 0.f;
        uz[nt] = 0.f;
        uz[nt - 1] = 0.f;
    }
    lanes_sync<LANES>(bar);

    const float inv_dt = 1.0f / dt;
    const float cscale = 6.0f / (2.0f * dt);
    const float zscale = dt * dt / 6.0f;
    // chunk length odd: lane l then reads word l*C + i, a distinct bank per lane
    const int C = ((nt + LANES - 1) / LANES) | 1;
    const int s = lane * C;
    const int e = min(s + C, nt);

    // forward sweep: u_i for i in [max(s,1), min(e, nt-1))
    {
        const int ib = max(s, 1), ie = min(e, nt - 1);
        if (ib < ie) {
            float up = 0.f;
            for (int i = max(1, ib - kWarm); i < ie; ++i) {
                const float d1 = (y[i + 1] - y[i]) * inv_dt;
                const float d0 = (y[i] - y[i - 1]) * inv_dt;
                const float ui = fmaf(d1 - d0, cscale, -0.5f * up) * tab.invp[min(i, kSplineTab - 1)];
                if (i >= ib) uz[i] = ui;
                up = ui;
            }
        }
    }
    lanes_sync<LANES>(bar);
    // back-substitution: y2_k for k in [s, min(e, nt-1)), y2_{nt-1} = 0; the
    // warm-up over the next lanes' u first, then this lane's chunk in place
    const int kb = s, ke = min(e, nt - 1);
    float yn = 0.f;
    if (kb < ke)
        for (int k = min(nt - 2, ke - 1 + kWarm); k >= ke; --k)
            yn = fmaf(tab.c[min(k, kSplineTab - 1)], yn, uz[k]);
    lanes_sync<LANES>(bar);
    if (kb < ke)
        for (int k = ke - 1; k >= kb; --k) {
            const float uk = (k == 0) ? 0.f : uz[k];
            const float y2k = fmaf(tab.c[min(k, kSplineTab - 1)], yn, uk);
            uz[k] = y2k * zscale;
            yn = y2k;
        }
    lanes_sync<LANES>(bar);
    for (int k = lane; k < nt; k += LANES)
        dst[k] = CoefRec<T>::make(y[k], y[k + 1], uz[k], uz[k + 1], k, t0, dt);
}

// one channel per pair of warps (named barrier 1 + pair index)
template <typename T>
__global__ void __launch_bounds__(256)
spline_coef_kernel(const T *__restrict__ rf, typename CoefRec<T>::raw *__restrict__ coef,
                   long long nch, int nt, float t0, float dt,
                   const __grid_constant__ SplineTable tab) {
    extern __shared__ float smem[];
    const int pr = threadIdx.x >> 6;
    const int ppb = blockDim.x >> 6;
    const long long ch = (long long)blockIdx.x * ppb + pr;
    if (ch >= nch) return;  // both warps of a pair leave together
    const int stride = (nt + 4) & ~3;
    spline_channel<T, 64>(rf + ch * (long long)nt, coef + ch * (long long)nt, nt, t0, dt, tab,
                          smem + (size_t)pr * 2 * stride, 1 + pr);
}

// Batched: one pair of warps per channel of any job (jobs' channels numbered
// consecutively from BatchJob::ch0), as spline_coef_kernel (the same
// records); shared memory per pair sized for the longest channel.
template <typename T>
__device__ __forceinline__ void batch_spline_one(const BatchJob &j, long long ch, float *sm,
                                                 const SplineTable &tab, int bar) {
    using raw = typename CoefRec<T>::raw;
    const int nt = j.a.nt;
    spline_channel<T, 64>(static_cast<const T *>(j.rf) + ch * (long long)nt,
                          static_cast<raw *>(const_cast<void *>(j.a.data)) + ch * (long long)nt, nt,
                          j.a.t0, j.a.dt, tab, sm, bar);
}

__global__ void __launch_bounds__(256)
batch_spline_kernel(const BatchJob *__restrict__ jobs, int njobs, long long nch_total,
                    int max_stride, const __grid_constant__ SplineTable tab) {
    extern __shared__ float smem[];
    const int w = threadIdx.x >> 6;  // pair
    const int wpb = blockDim.x >> 6;
    const long long gc = (long long)blockIdx.x * wpb + w;
    if (gc >= nch_total) return;  // both warps of a pair leave together
    // the job whose channel range holds gc (jobs sorted by ch0)
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].ch0 <= gc) lo = mid;
        else hi = mid - 1;
    }
    const BatchJob &j = jobs[lo];
    const long long ch = gc - j.ch0;
    float *sm = smem + (size_t)w * 2 * max_stride;
    switch (j.dtype) {
        case PYCBF_GB_F32: batch_spline_one<float>(j, ch, sm, tab, 1 + w); break;
        case PYCBF_GB_F16: batch_spline_one<__half>(j, ch, sm, tab, 1 + w); break;
        default: batch_spline_one<__nv_bfloat16>(j, ch, sm, tab, 1 + w); break;
    }
}

template <typename T>
static cudaError_t launch_spline_t(const SplineArgs &a, cudaStream_t s) {
    const size_t per_pair = sizeof(float) * 2 * (size_t)((a.nt + 4) & ~3);
    const int ppb = (int)std::min<size_t>(4, std::max<size_t>(1, (72 * 1024) / per_pair));
    const size_t smem = per_pair * ppb;
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    static SplineTable tab = [] {
        SplineTable t;
        make_spline_table(&t);
        return t;
    }();
    cudaError_t err = cudaFuncSetAttribute(spline_coef_kernel<T>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    const long long blocks = (a.nch + ppb - 1) / ppb;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    spline_coef_kernel<T><<<(unsigned)blocks, 64 * ppb, smem, s>>>(
        static_cast<const T *>(a.rf), static_cast<typename CoefRec<T>::raw *>(a.coef), a.nch, a.nt,
        a.t0, a.dt, tab);
    return cudaGetLastError();
}

cudaError_t launch_batch_spline(const BatchJob *jobs, int njobs, long long nch_total, int max_nt,
                                cudaStream_t s, bool set_attr) {
    const int stride = (max_nt + 4) & ~3;
    const size_t per_pair = sizeof(float) * 2 * (size_t)stride;
    const int ppb = (int)std::min<size_t>(4, std::max<size_t>(1, (72 * 1024) / per_pair));
    const size_t smem = per_pair * ppb;
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    static SplineTable tab = [] {
        SplineTable t;
        make_spline_table(&t);
        return t;
    }();
    if (set_attr) {
        cudaError_t err = cudaFuncSetAttribute(batch_spline_kernel,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    if (nch_total <= 0) return cudaSuccess;
    const long long blocks = (nch_total + ppb - 1) / ppb;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    batch_spline_kernel<<<(unsigned)blocks, 64 * ppb, smem, s>>>(jobs, njobs, nch_total, stride, tab);
    return cudaGetLastError();
}

cudaError_t launch_spline(const SplineArgs &a, int dtype, cudaStream_t s) {
    switch (dtype) {
        case PYCBF_GB_F32: return launch_spline_t<float>(a, s);
        case PYCBF_GB_F16: return launch_spline_t<__half>(a, s);
        case PYCBF_GB_BF16: return launch_spline_t<__nv_bfloat16>(a, s);
        case PYCBF_GB_I16: return launch_spline_t<short>(a, s);  // conversion fused into the staging
        default: return cudaErrorInvalidValue;
    }
}

// int16 -> float32 for the interpolations that gather samples directly:
// eight samples per thread (one 16-byte load, two 16-byte stores) where the
// buffers are 16-byte aligned, else one.
__global__ void __launch_bounds__(256) convert_i16_kernel(const short *__restrict__ src,
                                                          long long n, float *__restrict__ dst,
                                                          int vec) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (vec) {
        const long long n8 = n / 8;
        for (long long k = i; k < n8; k += stride) {
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(src) + k);
            const short *e = reinterpret_cast<const short *>(&v);
            float4 *d = reinterpret_cast<float4 *>(dst) + 2 * k;
            d[0] = make_float4(e[0], e[1], e[2], e[3]);
            d[1] = make_float4(e[4], e[5], e[6], e[7]);
        }
        for (long long k = n8 * 8 + i; k < n; k += stride) dst[k] = (float)__ldg(src + k);
    } else {
        for (long long k = i; k < n; k += stride) dst[k] = (float)__ldg(src + k);
    }
}

cudaError_t launch_convert_i16(const short *src, long long n, float *dst, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int vec = (reinterpret_cast<uintptr_t>(src) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(dst) % 16 == 0) ? 1 : 0;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        sms = 148;
    long long blocks = ((vec ? n / 8 : n) + 255) / 256;
    blocks = std::max(1LL, std::min(blocks, 8LL * sms));
    convert_i16_kernel<<<(unsigned)blocks, 256, 0, s>>>(src, n, dst, vec);
    return cudaGetLastError();
}

}  // namespace pgb

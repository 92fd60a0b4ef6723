// DMAS over separated images and short-lag spatial coherence (SLSC).
#include <algorithm>

#include "common.cuh"

namespace pgb {

// ---------------------------------------------------------------------------
// DMAS: one thread per pixel, one frame per grid row.  For each listed lag L
// the pairs (s, s+L) of the separated images are multiplied and summed as
// sign(p) sqrt|p| (signed square root) or p (power); the reference kernel
// (pycbf/gpu/__advanced_engines__.cu:17-61) does the same with one thread and
// one atomicAdd per (lag, s, pixel).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
dmas_kernel(const float *__restrict__ im, long long nsep, long long np, const int *__restrict__ lags,
            int nlag, int power, int sumlags, float *__restrict__ out) {
    const long long ip = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= np) return;
    const long long f = blockIdx.y;
    const float *col = im + f * nsep * np + ip;
    float tot = 0.f;
    for (int l = 0; l < nlag; ++l) {
        const long long lag = __ldg(lags + l);
        float acc = 0.f;
        if (lag >= 0) {
            for (long long s = 0; s + lag < nsep; ++s) {
                const float p = __fmul_rn(__ldg(col + s * np), __ldg(col + (s + lag) * np));
                acc += power ? p : copysignf(sqrtf(fabsf(p)), p);
            }
        }
        if (sumlags) tot += acc;
        else out[(f * nlag + l) * np + ip] = acc;
    }
    if (sumlags) out[f * np + ip] = tot;
}

cudaError_t launch_dmas(const float *im, long long nframes, long long nsep, long long np,
                        const int *lags, int nlag, int power, int sumlags, float *out,
                        cudaStream_t s) {
    const long long bx = (np + 255) / 256;
    dmas_kernel<<<dim3((unsigned)bx, (unsigned)nframes), 256, 0, s>>>(im, nsep, np, lags, nlag,
                                                                     power, sumlags, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// SLSC: one thread per pixel (ix, iz); consecutive threads take consecutive iz
// so every element row is read coalesced.  The thread walks the elements in
// order, keeps those whose receive mask is on over its whole axial kernel,
// normalises each kept element's kernel samples to zero mean and unit
// population deviation, and correlates it with the previous nlag kept
// elements, whose normalised samples wait in a ring in this thread's slice of
// shared memory ([slot][w][thread] layout: conflict-free).  Per lag it keeps
// the sum and count of valid pair correlations (the nan-mean of the notebook).
// ---------------------------------------------------------------------------
constexpr float kSigmaMin = 1e-10f;

__global__ void slsc_kernel(const float *__restrict__ im, const unsigned char *__restrict__ mask,
                            int nrx, int nx, int nz, int nlag, int nkern,
                            float *__restrict__ out) {
    extern __shared__ float ring[];
    const int tid = threadIdx.x;
    const int bs = blockDim.x;
    const long long pix = (long long)blockIdx.x * bs + tid;
    const long long npix = (long long)nx * nz;
    if (pix >= npix) return;
    const int ix = (int)(pix / nz), iz = (int)(pix % nz);
    const long long f = blockIdx.y;
    const int kmax = 2 * nkern + 1;
    const int z0 = max(0, iz - nkern), z1 = min(nz, iz + nkern + 1);
    const int L = z1 - z0;
    const float invL = 1.0f / (float)L;

    // per-lag sums and counts live in shared memory after the ring
    float *lag_sum = ring + (size_t)nlag * kmax * bs;
    int *lag_cnt = reinterpret_cast<int *>(lag_sum + (size_t)nlag * bs);
    for (int m = 0; m < nlag; ++m) {
        lag_sum[m * bs + tid] = 0.f;
        lag_cnt[m * bs + tid] = 0;
    }
    // validity of ring slots: bit per slot (nlag <= 32)
    unsigned valid = 0u;
    int nsel = 0;
    constexpr int kLmax = 64;
    float v[kLmax];

    for (int e = 0; e < nrx; ++e) {
        const long long row = ((long long)e * nx + ix) * nz;
        bool on = true;
        for (int z = z0; z < z1; ++z) on = on && (__ldg(mask + row + z) != 0);
        if (!on) continue;
        const float *x = im + (f * nrx) * (long long)nx * nz + row;
        float mu = 0.f;
        for (int w = 0; w < L; ++w) {
            v[w] = __ldg(x + z0 + w);
            mu += v[w];
        }
        mu *= invL;
        float var = 0.f;
        for (int w = 0; w < L; ++w) {
            v[w] -= mu;
            var = fmaf(v[w], v[w], var);
        }
        const float sd = sqrtf(var * invL);
        const bool ok = !(sd < kSigmaMin);
        const float inv_sd = ok ? 1.0f / sd : 0.f;
        for (int w = 0; w < L; ++w) v[w] *= inv_sd;
        // correlate with the previous kept elements k - m, m = 1..nlag
        const int k = nsel;
        for (int m = 1; m <= nlag && m <= k; ++m) {
            const int slot = (k - m) % nlag;
            if (ok && ((valid >> slot) & 1u)) {
                const float *prev = ring + (size_t)slot * kmax * bs + tid;
                float dot = 0.f;
                for (int w = 0; w < L; ++w) dot = fmaf(v[w], prev[(size_t)w * bs], dot);
                lag_sum[(m - 1) * bs + tid] += dot * invL;
                lag_cnt[(m - 1) * bs + tid] += 1;
            }
        }
        const int slot = k % nlag;
        float *dst = ring + (size_t)slot * kmax * bs + tid;
        for (int w = 0; w < L; ++w) dst[(size_t)w * bs] = v[w];
        valid = ok ? (valid | (1u << slot)) : (valid & ~(1u << slot));
        ++nsel;
    }
    float res = 0.f;
    if (nsel >= nlag + 1) {
        for (int m = 0; m < nlag; ++m) {
            const int c = lag_cnt[m * bs + tid];
            const float r = c ? lag_sum[m * bs + tid] / (float)c : __int_as_float(0x7fc00000);
            res += r / (float)nlag;
        }
    }
    out[f * npix + pix] = res;
}

cudaError_t launch_slsc(const float *im, const unsigned char *mask, long long nframes, int nrx,
                        int nx, int nz, int nlag, int nkern, float *out, cudaStream_t s) {
    const int kmax = 2 * nkern + 1;
    const size_t per_thread = sizeof(float) * ((size_t)nlag * kmax + 2 * (size_t)nlag);
    int bs = (int)std::min<size_t>(128, (200 * 1024) / per_thread);
    bs = (bs / 32) * 32;
    if (bs < 32) return cudaErrorInvalidValue;
    const size_t smem = per_thread * bs;
    cudaError_t err = cudaFuncSetAttribute(slsc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
    if (err != cudaSuccess) return err;
    const long long npix = (long long)nx * nz;
    const long long bx = (npix + bs - 1) / bs;
    slsc_kernel<<<dim3((unsigned)bx, (unsigned)nframes), bs, smem, s>>>(im, mask, nrx, nx, nz,
                                                                       nlag, nkern, out);
    return cudaGetLastError();
}

}  // namespace pgb

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

// ---------------------------------------------------------------------------
// SLSC with register-blocked lag accumulators (nlag <= 16, nkern <= 3, nrx <=
// 256): one thread per pixel (ix, iz), consecutive threads consecutive iz.
// The thread first marks, in a bit set, the elements whose receive mask is on
// over its whole axial kernel (the kept elements, in element order).  It then
// walks the kept elements in chunks of 16 with the loop unrolled, so that the
// normalised kernels of the previous 16 kept elements sit in a register ring
// with static slots: each kept element's kernel (mean-subtracted, divided by
// its population deviation; a zero vector when that deviation is below 1e-10)
// is correlated with the 16 ring entries, 7 multiply-adds each, into one sum
// per lag, and the valid pairs are counted per lag from a bit history of the
// valid kernels (four 8-bit counts per register).  The result is the mean over
// lags of sum / (pairs * kernel length), NaN for a lag without pairs, and 0
// where the pixel keeps at most nlag elements -- the definition of slsc_kernel.
// ---------------------------------------------------------------------------
constexpr int kSlscLags = 16;
constexpr int kSlscKern = 3;
constexpr int kSlscWin = 2 * kSlscKern + 1;
constexpr int kSlscWords = 8;  // kept-element bits: nrx <= 256

// Kept elements of pixel (ix, iz): bit e of kept[e / 32] is set when element
// e's receive mask is on over the whole axial kernel [z0, z1) (the mask bytes
// of one element are all in flight at once; positions past z1 read as on).
__device__ __forceinline__ void slsc_kept_bits(const unsigned char *__restrict__ mask, int nrx,
                                               int nx, int nz, int ix, int z0, int z1,
                                               unsigned (&kept)[kSlscWords]) {
#pragma unroll
    for (int q = 0; q < kSlscWords; ++q) kept[q] = 0u;
    for (int e = 0; e < nrx; ++e) {
        const unsigned char *m = mask + ((long long)e * nx + ix) * nz;
        unsigned on = 1u;
#pragma unroll
        for (int w = 0; w < kSlscWin; ++w) {
            const int z = z0 + w;
            on &= (z < z1) ? (unsigned)(__ldg(m + min(z, nz - 1)) != 0) : 1u;
        }
#pragma unroll
        for (int q = 0; q < kSlscWords; ++q)
            if (q == (e >> 5)) kept[q] |= on << (e & 31);
    }
}

// The kept-element bit sets of every pixel for one axial kernel half-width,
// word q of pixel p at kept[q * npix + p] (q < ceil(nrx / 32)): they depend
// on the receive mask only, so a beamformer computes them once and every
// frame's coherence pass reads 4 bytes per 32 elements instead of the
// kernel's mask bytes of every element.
__global__ void __launch_bounds__(128)
slsc_kept_kernel(const unsigned char *__restrict__ mask, int nrx, int nx, int nz, int nkern,
                 unsigned *__restrict__ kept_out) {
    const long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long npix = (long long)nx * nz;
    if (pix >= npix) return;
    const int ix = (int)(pix / nz), iz = (int)(pix % nz);
    const int z0 = max(0, iz - nkern), z1 = min(nz, iz + nkern + 1);
    unsigned kept[kSlscWords];
    slsc_kept_bits(mask, nrx, nx, nz, ix, z0, z1, kept);
    const int nw = (nrx + 31) >> 5;
#pragma unroll
    for (int q = 0; q < kSlscWords; ++q)
        if (q < nw) kept_out[q * npix + pix] = kept[q];
}

// PRE: the kept bit sets come from slsc_kept_kernel's array (kept_in), else
// from the mask bytes.
template <bool PRE>
__global__ void __launch_bounds__(128, 3)  // 3 CTAs (168 registers): 1.09 ms against 1.30 at 2
slsc_reg_kernel(const float *__restrict__ im, const unsigned char *__restrict__ mask,
                const unsigned *__restrict__ kept_in, int nrx, int nx, int nz, int nlag, int nkern,
                float *__restrict__ out) {
    const long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long npix = (long long)nx * nz;
    if (pix >= npix) return;
    const int ix = (int)(pix / nz), iz = (int)(pix % nz);
    const long long f = blockIdx.y;
    const int z0 = max(0, iz - nkern), z1 = min(nz, iz + nkern + 1);
    const int L = z1 - z0;
    const float invL = 1.0f / (float)L;

    // kept elements: receive mask on over the whole kernel
    unsigned kept[kSlscWords];
    if constexpr (PRE) {
        const int nw = (nrx + 31) >> 5;
#pragma unroll
        for (int q = 0; q < kSlscWords; ++q) kept[q] = q < nw ? __ldg(kept_in + q * npix + pix) : 0u;
    } else {
        slsc_kept_bits(mask, nrx, nx, nz, ix, z0, z1, kept);
    }
    int nsel = 0;
#pragma unroll
    for (int q = 0; q < kSlscWords; ++q) nsel += __popc(kept[q]);

    const float *base = im + (f * nrx) * (long long)nx * nz + (long long)ix * nz + z0;
    const long long estride = (long long)nx * nz;
    float ring[kSlscLags][kSlscWin];
#pragma unroll
    for (int u = 0; u < kSlscLags; ++u)
#pragma unroll
        for (int w = 0; w < kSlscWin; ++w) ring[u][w] = 0.f;
    float lag[kSlscLags];
#pragma unroll
    for (int m = 0; m < kSlscLags; ++m) lag[m] = 0.f;
    // bit k of vbits: the kept element k had a valid kernel (deviation >= 1e-10)
    unsigned vbits[kSlscWords];
#pragma unroll
    for (int q = 0; q < kSlscWords; ++q) vbits[q] = 0u;

    int q = 0;
    unsigned cur = kept[0];
    // the next kept element (element order), or -1
    auto next_elem = [&]() -> int {
        while (cur == 0u) {
            if (++q >= kSlscWords) return -1;
#pragma unroll
            for (int r = 0; r < kSlscWords; ++r)
                if (r == q) cur = kept[r];
        }
        const int b = __ffs(cur) - 1;
        cur &= cur - 1u;
        return 32 * q + b;
    };
    for (int k0 = 0; k0 < nsel; k0 += kSlscLags) {
#pragma unroll
        for (int u = 0; u < kSlscLags; ++u) {
            if (k0 + u < nsel) {
                const int e = next_elem();
                const float *x = base + (long long)e * estride;
                float v[kSlscWin];
                float mu = 0.f;
#pragma unroll
                for (int w = 0; w < kSlscWin; ++w) {
                    v[w] = (w < L) ? __ldg(x + w) : 0.f;
                    mu += v[w];
                }
                mu *= invL;
                float var = 0.f;
#pragma unroll
                for (int w = 0; w < kSlscWin; ++w) {
                    v[w] = (w < L) ? v[w] - mu : 0.f;
                    var = fmaf(v[w], v[w], var);
                }
                const float sd = sqrtf(var * invL);
                const bool ok = !(sd < kSigmaMin);
                const float inv_sd = ok ? 1.0f / sd : 0.f;
#pragma unroll
                for (int w = 0; w < kSlscWin; ++w) v[w] *= inv_sd;
#pragma unroll
                for (int m = 1; m <= kSlscLags; ++m) {
                    const float *pr = ring[(u - m + kSlscLags) % kSlscLags];
                    float d = lag[m - 1];
#pragma unroll
                    for (int w = 0; w < kSlscWin; ++w) d = fmaf(v[w], pr[w], d);
                    lag[m - 1] = d;
                }
#pragma unroll
                for (int w = 0; w < kSlscWin; ++w) ring[u][w] = v[w];
                const int k = k0 + u;
#pragma unroll
                for (int qq = 0; qq < kSlscWords; ++qq)
                    if (qq == (k >> 5)) vbits[qq] |= (ok ? 1u : 0u) << (k & 31);
            }
        }
    }
    float res = 0.f;
    if (nsel >= nlag + 1) {
        for (int m = 0; m < kSlscLags; ++m) {
            if (m < nlag) {
                // pairs of lag m + 1 with both kernels valid: popc(vbits & vbits >> (m + 1))
                int c = 0;
#pragma unroll
                for (int qq = 0; qq < kSlscWords; ++qq) {
                    const unsigned hi = qq + 1 < kSlscWords ? vbits[qq + 1] : 0u;
                    const unsigned sh = __funnelshift_r(vbits[qq], hi, m + 1);
                    c += __popc(vbits[qq] & sh);
                }
                const float r = c ? lag[m] * invL / (float)c : __int_as_float(0x7fc00000);
                res += r / (float)nlag;
            }
        }
    }
    out[f * npix + pix] = res;
}

bool slsc_kept_supported(int nrx, int nlag, int nkern) {
    return nlag <= kSlscLags && nkern <= kSlscKern && nrx <= 32 * kSlscWords;
}

cudaError_t launch_slsc_kept(const unsigned char *mask, int nrx, int nx, int nz, int nkern,
                             unsigned *kept, cudaStream_t s) {
    const long long npix = (long long)nx * nz;
    const long long bx = (npix + 127) / 128;
    slsc_kept_kernel<<<(unsigned)bx, 128, 0, s>>>(mask, nrx, nx, nz, nkern, kept);
    return cudaGetLastError();
}

cudaError_t launch_slsc(const float *im, const unsigned char *mask, const unsigned *kept,
                        long long nframes, int nrx, int nx, int nz, int nlag, int nkern, float *out,
                        cudaStream_t s) {
    if (slsc_kept_supported(nrx, nlag, nkern)) {
        const long long npix = (long long)nx * nz;
        const long long bx = (npix + 127) / 128;
        const dim3 grid((unsigned)bx, (unsigned)nframes);
        if (kept)
            slsc_reg_kernel<true><<<grid, 128, 0, s>>>(im, nullptr, kept, nrx, nx, nz, nlag, nkern,
                                                       out);
        else
            slsc_reg_kernel<false><<<grid, 128, 0, s>>>(im, mask, nullptr, nrx, nx, nz, nlag,
                                                        nkern, out);
        return cudaGetLastError();
    }
    if (!mask) return cudaErrorInvalidValue;
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

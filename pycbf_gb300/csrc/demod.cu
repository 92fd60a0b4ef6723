// IQ demodulation, envelope and log compression of beamformed images: the step
// after the delay-and-sum in the reference's examples.
//
// fft_tukey_demod (examples/SyntheticPointBeamforming.ipynb cell 1, the same
// function in SyntheticVsTabbed.ipynb cell 1 and develop_dmas_class.ipynb
// cell 7) takes the real FFT of every image line along one axis, keeps bins
// [ikmin, ikmax), weights them by a Tukey window, shifts them to base band
// (ifftshift) and inverse-FFTs the M = ikmax - ikmin bins to M complex
// samples.  Every step is linear, so the whole map is one complex n x M matrix
// W (built on the host in float64 by applying those steps to the identity,
// rounded to float32), and here iq[c][m] = sum_k x[c][k] W[k][m] is a
// real-by-complex matrix product in float32 on the FMA pipe (TF32 or BF16
// tensor-core operands would give up the ~3 decimal digits the parity bound
// needs; the product is ~1 % of a frame's delay-and-sum).  The epilogue writes
// the IQ samples and/or the envelope |iq|.
//
// The examples display 20 log10(env / percentile(env, 99) + 1e-10)
// (SyntheticPointBeamforming.ipynb cell 11).  The percentile is NumPy's
// 'linear' rule: the two order statistics at floor((n-1) q/100) and the next
// are selected exactly (four 8-bit radix passes over order-preserving keys of
// the float bits, both ranks at once), then interpolated in float64 as
// numpy's _lerp does.  The log compression reads the percentile from device
// memory, so the chain runs without a host round trip.
#include "common.cuh"

namespace pgb {

namespace {

constexpr int kDmC = 32;        // image lines per CTA
constexpr int kDmM = 32;        // complex outputs per CTA
constexpr int kDmK = 32;        // input samples per shared-memory stage
constexpr int kDmThreads = 128; // 8 x 16 threads, each 4 lines x 2 outputs

__global__ void __launch_bounds__(kDmThreads) demod_kernel(const float *__restrict__ x,
                                                           long long ncols, int n,
                                                           const float2 *__restrict__ W, int M,
                                                           float2 *__restrict__ iq,
                                                           float *__restrict__ env) {
    __shared__ float xs[kDmK][kDmC + 1];  // [k][line]: odd row length, no bank conflicts
    __shared__ float2 ws[kDmK][kDmM];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const long long c0 = (long long)blockIdx.x * kDmC;
    const int m0 = blockIdx.y * kDmM;
    float2 acc[4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) acc[i][j] = make_float2(0.f, 0.f);

    for (int k0 = 0; k0 < n; k0 += kDmK) {
        for (int e = tid; e < kDmC * kDmK; e += kDmThreads) {
            const int r = e / kDmK, kk = e % kDmK;
            const long long c = c0 + r;
            const int k = k0 + kk;
            xs[kk][r] = (c < ncols && k < n) ? __ldg(x + c * n + k) : 0.f;
        }
        for (int e = tid; e < kDmK * kDmM; e += kDmThreads) {
            const int kk = e / kDmM, mm = e % kDmM;
            const int k = k0 + kk, m = m0 + mm;
            ws[kk][mm] = (k < n && m < M) ? __ldg(W + (long long)k * M + m) : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < kDmK; ++kk) {
            float a[4];
            float2 b[2];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = xs[kk][ty + 8 * i];
#pragma unroll
            for (int j = 0; j < 2; ++j) b[j] = ws[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    acc[i][j].x = fmaf(a[i], b[j].x, acc[i][j].x);
                    acc[i][j].y = fmaf(a[i], b[j].y, acc[i][j].y);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const long long c = c0 + ty + 8 * i;
            const int m = m0 + tx + 16 * j;
            if (c < ncols && m < M) {
                const long long o = c * M + m;
                if (iq) iq[o] = acc[i][j];
                if (env) env[o] = sqrtf(fmaf(acc[i][j].x, acc[i][j].x, acc[i][j].y * acc[i][j].y));
            }
        }
}

// ---------------------------------------------------------------------------
// percentile: exact selection of two order statistics per segment
// ---------------------------------------------------------------------------
// workspace per segment: histograms [pass 4][rank 2][256] and a NaN flag
constexpr int kPctSegWords = 4 * 2 * 256 + 32;
constexpr int kPctNanWord = 4 * 2 * 256;

// order-preserving key of a float (NaN -> the largest key, which no number has)
__device__ __forceinline__ unsigned pct_key(float v) {
    const unsigned u = __float_as_uint(v);
    if (v != v) return 0xffffffffu;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float pct_value(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// One warp: the bin holding rank k (0-based) of the counts h[0..255]; k
// becomes the rank within that bin.
__device__ int warp_pick(const unsigned *h, unsigned &k) {
    const int lane = threadIdx.x & 31;
    unsigned c[8], s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        c[i] = h[lane * 8 + i];
        s += c[i];
    }
    unsigned incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, incl > k);
    const int owner = ballot ? __ffs(ballot) - 1 : 31;
    unsigned below = incl - s;
    int i_hit = 7;
    bool done = false;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        if (!done) {
            if (i == 7 || below + c[i] > k) {
                i_hit = i;
                done = true;
            } else {
                below += c[i];
            }
        }
    }
    int bin = __shfl_sync(0xffffffffu, lane * 8 + i_hit, owner);
    below = __shfl_sync(0xffffffffu, below, owner);
    k -= below;
    return bin;
}

// One warp: the key prefixes (the top 8*passes bits) and in-prefix ranks of
// both ranks after `passes` passes.  Rank 1 counts in its own histogram only
// from the pass where its prefix first differs from rank 0's.
__device__ void pct_replay(const unsigned *hs, int passes, unsigned k0, unsigned k1,
                           unsigned pre[2], unsigned kr[2]) {
    pre[0] = pre[1] = 0;
    kr[0] = k0;
    kr[1] = k1;
    for (int q = 0; q < passes; ++q) {
        const int shift = 24 - 8 * q;
        const bool split = pre[0] != pre[1];
        const unsigned *h0 = hs + (q * 2 + 0) * 256;
        const unsigned *h1 = split ? hs + (q * 2 + 1) * 256 : h0;
        const int b0 = warp_pick(h0, kr[0]);
        const int b1 = warp_pick(h1, kr[1]);
        pre[0] |= (unsigned)b0 << shift;
        pre[1] |= (unsigned)b1 << shift;
    }
}

__global__ void __launch_bounds__(256) pct_hist_kernel(const float *__restrict__ v, long long n,
                                                       int pass, unsigned k0, unsigned k1,
                                                       unsigned *__restrict__ ws) {
    __shared__ unsigned h[2][256];
    __shared__ unsigned s_pre[2];
    __shared__ int s_split;
    const int tid = threadIdx.x;
    unsigned *hs = ws + (long long)blockIdx.y * kPctSegWords;
    h[0][tid] = 0;
    h[1][tid] = 0;
    if (tid < 32) {
        unsigned pre[2], kr[2];
        pct_replay(hs, pass, k0, k1, pre, kr);
        if (tid == 0) {
            s_pre[0] = pre[0];
            s_pre[1] = pre[1];
            s_split = pre[0] != pre[1];
        }
    }
    __syncthreads();
    const int shift = 24 - 8 * pass;
    const unsigned p0 = s_pre[0], p1 = s_pre[1];
    const bool split = s_split != 0;
    const float *vs = v + (long long)blockIdx.y * n;
    bool nan_seen = false;
    for (long long i = (long long)blockIdx.x * blockDim.x + tid; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float val = __ldg(vs + i);
        nan_seen |= val != val;
        const unsigned key = pct_key(val);
        const unsigned d = (key >> shift) & 255u;
        if (pass == 0) {
            atomicAdd(&h[0][d], 1u);
        } else {
            const int hi = shift + 8;  // 8..24
            if ((key >> hi) == (p0 >> hi)) atomicAdd(&h[0][d], 1u);
            if (split && (key >> hi) == (p1 >> hi)) atomicAdd(&h[1][d], 1u);
        }
    }
    const int any_nan = __syncthreads_or(nan_seen ? 1 : 0);
    if (h[0][tid]) atomicAdd(hs + (pass * 2 + 0) * 256 + tid, h[0][tid]);
    if (split && h[1][tid]) atomicAdd(hs + (pass * 2 + 1) * 256 + tid, h[1][tid]);
    if (tid == 0 && any_nan) atomicOr(hs + kPctNanWord, 1u);
}

// one warp per segment: both order statistics, then numpy's _lerp in float64
__global__ void __launch_bounds__(32) pct_final_kernel(unsigned k0, unsigned k1, double gamma,
                                                       const unsigned *__restrict__ ws,
                                                       float *__restrict__ out) {
    const unsigned *hs = ws + (long long)blockIdx.x * kPctSegWords;
    unsigned pre[2], kr[2];
    pct_replay(hs, 4, k0, k1, pre, kr);
    if (threadIdx.x == 0) {
        if (hs[kPctNanWord]) {
            out[blockIdx.x] = __int_as_float(0x7fc00000);
            return;
        }
        const double a = pct_value(pre[0]), b = pct_value(pre[1]);
        const double d = b - a;
        const double r = (gamma >= 0.5) ? b - d * (1.0 - gamma) : a + d * gamma;
        out[blockIdx.x] = __double2float_rn(r);
    }
}

// env and out may be the same array (each element is read, then written, by one thread)
__global__ void __launch_bounds__(256) log_compress_kernel(const float *env, long long nseg,
                                                           long long n,
                                                           const float *__restrict__ ref,
                                                           float floor_add, float *out) {
    const long long total = nseg * n;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const float r = __ldg(ref + i / n);
        out[i] = 20.0f * log10f(__fadd_rn(__fdiv_rn(env[i], r), floor_add));
    }
}

int sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        sms = 148;
    return sms;
}

}  // namespace

cudaError_t launch_demod(const float *x, long long ncols, int n, const float2 *W, int M,
                         float2 *iq, float *env, cudaStream_t s) {
    if (ncols == 0) return cudaSuccess;
    const long long gx = (ncols + kDmC - 1) / kDmC;
    const long long gy = ((long long)M + kDmM - 1) / kDmM;
    if (gx > 0x7fffffffLL || gy > 65535) return cudaErrorInvalidValue;
    demod_kernel<<<dim3((unsigned)gx, (unsigned)gy), kDmThreads, 0, s>>>(x, ncols, n, W, M, iq, env);
    return cudaGetLastError();
}

size_t percentile_workspace_bytes(long long nseg) {
    return (size_t)nseg * kPctSegWords * sizeof(unsigned);
}

cudaError_t launch_percentile(const float *v, long long nseg, long long n, double q, float *out,
                              void *ws, cudaStream_t s) {
    if (nseg == 0) return cudaSuccess;
    const double idx = (double)(n - 1) * (q / 100.0);
    const long long lo = (long long)floor(idx);
    const long long k0 = lo < 0 ? 0 : (lo > n - 1 ? n - 1 : lo);
    const long long k1 = k0 + 1 < n ? k0 + 1 : n - 1;
    const double gamma = idx - (double)lo;
    cudaError_t e = cudaMemsetAsync(ws, 0, percentile_workspace_bytes(nseg), s);
    if (e != cudaSuccess) return e;
    long long gx = (n + 4095) / 4096;
    const long long want = (4LL * sm_count() + nseg - 1) / nseg;
    if (gx > want) gx = want;
    if (gx < 1) gx = 1;
    unsigned *w = static_cast<unsigned *>(ws);
    for (int pass = 0; pass < 4; ++pass) {
        pct_hist_kernel<<<dim3((unsigned)gx, (unsigned)nseg), 256, 0, s>>>(v, n, pass, (unsigned)k0,
                                                                          (unsigned)k1, w);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    pct_final_kernel<<<(unsigned)nseg, 32, 0, s>>>((unsigned)k0, (unsigned)k1, gamma, w, out);
    return cudaGetLastError();
}

cudaError_t launch_log_compress(const float *env, long long nseg, long long n, const float *ref,
                                float floor_add, float *out, cudaStream_t s) {
    const long long total = nseg * n;
    if (total == 0) return cudaSuccess;
    long long blocks = (total + 255) / 256;
    const long long cap = 8LL * sm_count();
    if (blocks > cap) blocks = cap;
    log_compress_kernel<<<(unsigned)blocks, 256, 0, s>>>(env, nseg, n, ref, floor_add, out);
    return cudaGetLastError();
}

}  // namespace pgb

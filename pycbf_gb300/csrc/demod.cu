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
#include <algorithm>

#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace pgb {

namespace {

constexpr int kDmC = 16;        // image lines per CTA
constexpr int kDmM = 32;        // complex outputs per CTA
constexpr int kDmK = 32;        // input samples per stage
constexpr int kDmGroup = 128;   // threads of one K group: 8 x 16, each 2 lines x 2 outputs
constexpr int kDmGroups = 4;    // K groups per CTA (stages g, g+4, ...), summed at the end

// Each K group stages its x and W tiles through registers: the next stage's
// loads are issued before the current stage's products, so their latency
// hides behind the arithmetic.  The groups' partial sums are added in a fixed
// order, so the result does not depend on scheduling.
__global__ void __launch_bounds__(kDmGroup * kDmGroups) demod_kernel(
    const float *__restrict__ x, long long ncols, int n, const float2 *__restrict__ W, int M,
    float2 *__restrict__ iq, float *__restrict__ env) {
    __shared__ float xs[kDmGroups][kDmK][kDmC + 1];  // [k][line]: odd rows, no bank conflicts
    __shared__ __align__(16) float2 ws[kDmGroups][kDmK][kDmM];
    const int tid = threadIdx.x, grp = tid / kDmGroup, t = tid % kDmGroup;
    const int tx = t & 15, ty = t >> 4;
    const long long c0 = (long long)blockIdx.x * kDmC;
    const int m0 = blockIdx.y * kDmM;
    const int nst = (n + kDmK - 1) / kDmK;
    constexpr int XQ = kDmC * kDmK / kDmGroup;  // 4 x values per thread and stage
    constexpr int WQ = kDmK * kDmM / kDmGroup;  // 8 W values
    float xr[XQ];
    float2 wr[WQ];
    auto fetch = [&](int st) {
        const int k0 = st * kDmK;
#pragma unroll
        for (int q = 0; q < XQ; ++q) {
            const int e = t + kDmGroup * q, r = e / kDmK, kk = e % kDmK;
            const long long c = c0 + r;
            const int k = k0 + kk;
            xr[q] = (c < ncols && k < n) ? __ldg(x + c * n + k) : 0.f;
        }
#pragma unroll
        for (int q = 0; q < WQ; ++q) {
            const int e = t + kDmGroup * q, kk = e / kDmM, mm = e % kDmM;
            const int k = k0 + kk, m = m0 + mm;
            wr[q] = (k < n && m < M) ? __ldg(W + (long long)k * M + m) : make_float2(0.f, 0.f);
        }
    };
    auto group_sync = [&]() {  // named barrier of this group's 128 threads
        asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "r"(kDmGroup) : "memory");
    };
    float2 acc[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) acc[i][j] = make_float2(0.f, 0.f);

    int st = grp;
    if (st < nst) fetch(st);
    for (; st < nst; st += kDmGroups) {
#pragma unroll
        for (int q = 0; q < XQ; ++q) {
            const int e = t + kDmGroup * q;
            xs[grp][e % kDmK][e / kDmK] = xr[q];
        }
#pragma unroll
        for (int q = 0; q < WQ; ++q) {
            const int e = t + kDmGroup * q;
            ws[grp][e / kDmM][e % kDmM] = wr[q];
        }
        group_sync();
        if (st + kDmGroups < nst) fetch(st + kDmGroups);
#pragma unroll 8
        for (int kk = 0; kk < kDmK; ++kk) {
            const float a0 = xs[grp][kk][ty], a1 = xs[grp][kk][ty + 8];
            const float2 b0 = ws[grp][kk][tx], b1 = ws[grp][kk][tx + 16];
            acc[0][0].x = fmaf(a0, b0.x, acc[0][0].x);
            acc[0][0].y = fmaf(a0, b0.y, acc[0][0].y);
            acc[0][1].x = fmaf(a0, b1.x, acc[0][1].x);
            acc[0][1].y = fmaf(a0, b1.y, acc[0][1].y);
            acc[1][0].x = fmaf(a1, b0.x, acc[1][0].x);
            acc[1][0].y = fmaf(a1, b0.y, acc[1][0].y);
            acc[1][1].x = fmaf(a1, b1.x, acc[1][1].x);
            acc[1][1].y = fmaf(a1, b1.y, acc[1][1].y);
        }
        group_sync();
    }
    __syncthreads();
    // groups 1.. hand their partial sums to group 0 through their W tiles;
    // group 0 adds them in group order
    if (grp != 0) {
        float4 *red = reinterpret_cast<float4 *>(&ws[grp][0][0]);
        red[2 * t] = make_float4(acc[0][0].x, acc[0][0].y, acc[0][1].x, acc[0][1].y);
        red[2 * t + 1] = make_float4(acc[1][0].x, acc[1][0].y, acc[1][1].x, acc[1][1].y);
    }
    __syncthreads();
    if (grp != 0) return;
#pragma unroll
    for (int g = 1; g < kDmGroups; ++g) {
        const float4 *red = reinterpret_cast<const float4 *>(&ws[g][0][0]);
        const float4 r0 = red[2 * t], r1 = red[2 * t + 1];
        acc[0][0].x += r0.x;
        acc[0][0].y += r0.y;
        acc[0][1].x += r0.z;
        acc[0][1].y += r0.w;
        acc[1][0].x += r1.x;
        acc[1][0].y += r1.y;
        acc[1][1].x += r1.z;
        acc[1][1].y += r1.w;
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
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

// Counts a key (when valid) into the pass's histograms: rank 0's, and rank
// 1's once the two prefixes differ.  One shared-memory atomic per distinct
// bin of the warp (most keys of an image share their top byte, and 32 lanes
// adding to one bin one by one serialise).  Every lane of the warp calls it.
__device__ __forceinline__ void count_key(unsigned (*h)[256], unsigned key, bool valid, int pass,
                                          unsigned p0, unsigned p1, bool split) {
    const int shift = 24 - 8 * pass;
    const unsigned d = (key >> shift) & 255u;
    bool t0 = valid, t1 = false;
    if (pass > 0) {
        const int hi = shift + 8;  // 8..24
        t0 = valid && (key >> hi) == (p0 >> hi);
        t1 = valid && split && (key >> hi) == (p1 >> hi);
    }
    const int lane = threadIdx.x & 31;
    const unsigned m0 = __match_any_sync(0xffffffffu, t0 ? d : 0x100u);
    if (t0 && lane == __ffs(m0) - 1) atomicAdd(&h[0][d], (unsigned)__popc(m0));
    if (split) {  // uniform over the CTA
        const unsigned m1 = __match_any_sync(0xffffffffu, t1 ? d : 0x100u);
        if (t1 && lane == __ffs(m1) - 1) atomicAdd(&h[1][d], (unsigned)__popc(m1));
    }
}

// One warp: the bin holding rank k (0-based) of 256 counts, lane l holding
// bins 8l..8l+7 in c; k becomes the rank within that bin.
__device__ int warp_pick_counts(const unsigned (&c)[8], unsigned &k) {
    const int lane = threadIdx.x & 31;
    unsigned s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += c[i];
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
__device__ int warp_pick(const unsigned *h, unsigned &k) {
    const int lane = threadIdx.x & 31;
    unsigned c[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) c[i] = h[lane * 8 + i];
    return warp_pick_counts(c, k);
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
    const unsigned p0 = s_pre[0], p1 = s_pre[1];
    const bool split = s_split != 0;
    const float *vs = v + (long long)blockIdx.y * n;
    bool nan_seen = false;
    for (long long i0 = (long long)blockIdx.x * blockDim.x; i0 < n;
         i0 += (long long)gridDim.x * blockDim.x) {  // i0 uniform: whole warps in count_key
        const long long i = i0 + tid;
        const bool valid = i < n;
        const float val = valid ? __ldg(vs + i) : 0.f;
        nan_seen |= val != val;
        count_key(h, pct_key(val), valid, pass, p0, p1, split);
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

// Small segments: one CTA per segment runs the four radix
// passes with its histograms in shared memory (no workspace, no replays),
// writes the interpolated percentile to ref[seg] and, when out is given, the
// segment's log compression with it.  v and out may be the same array.
constexpr int kPctCta = 1024;
constexpr long long kPctCtaSmall = 8192;  // one CTA per segment up to this size

__global__ void __launch_bounds__(kPctCta) pct_cta_kernel(const float *v, long long n, unsigned k0,
                                                          unsigned k1, double gamma,
                                                          float *__restrict__ ref, float floor_add,
                                                          float *out) {
    __shared__ unsigned h[2][256];
    __shared__ unsigned s_pre[2], s_kr[2];
    __shared__ int s_nan;
    __shared__ float s_ref;
    const int tid = threadIdx.x;
    const long long base = (long long)blockIdx.x * n;
    const float *vs = v + base;
    if (tid == 0) {
        s_pre[0] = s_pre[1] = 0;
        s_kr[0] = k0;
        s_kr[1] = k1;
        s_nan = 0;
    }
    for (int pass = 0; pass < 4; ++pass) {
        if (tid < 512) h[tid >> 8][tid & 255] = 0;
        __syncthreads();
        const int shift = 24 - 8 * pass;
        const unsigned p0 = s_pre[0], p1 = s_pre[1];
        const bool split = p0 != p1;
        bool nan_seen = false;
        for (long long i0 = 0; i0 < n; i0 += kPctCta) {
            const long long i = i0 + tid;
            const bool valid = i < n;
            const float val = valid ? vs[i] : 0.f;
            nan_seen |= val != val;
            count_key(h, pct_key(val), valid, pass, p0, p1, split);
        }
        if (__syncthreads_or(nan_seen ? 1 : 0) && tid == 0) s_nan = 1;
        if (tid < 32) {
            unsigned kr0 = s_kr[0], kr1 = s_kr[1];
            const int b0 = warp_pick(h[0], kr0);
            const int b1 = warp_pick(split ? h[1] : h[0], kr1);
            if (tid == 0) {
                s_pre[0] = p0 | ((unsigned)b0 << shift);
                s_pre[1] = p1 | ((unsigned)b1 << shift);
                s_kr[0] = kr0;
                s_kr[1] = kr1;
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        float r;
        if (s_nan) {
            r = __int_as_float(0x7fc00000);
        } else {
            const double a = pct_value(s_pre[0]), b = pct_value(s_pre[1]);
            const double d = b - a;
            r = __double2float_rn((gamma >= 0.5) ? b - d * (1.0 - gamma) : a + d * gamma);
        }
        s_ref = r;
        ref[blockIdx.x] = r;
    }
    if (!out) return;
    __syncthreads();
    const float r = s_ref;
    for (long long i = tid; i < n; i += kPctCta)
        out[base + i] = 20.0f * log10f(__fadd_rn(__fdiv_rn(vs[i], r), floor_add));
}

// Segments of up to kCluMaxChunk * kClu values: a cluster of kClu CTAs per
// segment, each holding a slice in its shared memory for all four passes.
// After each CTA has counted its slice, every CTA sums the cluster's
// histograms through distributed shared memory (one warp per rank) and makes
// the same pick, so the passes need no global memory and no further
// launches; the log compression then runs from the resident slices.  Two
// cluster barriers per pass: one before the histograms are read, one before
// they are reset.
constexpr int kClu = 8;
constexpr int kCluThreads = 1024;
constexpr long long kCluMaxChunk = 52 * 1024;  // floats per CTA (208 KB)

__global__ void __cluster_dims__(kClu, 1, 1) __launch_bounds__(kCluThreads)
    pct_cluster_kernel(const float *v, long long n, unsigned k0, unsigned k1, double gamma,
                       float *__restrict__ ref, float floor_add, float *out) {
    extern __shared__ float sv[];
    __shared__ unsigned h[2][256];     // this slice's counts, read by the whole cluster
    __shared__ unsigned hsum[2][256];  // the cluster's counts
    __shared__ unsigned s_pre[2], s_kr[2];
    __shared__ int s_nan, s_nan_all;
    cg::cluster_group cl = cg::this_cluster();
    const int tid = threadIdx.x;
    const unsigned rank = cl.block_rank();
    const long long seg = blockIdx.x / kClu;
    const long long chunk = (n + kClu - 1) / kClu;
    const long long lo = (long long)rank * chunk;
    const int cnt = (int)max(0LL, min(n, lo + chunk) - lo);
    const long long base = seg * n + lo;
    bool nan_seen = false;
    for (int i = tid; i < cnt; i += kCluThreads) {
        const float x = v[base + i];
        sv[i] = x;
        nan_seen |= x != x;
    }
    const int any_nan = __syncthreads_or(nan_seen ? 1 : 0);
    if (tid == 0) {
        s_nan = any_nan;
        s_nan_all = 0;
        s_pre[0] = s_pre[1] = 0;
        s_kr[0] = k0;
        s_kr[1] = k1;
    }
    for (int pass = 0; pass < 4; ++pass) {
        if (tid < 512) {
            h[tid >> 8][tid & 255] = 0;
            hsum[tid >> 8][tid & 255] = 0;
        }
        __syncthreads();
        const int shift = 24 - 8 * pass;
        const unsigned p0 = s_pre[0], p1 = s_pre[1];
        const bool split = p0 != p1;
        for (int i0 = 0; i0 < cnt; i0 += kCluThreads) {
            const int i = i0 + tid;
            const bool valid = i < cnt;
            count_key(h, pct_key(valid ? sv[i] : 0.f), valid, pass, p0, p1, split);
        }
        cl.sync();  // every slice counted
        // warp r adds rank r's histograms into this CTA's sums (the remote
        // reads of the ranks in flight at once, one warp each)
        if (tid < 32 * kClu) {
            const int r = tid >> 5, lane = tid & 31;
            const unsigned *rh = cl.map_shared_rank(&h[0][0], (unsigned)r);
            unsigned c0[8], c1[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                c0[i] = rh[lane * 8 + i];
                c1[i] = split ? rh[256 + lane * 8 + i] : 0u;
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (c0[i]) atomicAdd(&hsum[0][lane * 8 + i], c0[i]);
                if (c1[i]) atomicAdd(&hsum[1][lane * 8 + i], c1[i]);
            }
            if (pass == 3 && lane == 0 && *cl.map_shared_rank(&s_nan, (unsigned)r)) s_nan_all = 1;
        }
        cl.sync();  // every CTA has read the histograms (and s_nan) before they change
        if (tid < 32) {
            unsigned c0[8], c1[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                c0[i] = hsum[0][tid * 8 + i];
                c1[i] = hsum[1][tid * 8 + i];
            }
            unsigned kr0 = s_kr[0], kr1 = s_kr[1];
            const int b0 = warp_pick_counts(c0, kr0);
            const int b1 = split ? warp_pick_counts(c1, kr1) : warp_pick_counts(c0, kr1);
            if (tid == 0) {
                s_pre[0] = p0 | ((unsigned)b0 << shift);
                s_pre[1] = p1 | ((unsigned)b1 << shift);
                s_kr[0] = kr0;
                s_kr[1] = kr1;
            }
        }
        __syncthreads();  // the pick is made before the sums are reset
    }
    float r;
    if (s_nan_all) {
        r = __int_as_float(0x7fc00000);
    } else {
        const double a = pct_value(s_pre[0]), b = pct_value(s_pre[1]);
        const double d = b - a;
        r = __double2float_rn((gamma >= 0.5) ? b - d * (1.0 - gamma) : a + d * gamma);
    }
    if (rank == 0 && tid == 0) ref[seg] = r;
    if (!out) return;
    for (int i = tid; i < cnt; i += kCluThreads)
        out[base + i] = 20.0f * log10f(__fadd_rn(__fdiv_rn(sv[i], r), floor_add));
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

// whether a cluster of kClu CTAs of the cluster kernel fits on this GPU
bool cluster_ok() {
    static const bool ok = [] {
        if (cudaFuncSetAttribute(pct_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(kCluMaxChunk * sizeof(float))) != cudaSuccess)
            return false;
        cudaLaunchConfig_t cfg = {};  // the cluster size is the kernel's compile-time one
        cfg.gridDim = dim3(kClu);
        cfg.blockDim = dim3(kCluThreads);
        cfg.dynamicSmemBytes = kCluMaxChunk * sizeof(float);
        int nclusters = 0;
        return cudaOccupancyMaxActiveClusters(&nclusters, pct_cluster_kernel, &cfg) == cudaSuccess &&
               nclusters > 0;
    }();
    return ok;
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
    demod_kernel<<<dim3((unsigned)gx, (unsigned)gy), kDmGroup * kDmGroups, 0, s>>>(x, ncols, n, W, M,
                                                                                iq, env);
    return cudaGetLastError();
}

size_t percentile_workspace_bytes(long long nseg) {
    return (size_t)nseg * kPctSegWords * sizeof(unsigned);
}

cudaError_t launch_percentile(const float *v, long long nseg, long long n, double q, float *out,
                              void *ws, cudaStream_t s, float floor_add, float *logout) {
    if (nseg == 0) return cudaSuccess;
    const double idx = (double)(n - 1) * (q / 100.0);
    const long long lo = (long long)floor(idx);
    const long long k0 = lo < 0 ? 0 : (lo > n - 1 ? n - 1 : lo);
    const long long k1 = k0 + 1 < n ? k0 + 1 : n - 1;
    const double gamma = idx - (double)lo;
    cudaError_t e;
    if (n <= kPctCtaSmall) {
        pct_cta_kernel<<<(unsigned)nseg, kPctCta, 0, s>>>(v, n, (unsigned)k0, (unsigned)k1, gamma, out,
                                                         floor_add, logout);
        return cudaGetLastError();
    }
    if (n <= kCluMaxChunk * kClu && cluster_ok()) {
        const long long chunk = (n + kClu - 1) / kClu;
        const int smem = (int)(chunk * sizeof(float));  // within the limit cluster_ok() set
        pct_cluster_kernel<<<(unsigned)(nseg * kClu), kCluThreads, smem, s>>>(
            v, n, (unsigned)k0, (unsigned)k1, gamma, out, floor_add, logout);
        return cudaGetLastError();
    }
    if ((e = cudaMemsetAsync(ws, 0, percentile_workspace_bytes(nseg), s)) != cudaSuccess) return e;
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
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return logout ? launch_log_compress(v, nseg, n, out, floor_add, logout, s) : cudaSuccess;
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

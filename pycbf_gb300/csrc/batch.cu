// Uneven batches in one persistent launch (no reference counterpart).
//
// A batch is a list of jobs, each one frame of one beamformer (Tabbed or
// Synthetic, any ntx / nrx / nt / pixel count, float32 / float16 / bfloat16
// channel data), cubic interpolation, summed over transmits and receives.
// The work items are (job, run of tiles_per_item tiles of kBlock pixels) in
// an order the host chooses (largest first, or job order); a grid of `ctas`
// CTAs takes them from a queue head in global memory until it runs dry, so
// frames of very different cost share the GPU without a launch per frame.
//
// Two per-pixel forms, which the autotuner chooses between: the transmits
// taken TXC at a time into registers (TXC 4, 8 or 12; for each chunk every
// receive adds its chunk sum to the pixel's accumulator, so with one chunk,
// ntx <= TXC, the images are bitwise the single-frame ones), or (tx_chunk 0)
// the single-frame kernel's own body, bitwise the same for every ntx.
#include "das_impl.cuh"

namespace pgb {

namespace {

template <int GEOM, typename T, int TXC>
__device__ __forceinline__ void batch_tile(const DasArgs &a, long long tile) {
    using K = Kind<PYCBF_GB_INTERP_CUBIC, T>;
    constexpr int G = (TXC < kGroup) ? TXC : kGroup;  // taps whose gathers are in flight together
    const long long i = tile * kBlock + threadIdx.x;
    if (i >= a.np) return;
    const long long np = a.np;
    const int ntx = a.ntx, nrx = a.nrx;
    const long long op = a.pixel_index ? (long long)__ldg(a.pixel_index + i) : i;
    const long long chs = (long long)nrx * a.nt;
    float pnt[3] = {0.f, 0.f, 0.f};
    if (GEOM == GEOM_SYNTH)
        for (int k = 0; k < 3; ++k) if (k < a.ndim) pnt[k] = __ldg(a.geo.pnts + i * a.ndim + k);

    float acc = 0.f;
    for (int t0 = 0; t0 < ntx; t0 += TXC) {
        float rtau[TXC], rapod[TXC];
        float amax = 0.f;
#pragma unroll
        for (int k = 0; k < TXC; ++k) {
            rtau[k] = 0.f;
            rapod[k] = 0.f;
            const int t = t0 + k;
            if (t < ntx) {
                if (GEOM == GEOM_TABBED) {
                    rtau[k] = __ldg(a.tautx + (long long)t * np + i);
                    rapod[k] = __ldg(a.apodtx + (long long)t * np + i);
                    amax = fmaxf(amax, fabsf(rapod[k]));
                } else {
                    rtau[k] = synth_tx_delay(a, t, pnt);
                    rapod[k] = 1.f;
                }
            }
        }
        const int nk_chunk = min(TXC, ntx - t0);
        float bacc = 0.f;  // blocks of kRxBlockSum receives, as the other kernels sum
        for (int r = 0; r < nrx; ++r) {
            if (r > 0 && r % kRxBlockSum == 0) {
                acc += bacc;
                bacc = 0.f;
            }
            float trx, arx;
            bool live;
            if (GEOM == GEOM_TABBED) {
                trx = __ldg(a.taurx + (long long)r * np + i);
                arx = __ldg(a.apodrx + (long long)r * np + i);
                live = __fmul_rn(amax, fabsf(arx)) >= a.thresh;
            } else {
                trx = synth_rx_delay(a, r, pnt);
                arx = 1.f;
                live = trx != __int_as_float(0x7f800000);
            }
            if (!live) continue;
            const long long ch0 = ((long long)t0 * nrx + r) * a.nt;
            float accr = 0.f;
#pragma unroll
            for (int g = 0; g < TXC; g += G) {
                if (g >= nk_chunk) break;
                const int nk = min(G, nk_chunk - g);
                float xs[G], ap[G];
                int ix[G];
                unsigned hit = 0u, fix = 0u;
#pragma unroll
                for (int k = 0; k < G; ++k) {
                    xs[k] = 0.f;
                    ap[k] = 0.f;
                    ix[k] = 0;
                    if (k < nk) {
                        const float x = __fadd_rn(rtau[g + k], trx);
                        float apod = 1.f;
                        bool h = true;
                        if (GEOM == GEOM_TABBED) {
                            apod = __fmul_rn(rapod[g + k], arx);
                            h = fabsf(apod) >= a.thresh;
                        }
                        bool fx;
                        int idx;
                        const bool inr = K::index(x, a, idx, fx);
                        xs[k] = x;
                        ap[k] = apod;
                        ix[k] = idx;
                        hit |= (unsigned)(h && inr) << k;
                        fix |= (unsigned)(h && fx) << k;
                    }
                }
                if (fix) {
#pragma unroll
                    for (int k = 0; k < G; ++k) {
                        if ((fix >> k) & 1u) {
                            int idx;
                            const bool inr = K::index_exact(xs[k], a, idx);
                            ix[k] = idx;
                            hit = inr ? (hit | (1u << k)) : (hit & ~(1u << k));
                        }
                    }
                }
                typename K::P pv[G];
#pragma unroll
                for (int k = 0; k < G; ++k)
                    if ((hit >> k) & 1u) pv[k] = K::load(a.data, ch0 + (long long)(g + k) * chs, ix[k], a);
#pragma unroll
                for (int k = 0; k < G; ++k)
                    if ((hit >> k) & 1u)
                        accr = fmaf(ap[k], K::value(pv[k], xs[k], (float)ix[k], a), accr);
            }
            bacc += accr;
        }
        acc += bacc;
    }
    a.out[op] = acc;
}

template <int TXC>
__global__ void __launch_bounds__(kBlock, 4)
batch_das_kernel(const BatchJob *__restrict__ jobs, const int2 *__restrict__ items,
                 long long nitems, int tiles_per_item, unsigned long long *counter) {
    __shared__ __align__(16) BatchJob s_job;
    __shared__ long long s_k;
    constexpr int kWords = (int)(sizeof(BatchJob) / sizeof(int));
    for (;;) {
        if (threadIdx.x == 0) s_k = (long long)atomicAdd(counter, 1ULL);
        __syncthreads();
        const long long k = s_k;
        if (k >= nitems) break;
        const int2 it = __ldg(items + k);
        const int *src = reinterpret_cast<const int *>(jobs + it.x);
        int *dst = reinterpret_cast<int *>(&s_job);
        for (int w = threadIdx.x; w < kWords; w += blockDim.x) dst[w] = __ldg(src + w);
        __syncthreads();
        const int geom = s_job.geom, dtype = s_job.dtype;
        for (int sub = 0; sub < tiles_per_item; ++sub) {
            const long long tile = (long long)it.y * tiles_per_item + sub;
            if (geom == GEOM_TABBED) {
                if (dtype == PYCBF_GB_F32) batch_tile<GEOM_TABBED, float, TXC>(s_job.a, tile);
                else if (dtype == PYCBF_GB_F16) batch_tile<GEOM_TABBED, __half, TXC>(s_job.a, tile);
                else batch_tile<GEOM_TABBED, __nv_bfloat16, TXC>(s_job.a, tile);
            } else {
                if (dtype == PYCBF_GB_F32) batch_tile<GEOM_SYNTH, float, TXC>(s_job.a, tile);
                else if (dtype == PYCBF_GB_F16) batch_tile<GEOM_SYNTH, __half, TXC>(s_job.a, tile);
                else batch_tile<GEOM_SYNTH, __nv_bfloat16, TXC>(s_job.a, tile);
            }
        }
        __syncthreads();  // every thread is done with s_job and s_k
    }
}

// The same queue, each pixel run by the single-frame kernel's body
// (das_pixel): transmits in registers up to kTxReg, in the thread's column of
// shared memory beyond, every receive's delay and reject computed once.  The
// images are bitwise those of the single-frame calls for every ntx.
__global__ void __launch_bounds__(kBlock, 4)
batch_das_full_kernel(const BatchJob *__restrict__ jobs, const int2 *__restrict__ items,
                      long long nitems, int tiles_per_item, unsigned long long *counter) {
    extern __shared__ float sm[];
    __shared__ __align__(16) BatchJob s_job;
    __shared__ long long s_k;
    constexpr int kWords = (int)(sizeof(BatchJob) / sizeof(int));
    constexpr int CUB = PYCBF_GB_INTERP_CUBIC, SUM = PYCBF_GB_SUM_TX_AND_RX;
    for (;;) {
        if (threadIdx.x == 0) s_k = (long long)atomicAdd(counter, 1ULL);
        __syncthreads();
        const long long k = s_k;
        if (k >= nitems) break;
        const int2 it = __ldg(items + k);
        const int *src = reinterpret_cast<const int *>(jobs + it.x);
        int *dst = reinterpret_cast<int *>(&s_job);
        for (int w = threadIdx.x; w < kWords; w += blockDim.x) dst[w] = __ldg(src + w);
        __syncthreads();
        const int geom = s_job.geom, dtype = s_job.dtype;
        for (int sub = 0; sub < tiles_per_item; ++sub) {
            const long long i = ((long long)it.y * tiles_per_item + sub) * kBlock + threadIdx.x;
            if (geom == GEOM_TABBED) {
                if (dtype == PYCBF_GB_F32) das_pixel<GEOM_TABBED, CUB, SUM, float, false>(s_job.a, i, 0, sm);
                else if (dtype == PYCBF_GB_F16) das_pixel<GEOM_TABBED, CUB, SUM, __half, false>(s_job.a, i, 0, sm);
                else das_pixel<GEOM_TABBED, CUB, SUM, __nv_bfloat16, false>(s_job.a, i, 0, sm);
            } else {
                if (dtype == PYCBF_GB_F32) das_pixel<GEOM_SYNTH, CUB, SUM, float, false>(s_job.a, i, 0, sm);
                else if (dtype == PYCBF_GB_F16) das_pixel<GEOM_SYNTH, CUB, SUM, __half, false>(s_job.a, i, 0, sm);
                else das_pixel<GEOM_SYNTH, CUB, SUM, __nv_bfloat16, false>(s_job.a, i, 0, sm);
            }
        }
        __syncthreads();  // every thread is done with s_job and s_k
    }
}

// The same for a batch of one storage type T: each pixel runs the single-frame
// kernels' cubic body in its shared-memory column form, whatever the job's
// ntx (the column is sized for the batch's largest ntx; per-receive sums are
// sequential over transmits either way, so the images are those of the
// single-frame calls bit for bit).  The kernel carries the paths of one
// storage type only -- the mixed kernel above spills -- and each geometry's
// body sits behind a call of its own, so the compiler allocates its registers
// apart from the other's (one call per pixel, not per tap).  A CTA copies a
// job's descriptor only when its next item belongs to another job.  Measured
// on the 64-frame batch: with the register form as well for ntx <= 12 the
// float32 kernel took 43 ms, without it 38 ms.
template <int GEOM, typename T>
__device__ __noinline__ void batch_pixel(const DasArgs &a, long long i, float *sm) {
    das_pixel<GEOM, PYCBF_GB_INTERP_CUBIC, PYCBF_GB_SUM_TX_AND_RX, T, false, kTxSmem>(a, i, 0, sm);
}

// five CTAs per SM for 16-bit records (42 against 43 ms), four for float32
// records, whose body spills under five's register cap (47 against 38 ms)
template <typename T>
__global__ void __launch_bounds__(kBlock, CoefRec<T>::kPoly ? 4 : 5)
batch_das_typed_kernel(const BatchJob *__restrict__ jobs, const int2 *__restrict__ items,
                       long long nitems, int tiles_per_item, unsigned long long *counter) {
    extern __shared__ float sm[];
    __shared__ __align__(16) BatchJob s_job;
    __shared__ long long s_k;
    constexpr int kWords = (int)(sizeof(BatchJob) / sizeof(int));
    int cur = -1;  // the job whose descriptor s_job holds
    for (;;) {
        if (threadIdx.x == 0) s_k = (long long)atomicAdd(counter, 1ULL);
        __syncthreads();
        const long long k = s_k;
        if (k >= nitems) break;
        const int2 it = __ldg(items + k);
        if (it.x != cur) {  // the same in every thread: the barrier below is uniform
            const int *src = reinterpret_cast<const int *>(jobs + it.x);
            int *dst = reinterpret_cast<int *>(&s_job);
            for (int w = threadIdx.x; w < kWords; w += blockDim.x) dst[w] = __ldg(src + w);
            __syncthreads();
            cur = it.x;
        }
        const bool tabbed = s_job.geom == GEOM_TABBED;
        for (int sub = 0; sub < tiles_per_item; ++sub) {
            const long long i = ((long long)it.y * tiles_per_item + sub) * kBlock + threadIdx.x;
            if (tabbed) batch_pixel<GEOM_TABBED, T>(s_job.a, i, sm);
            else batch_pixel<GEOM_SYNTH, T>(s_job.a, i, sm);
        }
        __syncthreads();  // every thread is done with s_k (and, before a new job, s_job)
    }
}

}  // namespace

// the column of every job's transmit delays (the typed kernel uses the column
// form for every ntx, so this holds even when max_ntx <= kTxReg)
size_t batch_full_smem_bytes(int max_ntx) {
    return (size_t)std::max(max_ntx, 1) * kBlock * sizeof(float);
}

cudaError_t prepare_batch_das(int max_ntx) {
    const size_t smem = batch_full_smem_bytes(max_ntx);
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    const int lim = (int)std::max<size_t>(smem, 48 * 1024);
    cudaError_t err =
        cudaFuncSetAttribute(batch_das_full_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(batch_das_typed_kernel<float>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(batch_das_typed_kernel<__half>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(batch_das_typed_kernel<__nv_bfloat16>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    return err;
}

cudaError_t launch_batch_das(const BatchJob *jobs, const int2 *items, long long nitems,
                             int tiles_per_item, unsigned long long *counter, int tx_chunk,
                             int ctas, cudaStream_t s, int max_ntx, int dtypes) {
    cudaError_t err = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    if (err != cudaSuccess) return err;
    if (nitems <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)std::max(1, ctas);
    if (tx_chunk == 0) {  // shared-memory size set by prepare_batch_das, outside any capture
        const size_t smem = batch_full_smem_bytes(max_ntx);
        if (dtypes == 1 << PYCBF_GB_F32)
            batch_das_typed_kernel<float><<<grid, kBlock, smem, s>>>(jobs, items, nitems,
                                                                     tiles_per_item, counter);
        else if (dtypes == 1 << PYCBF_GB_F16)
            batch_das_typed_kernel<__half><<<grid, kBlock, smem, s>>>(jobs, items, nitems,
                                                                      tiles_per_item, counter);
        else if (dtypes == 1 << PYCBF_GB_BF16)
            batch_das_typed_kernel<__nv_bfloat16><<<grid, kBlock, smem, s>>>(
                jobs, items, nitems, tiles_per_item, counter);
        else
            batch_das_full_kernel<<<grid, kBlock, smem, s>>>(jobs, items, nitems, tiles_per_item,
                                                             counter);
        return cudaGetLastError();
    }
    switch (tx_chunk) {
        case 4: batch_das_kernel<4><<<grid, kBlock, 0, s>>>(jobs, items, nitems, tiles_per_item, counter); break;
        case 8: batch_das_kernel<8><<<grid, kBlock, 0, s>>>(jobs, items, nitems, tiles_per_item, counter); break;
        case 12: batch_das_kernel<12><<<grid, kBlock, 0, s>>>(jobs, items, nitems, tiles_per_item, counter); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace pgb

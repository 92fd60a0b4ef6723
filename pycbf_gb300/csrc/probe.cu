// FP32 throughput probe: the denominator of the FP32 roofline that the
// benchmark reports beside the HBM one.  Each thread runs `iters` rounds of
// eight independent FMAs; the result is stored so nothing is eliminated.
#include "common.cuh"

namespace {

__global__ void __launch_bounds__(256) fma_probe_kernel(float *out, int iters, float seed) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-3f + k;
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int pycbf_gb_fp32_probe(float *out, int blocks, int iters, void *stream) {
    if (!out || blocks <= 0 || iters <= 0) return PYCBF_GB_EINVAL;
    fma_probe_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(out, iters, 1.0f);
    return cudaGetLastError() == cudaSuccess ? PYCBF_GB_OK : PYCBF_GB_ECUDA;
}

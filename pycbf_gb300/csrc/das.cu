// Dispatch of the delay-and-sum kernels by geometry and channel-data type.
#include "das_staged.cuh"

namespace pgb {

cudaError_t launch_das_tabbed_f32(const DasArgs &, int, int, bool, cudaStream_t);
cudaError_t launch_das_tabbed_f16(const DasArgs &, int, int, bool, cudaStream_t);
cudaError_t launch_das_tabbed_bf16(const DasArgs &, int, int, bool, cudaStream_t);
cudaError_t launch_das_synth_f32(const DasArgs &, int, int, bool, cudaStream_t);
cudaError_t launch_das_synth_f16(const DasArgs &, int, int, bool, cudaStream_t);
cudaError_t launch_das_synth_bf16(const DasArgs &, int, int, bool, cudaStream_t);
cudaError_t launch_plan_f32(const DasArgs &, int, int *, cudaStream_t);
cudaError_t launch_plan_f16(const DasArgs &, int, int *, cudaStream_t);
cudaError_t launch_plan_bf16(const DasArgs &, int, int *, cudaStream_t);
cudaError_t launch_staged_f32(const DasArgs &, int, int, const int *, int *, cudaStream_t);
cudaError_t launch_staged_f16(const DasArgs &, int, int, const int *, int *, cudaStream_t);
cudaError_t launch_staged_bf16(const DasArgs &, int, int, const int *, int *, cudaStream_t);
cudaError_t launch_staged_adj_f32(const DasArgs &, int, const int *, cudaStream_t);

long long tabbed_plan_words(long long np, int ntx, int nrx) {
    return plan_layout(np, ntx, nrx).total;
}

cudaError_t launch_tabbed_plan(const DasArgs &a, int interp, int dtype, int *plan, cudaStream_t s) {
    switch (dtype) {
        case PYCBF_GB_F32: return launch_plan_f32(a, interp, plan, s);
        case PYCBF_GB_F16: return launch_plan_f16(a, interp, plan, s);
        case PYCBF_GB_BF16: return launch_plan_bf16(a, interp, plan, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_das_staged(const DasArgs &a, int interp, int sumtype, int dtype, const int *plan,
                              int *status, cudaStream_t s) {
    switch (dtype) {
        case PYCBF_GB_F32: return launch_staged_f32(a, interp, sumtype, plan, status, s);
        case PYCBF_GB_F16: return launch_staged_f16(a, interp, sumtype, plan, status, s);
        case PYCBF_GB_BF16: return launch_staged_bf16(a, interp, sumtype, plan, status, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_das(const DasArgs &a, int geom, int interp, int sumtype, int dtype, bool census,
                       cudaStream_t s) {
    if (geom == GEOM_TABBED) {
        switch (dtype) {
            case PYCBF_GB_F32: return launch_das_tabbed_f32(a, interp, sumtype, census, s);
            case PYCBF_GB_F16: return launch_das_tabbed_f16(a, interp, sumtype, census, s);
            case PYCBF_GB_BF16: return launch_das_tabbed_bf16(a, interp, sumtype, census, s);
        }
    } else {
        switch (dtype) {
            case PYCBF_GB_F32: return launch_das_synth_f32(a, interp, sumtype, census, s);
            case PYCBF_GB_F16: return launch_das_synth_f16(a, interp, sumtype, census, s);
            case PYCBF_GB_BF16: return launch_das_synth_bf16(a, interp, sumtype, census, s);
        }
    }
    return cudaErrorInvalidValue;
}

// receive masks of a synthetic geometry: mask[r, i] = 1 where receive r accepts pixel i
__global__ void synth_rx_mask_kernel(const __grid_constant__ DasArgs a, unsigned char *mask) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.np) return;
    float pnt[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < 3; ++k) if (k < a.ndim) pnt[k] = __ldg(a.geo.pnts + i * a.ndim + k);
    for (int r = 0; r < a.nrx; ++r)
        mask[(long long)r * a.np + i] = isinf(synth_rx_delay(a, r, pnt)) ? 0 : 1;
}

cudaError_t launch_synth_rx_mask(const DasArgs &a, unsigned char *mask, cudaStream_t s) {
    const long long bx = (a.np + 255) / 256;
    synth_rx_mask_kernel<<<(unsigned)bx, 256, 0, s>>>(a, mask);
    return cudaGetLastError();
}

cudaError_t launch_das_staged_adj(const DasArgs &a, int sumtype, int dtype, const int *plan,
                                  cudaStream_t s) {
    if (dtype != PYCBF_GB_F32) return cudaErrorInvalidValue;  // float32 records (F32, I16 data)
    return launch_staged_adj_f32(a, sumtype, plan, s);
}

}  // namespace pgb

// Cubic upsampling of channel data for nearest-neighbour beamforming with
// usf > 1 (the upsampling inside beamform_nearest, pycbf/cpu/pycbf.c:223-253).
//
// Sample it of the upsampled channel is the natural cubic spline of the
// channel at t = t0 + it * fl(dt / usf) (two roundings, as the reference
// builds its time vector at :239), with the reference's knot and range rules
// (cubic1D_fixed, pycbf.c:14-56): outside [t0, t0 + dt (nt-1)] the fill 0.
// The spline records come from the prefilter; one thread per output sample.
#include "das_impl.cuh"

namespace pgb {

namespace {

template <typename T>
__global__ void upsample_kernel(const __grid_constant__ DasArgs a, float *__restrict__ out,
                                long long nch, int ntu, float dtu) {
    using K = Kind<PYCBF_GB_INTERP_CUBIC, T>;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nch * (long long)ntu) return;
    const long long ch = n / ntu;
    const int it = (int)(n - ch * ntu);
    const float x = __fadd_rn(a.t0, __fmul_rn((float)it, dtu));
    int idx;
    bool fix;
    bool inr = K::index(x, a, idx, fix);
    if (fix) inr = K::index_exact(x, a, idx);
    float v = 0.f;
    if (inr) v = K::value(K::load(a.data, ch * (long long)a.nt, idx, a), x, (float)idx, a);
    out[n] = v;
}

}  // namespace

cudaError_t launch_upsample(const DasArgs &a, int dtype, float *out, long long nch, int ntu,
                            float dtu, cudaStream_t s) {
    const long long total = nch * (long long)ntu;
    const long long blocks = (total + 255) / 256;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    switch (dtype) {
        case PYCBF_GB_F32: upsample_kernel<float><<<(unsigned)blocks, 256, 0, s>>>(a, out, nch, ntu, dtu); break;
        case PYCBF_GB_F16: upsample_kernel<__half><<<(unsigned)blocks, 256, 0, s>>>(a, out, nch, ntu, dtu); break;
        case PYCBF_GB_BF16: upsample_kernel<__nv_bfloat16><<<(unsigned)blocks, 256, 0, s>>>(a, out, nch, ntu, dtu); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace pgb

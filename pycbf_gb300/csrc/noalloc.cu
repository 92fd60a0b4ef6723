// Cubic Tabbed delay-and-sum for callers that cannot allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc: a language runtime that
// reaches it only through a C FFI and owns no CUDA allocator, a service whose
// device-memory budget is fixed when it starts, or a caller that must not
// trigger the implicit synchronisation an allocation can cause.  They still
// own their inputs and outputs, but not the workspace for the spline
// coefficients that pycbf_gb_das_tabbed asks for.  This entry point keeps
// that workspace in a file-scope device array instead:
//
//   - the array has a fixed size, PYCBF_GB_NOALLOC_SCRATCH_BYTES (64 MiB), and
//     every GPU that loads this library holds it until the process exits;
//   - the first call on a device looks up the array's device address for that
//     device (cudaGetSymbolAddress, with the device current) and remembers it,
//     so that first call should come before any stream capture; the
//     remembered address assumes the device is not reset
//     (cudaDeviceReset) while the library stays loaded;
//   - every call shares the array and leaves the last call's coefficients in
//     it; nothing in it needs to start at zero (the prefilter overwrites every
//     coefficient it later reads), but calls whose work overlaps on the GPU --
//     on two streams, or from two host threads -- race on it;
//   - every argument is checked before any work is queued: channel data whose
//     coefficients exceed the array are rejected with PYCBF_GB_ERANGE, and the
//     delay-and-sum's own checks (pointers, sizes, sum type, threshold) run
//     first too, so a rejected call leaves the array untouched; np == 0 is a
//     successful call that queues nothing.
//
// The work itself is the existing prefilter and cubic delay-and-sum entry
// points, pointed at the array; nothing here calls cudaMalloc, cudaFree or an
// allocating library routine.
#include <mutex>

#include "common.cuh"

namespace {

constexpr size_t kScratchBytes = PYCBF_GB_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 256;
std::mutex g_scratch_mutex;
void *g_scratch_ptr[kMaxDevices] = {};

// A non-null, 16-byte aligned placeholder for the argument checks (never
// dereferenced: the host-side name of a device array is not its address).
const void *placeholder_coef() { return reinterpret_cast<const void *>(256); }

// Device address of the array on the current device (looked up once per device).
int scratch_address(void **out) {
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return PYCBF_GB_ECUDA;
    if (dev < 0 || dev >= kMaxDevices) return PYCBF_GB_ERANGE;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (err != cudaSuccess || !p) return PYCBF_GB_ECUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return PYCBF_GB_OK;
}

}  // namespace

extern "C" int pycbf_gb_das_tabbed_cubic_noalloc(const pycbf_gb_rfinfo *rf, const void *rfdata,
                                                 const float *tautx, const float *apodtx,
                                                 const float *taurx, const float *apodrx,
                                                 long long np, const int *pixel_index,
                                                 float thresh, int sumtype, float *out,
                                                 void *stream) {
    if (!rf) return PYCBF_GB_EINVAL;
    if (!rfdata) return PYCBF_GB_EINVAL;
    // the delay-and-sum's checks, with the (16-byte aligned) array standing in for
    // the coefficients it will read
    int st = pgb::check_tabbed_prefiltered(rf, placeholder_coef(), tautx, apodtx, taurx,
                                           apodrx, np, thresh, sumtype, out);
    if (st) return st;
    const size_t need = pycbf_gb_workspace_bytes(rf, PYCBF_GB_INTERP_CUBIC);
    if (need > kScratchBytes) return PYCBF_GB_ERANGE;
    if (np == 0) return PYCBF_GB_OK;
    void *scratch = nullptr;
    st = scratch_address(&scratch);
    if (st) return st;
    st = pycbf_gb_spline_coefficients(rf, rfdata, scratch, kScratchBytes, stream);
    if (st) return st;
    return pycbf_gb_das_tabbed_prefiltered(rf, scratch, tautx, apodtx, taurx, apodrx, np,
                                           pixel_index, thresh, sumtype, nullptr, out, stream);
}

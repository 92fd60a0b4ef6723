// The C ABI (include/pycbf_gb300.h): host-side validation, then stream-ordered
// launches.  No allocation, no synchronisation, no mutable shared state.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

#include "common.cuh"

using namespace pgb;

namespace {

thread_local int g_last_cuda_error = 0;

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return PYCBF_GB_OK;
    g_last_cuda_error = (int)e;
    return PYCBF_GB_ECUDA;
}

size_t dtype_bytes(int dtype) {
    switch (dtype) {
        case PYCBF_GB_F32: return 4;
        case PYCBF_GB_F16:
        case PYCBF_GB_BF16:
        case PYCBF_GB_I16: return 2;
        default: return 0;
    }
}

// Largest sample count the nearest-neighbour rounding handles exactly in float.
constexpr int kMaxNt = 1 << 22;
constexpr int kMaxNtSpline = 18000;  // two shared-memory copies of a channel per warp (144 KB)

// i16_ok: the entry point converts int16 channel data itself (or reads none)
int check_rf(const pycbf_gb_rfinfo *rf, bool synthetic, bool i16_ok = false) {
    if (!rf) return PYCBF_GB_EINVAL;
    if (rf->ntx <= 0 || rf->nrx <= 0 || rf->nt <= 0 || rf->nframes <= 0) return PYCBF_GB_EINVAL;
    if (!dtype_bytes(rf->dtype)) return PYCBF_GB_EINVAL;
    if (rf->dtype == PYCBF_GB_I16 && !i16_ok) return PYCBF_GB_EUNSUPPORTED;
    if (!std::isfinite(rf->t0) || !std::isfinite(rf->dt) || !(rf->dt > 0.f)) return PYCBF_GB_EINVAL;
    if (synthetic && rf->ndim != 2 && rf->ndim != 3) return PYCBF_GB_EINVAL;
    if (rf->ntx > (1 << 20) || rf->nrx > (1 << 20) || rf->nt >= kMaxNt || rf->nframes > 65535)
        return PYCBF_GB_ERANGE;
    return PYCBF_GB_OK;
}

// 4 ulp of the largest quotient magnitude that can still be in range: the
// fast reciprocal quotient is within 1.5 ulp of the correctly rounded one.
float boundary_eps(int nt) {
    int k = 0;
    while ((1LL << k) < (long long)nt + 2) ++k;
    return std::ldexp(1.0f, k - 22);
}

void fill_time_axis(DasArgs &a, const pycbf_gb_rfinfo *rf) {
    a.ntx = (int)rf->ntx;
    a.nrx = (int)rf->nrx;
    a.nt = rf->nt;
    a.nframes = (int)rf->nframes;
    a.t0 = rf->t0;
    a.dt = rf->dt;
    a.inv_dt = 1.0f / rf->dt;
    // xmax = t0 + dt*(nt-1), two roundings as in pycbf.c:77
    volatile float span = rf->dt * (float)(rf->nt - 1);
    a.xmax = rf->t0 + span;
    // x0 + dx*nx of the reference linear_interp (__engines__.cu:47), two roundings
    volatile float span2 = rf->dt * (float)rf->nt;
    a.xend = rf->t0 + span2;
    a.eps = boundary_eps(rf->nt);
    {
        int k = 0;
        while ((1LL << k) < (long long)rf->nt) ++k;
        a.eps_fast = std::ldexp(1.25f * 1.5f, k - 23);
    }
    // the last knot as NVRTC compiles x0 + dx*(nx-1) in the reference's CUDA kernels
    a.xfma = std::fmaf(rf->dt, (float)(rf->nt - 1), rf->t0);
}

bool das_shape_ok(int geom, int sumtype, long long ntx) {
    if (ntx <= 16) return true;
    (void)geom;
    const size_t per = 1 + (sumtype == PYCBF_GB_SUM_RX_ONLY ? 1 : 0);  // das_smem_bytes
    return per * (size_t)ntx * 128 * sizeof(float) <= 227 * 1024;
}

}  // namespace

// The argument checks of pycbf_gb_das_tabbed_prefiltered, in its order (also
// run up front by the allocation-free entry point, before it queues any work).
// coef may be a placeholder here: only its alignment is checked.
int pgb::check_tabbed_prefiltered(const pycbf_gb_rfinfo *rf, const void *coef, const float *tautx,
                                  const float *apodtx, const float *taurx, const float *apodrx,
                                  long long np, float thresh, int sumtype, const float *out) {
    int st = check_rf(rf, false, true);
    if (st) return st;
    if (!coef || !tautx || !apodtx || !taurx || !apodrx || !out) return PYCBF_GB_EINVAL;
    if (reinterpret_cast<uintptr_t>(coef) % 16) return PYCBF_GB_EINVAL;
    if (np < 0 || np >= (1LL << 31)) return PYCBF_GB_ERANGE;
    if (np == 0) return PYCBF_GB_OK;
    if (sumtype < 0 || sumtype > 5 || std::isnan(thresh)) return PYCBF_GB_EINVAL;
    if (!das_shape_ok(GEOM_TABBED, sumtype, rf->ntx)) return PYCBF_GB_ERANGE;
    return PYCBF_GB_OK;
}

namespace {

// The TMA-staged kernel covers ntx <= 12 with the sums over transmits per
// receive; its 16-byte bulk copies need channel strides and the data base
// aligned to 16 bytes.
bool staged_ok(const pycbf_gb_rfinfo *rf, int interp, int sumtype, const void *data) {
    if (rf->ntx > 12 || rf->nrx > 4096 || interp > PYCBF_GB_INTERP_CUBIC) return false;
    if (sumtype != PYCBF_GB_SUM_TX_ONLY && sumtype != PYCBF_GB_SUM_TX_AND_RX &&
        sumtype != PYCBF_GB_SUM_DMAS_SSR && sumtype != PYCBF_GB_SUM_DMAS_POWER)
        return false;
    const size_t elem = interp == PYCBF_GB_INTERP_CUBIC ? (rf->dtype == PYCBF_GB_F32 ? 16 : 8)
                                                        : dtype_bytes(rf->dtype);
    return ((size_t)rf->nt * elem) % 16 == 0 && reinterpret_cast<uintptr_t>(data) % 16 == 0;
}

int launch_tabbed(const pycbf_gb_rfinfo *rf, DasArgs &a, int interp, int sumtype, const void *plan,
                  cudaStream_t s) {
    if (plan && staged_ok(rf, interp, sumtype, a.data)) {
        if (sumtype == PYCBF_GB_SUM_TX_ONLY) {  // rows of receives no pixel of a tile uses stay 0
            const size_t bytes = sizeof(float) * (size_t)rf->nframes * rf->nrx * (size_t)a.np;
            int st = cuda_status(cudaMemsetAsync(a.out, 0, bytes, s));
            if (st) return st;
        }
        int *pl = static_cast<int *>(const_cast<void *>(plan));
        return cuda_status(launch_das_staged(a, interp, sumtype, rf->dtype, pl, pl, s));
    }
    return cuda_status(launch_das(a, GEOM_TABBED, interp, sumtype, rf->dtype, false, s));
}

// The data the delay-and-sum gathers from, and its rfinfo (eff): the spline
// records for cubic, the channels themselves for nearest/linear.  int16
// channels come out as float32: converted inside the prefilter for cubic,
// by one conversion pass into the workspace otherwise.
int prepare_data(const pycbf_gb_rfinfo *rf, const void *rfdata, int interp, void *workspace,
                 size_t workspace_bytes, cudaStream_t s, const void **data,
                 pycbf_gb_rfinfo *eff) {
    *eff = *rf;
    if (rf->dtype == PYCBF_GB_I16) eff->dtype = PYCBF_GB_F32;
    if (interp != PYCBF_GB_INTERP_CUBIC) {
        if (rf->dtype != PYCBF_GB_I16) {
            *data = rfdata;
            return PYCBF_GB_OK;
        }
        const size_t need = pycbf_gb_workspace_bytes(rf, interp);
        if (!workspace || workspace_bytes < need) return PYCBF_GB_EWORKSPACE;
        if (reinterpret_cast<uintptr_t>(workspace) % 16) return PYCBF_GB_EINVAL;
        const long long n = rf->nframes * rf->ntx * rf->nrx * (long long)rf->nt;
        int st = cuda_status(launch_convert_i16(static_cast<const short *>(rfdata), n,
                                                static_cast<float *>(workspace), s));
        if (st) return st;
        *data = workspace;
        return PYCBF_GB_OK;
    }
    const size_t need = pycbf_gb_workspace_bytes(rf, interp);
    if (!workspace || workspace_bytes < need) return PYCBF_GB_EWORKSPACE;
    if (reinterpret_cast<uintptr_t>(workspace) % 16) return PYCBF_GB_EINVAL;
    if (rf->nt > kMaxNtSpline) return PYCBF_GB_ERANGE;
    SplineArgs sa;
    sa.rf = rfdata;
    sa.coef = workspace;
    sa.nch = rf->nframes * rf->ntx * rf->nrx;
    sa.nt = rf->nt;
    sa.t0 = rf->t0;
    sa.dt = rf->dt;
    int st = cuda_status(launch_spline(sa, rf->dtype, s));
    if (st) return st;
    *data = workspace;
    return PYCBF_GB_OK;
}

// the kernels' interpolation kind of an interp code (akima and makima share
// their gather: they differ only in the prefilter)
int gather_kind(int interp) {
    if (interp == PYCBF_GB_INTERP_KORDER) return KIND_POLY_NORM;
    if (interp == PYCBF_GB_INTERP_AKIMA || interp == PYCBF_GB_INTERP_MAKIMA) return KIND_POLY_DELTA;
    return interp;
}

bool geo_ok(const pycbf_gb_synthetic *g) {
    return g && g->ovectx && g->nvectx && g->t0tx && g->alatx && g->doftx && g->cosalatx &&
           g->secalatx && g->halfdofsintx && g->ovecrx && g->nvecrx && g->cosalarx && g->pnts &&
           g->np > 0 && g->np < (1LL << 31) && std::isfinite(g->c0) && g->c0 != 0.f;
}

}  // namespace

extern "C" {

int pycbf_gb_abi_version(void) { return PYCBF_GB_ABI_VERSION; }

const char *pycbf_gb_status_string(int status) {
    switch (status) {
        case PYCBF_GB_OK: return "ok";
        case PYCBF_GB_EINVAL: return "invalid argument";
        case PYCBF_GB_ERANGE: return "size out of supported range";
        case PYCBF_GB_EWORKSPACE: return "workspace missing, misaligned or too small";
        case PYCBF_GB_EUNSUPPORTED: return "unsupported combination";
        case PYCBF_GB_ECUDA: return "CUDA error";
        default: return "unknown status";
    }
}

int pycbf_gb_last_cuda_error(void) { return g_last_cuda_error; }

size_t pycbf_gb_workspace_bytes(const pycbf_gb_rfinfo *rf, int interp) {
    if (!rf || rf->ntx <= 0 || rf->nrx <= 0 || rf->nt <= 0 || rf->nframes <= 0) return 0;
    const size_t nsamp = (size_t)rf->nframes * (size_t)rf->ntx * (size_t)rf->nrx * (size_t)rf->nt;
    const bool f32rec = rf->dtype == PYCBF_GB_F32 || rf->dtype == PYCBF_GB_I16;
    if (interp == PYCBF_GB_INTERP_CUBIC) return nsamp * (f32rec ? 16 : 8);
    if (rf->dtype == PYCBF_GB_I16 &&
        (interp == PYCBF_GB_INTERP_NEAREST || interp == PYCBF_GB_INTERP_LINEAR ||
         interp == PYCBF_GB_INTERP_LINEAR_FLOOR))
        return nsamp * sizeof(float);
    return 0;
}

int pycbf_gb_spline_coefficients(const pycbf_gb_rfinfo *rf, const void *rfdata, void *coef,
                                 size_t coef_bytes, void *stream) {
    int st = check_rf(rf, false, true);
    if (st) return st;
    if (!rfdata) return PYCBF_GB_EINVAL;
    const void *data = nullptr;
    pycbf_gb_rfinfo eff;
    return prepare_data(rf, rfdata, PYCBF_GB_INTERP_CUBIC, coef, coef_bytes,
                        static_cast<cudaStream_t>(stream), &data, &eff);
}

size_t pycbf_gb_tabbed_plan_bytes(long long np, int ntx, int nrx) {
    if (np <= 0 || ntx <= 0 || nrx <= 0) return 0;
    return sizeof(int) * (size_t)tabbed_plan_words(np, ntx, nrx);
}

int pycbf_gb_tabbed_plan(const pycbf_gb_rfinfo *rf, const float *tautx, const float *apodtx,
                         const float *taurx, const float *apodrx, long long np, int interp,
                         float thresh, void *plan, size_t plan_bytes, void *stream) {
    int st = check_rf(rf, false, true);
    if (st) return st;
    if (!tautx || !apodtx || !taurx || !apodrx || !plan) return PYCBF_GB_EINVAL;
    if (np <= 0 || np >= (1LL << 31)) return PYCBF_GB_ERANGE;
    if (interp < 0 || interp > PYCBF_GB_INTERP_CUBIC || std::isnan(thresh)) return PYCBF_GB_EINVAL;
    if (rf->ntx > 12) return PYCBF_GB_EUNSUPPORTED;
    if (plan_bytes < pycbf_gb_tabbed_plan_bytes(np, (int)rf->ntx, (int)rf->nrx) ||
        reinterpret_cast<uintptr_t>(plan) % 16)
        return PYCBF_GB_EWORKSPACE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.tautx = tautx;
    a.apodtx = apodtx;
    a.taurx = taurx;
    a.apodrx = apodrx;
    a.np = np;
    a.thresh = thresh;
    st = cuda_status(cudaMemsetAsync(plan, 0, sizeof(int) * 4, s));
    if (st) return st;
    const int gdt = rf->dtype == PYCBF_GB_I16 ? PYCBF_GB_F32 : rf->dtype;  // as gathered
    return cuda_status(launch_tabbed_plan(a, interp, gdt, static_cast<int *>(plan), s));
}

int pycbf_gb_das_tabbed(const pycbf_gb_rfinfo *rf, const void *rfdata, const float *tautx,
                        const float *apodtx, const float *taurx, const float *apodrx,
                        long long np, const int *pixel_index, int interp, float thresh,
                        int sumtype, const void *plan, float *out, void *workspace,
                        size_t workspace_bytes, void *stream) {
    int st = check_rf(rf, false, true);
    if (st) return st;
    if (!rfdata || !tautx || !apodtx || !taurx || !apodrx || !out) return PYCBF_GB_EINVAL;
    if (np <= 0 || np >= (1LL << 31)) return np == 0 ? PYCBF_GB_OK : PYCBF_GB_ERANGE;
    if (interp >= PYCBF_GB_INTERP_KORDER && interp <= PYCBF_GB_INTERP_MAKIMA)
        return PYCBF_GB_EUNSUPPORTED;  // pycbf_gb_das_tabbed_poly
    if (interp < 0 || interp > 3 || sumtype < 0 || sumtype > 5) return PYCBF_GB_EINVAL;
    if (std::isnan(thresh)) return PYCBF_GB_EINVAL;
    if (!das_shape_ok(GEOM_TABBED, sumtype, rf->ntx)) return PYCBF_GB_ERANGE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const void *data = nullptr;
    pycbf_gb_rfinfo eff;
    st = prepare_data(rf, rfdata, interp, workspace, workspace_bytes, s, &data, &eff);
    if (st) return st;
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.data = data;
    a.tautx = tautx;
    a.apodtx = apodtx;
    a.taurx = taurx;
    a.apodrx = apodrx;
    a.pixel_index = pixel_index;
    a.out = out;
    a.np = np;
    a.thresh = thresh;
    return launch_tabbed(&eff, a, interp, sumtype, plan, s);
}

int pycbf_gb_das_tabbed_prefiltered(const pycbf_gb_rfinfo *rf, const void *coef,
                                    const float *tautx, const float *apodtx, const float *taurx,
                                    const float *apodrx, long long np, const int *pixel_index,
                                    float thresh, int sumtype, const void *plan, float *out,
                                    void *stream) {
    int st = pgb::check_tabbed_prefiltered(rf, coef, tautx, apodtx, taurx, apodrx, np, thresh,
                                           sumtype, out);
    if (st) return st;
    if (np == 0) return PYCBF_GB_OK;
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.data = coef;
    a.tautx = tautx;
    a.apodtx = apodtx;
    a.taurx = taurx;
    a.apodrx = apodrx;
    a.pixel_index = pixel_index;
    a.out = out;
    a.np = np;
    a.thresh = thresh;
    pycbf_gb_rfinfo eff = *rf;  // int16 channels were prefiltered into float32 records
    if (rf->dtype == PYCBF_GB_I16) eff.dtype = PYCBF_GB_F32;
    return launch_tabbed(&eff, a, PYCBF_GB_INTERP_CUBIC, sumtype, plan,
                         static_cast<cudaStream_t>(stream));
}

int pycbf_gb_das_tabbed_stall_test(const pycbf_gb_rfinfo *rf, const void *coef,
                                   const float *tautx, const float *apodtx, const float *taurx,
                                   const float *apodrx, long long np, const int *pixel_index,
                                   float thresh, const void *plan, float *out,
                                   long long wait_cycles, void *stream) {
    int st = check_rf(rf, false);
    if (st) return st;
    if (!coef || !tautx || !apodtx || !taurx || !apodrx || !out || !plan) return PYCBF_GB_EINVAL;
    if (reinterpret_cast<uintptr_t>(coef) % 16) return PYCBF_GB_EINVAL;
    if (np <= 0 || np >= (1LL << 31) || wait_cycles < 1000 || wait_cycles > (1LL << 31))
        return PYCBF_GB_ERANGE;
    if (std::isnan(thresh)) return PYCBF_GB_EINVAL;
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.data = coef;
    a.tautx = tautx;
    a.apodtx = apodtx;
    a.taurx = taurx;
    a.apodrx = apodrx;
    a.pixel_index = pixel_index;
    a.out = out;
    a.np = np;
    a.thresh = thresh;
    a.wait_cycles = wait_cycles;
    a.stall_test = 1;
    if (!staged_ok(rf, PYCBF_GB_INTERP_CUBIC, PYCBF_GB_SUM_TX_AND_RX, coef))
        return PYCBF_GB_EUNSUPPORTED;
    return launch_tabbed(rf, a, PYCBF_GB_INTERP_CUBIC, PYCBF_GB_SUM_TX_AND_RX, plan,
                         static_cast<cudaStream_t>(stream));
}

int pycbf_gb_das_synthetic(const pycbf_gb_rfinfo *rf, const void *rfdata,
                           const pycbf_gb_synthetic *geo, const int *pixel_index, int interp,
                           int sumtype, float *out, void *workspace, size_t workspace_bytes,
                           void *stream) {
    int st = check_rf(rf, true, true);
    if (st) return st;
    if (!rfdata || !out || !geo_ok(geo)) return PYCBF_GB_EINVAL;
    if (interp >= PYCBF_GB_INTERP_KORDER && interp <= PYCBF_GB_INTERP_MAKIMA)
        return PYCBF_GB_EUNSUPPORTED;  // pycbf_gb_das_synthetic_poly
    if (interp < 0 || interp > 3 || sumtype < 0 || sumtype > 5) return PYCBF_GB_EINVAL;
    if (!das_shape_ok(GEOM_SYNTH, sumtype, rf->ntx)) return PYCBF_GB_ERANGE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const void *data = nullptr;
    pycbf_gb_rfinfo eff;
    st = prepare_data(rf, rfdata, interp, workspace, workspace_bytes, s, &data, &eff);
    if (st) return st;
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.data = data;
    a.geo = *geo;
    a.ndim = rf->ndim;
    a.pixel_index = pixel_index;
    a.out = out;
    a.np = geo->np;
    a.thresh = 0.01f;
    return cuda_status(launch_das(a, GEOM_SYNTH, interp, sumtype, eff.dtype, false, s));
}

int pycbf_gb_tap_census_tabbed(const pycbf_gb_rfinfo *rf, const float *tautx,
                               const float *apodtx, const float *taurx, const float *apodrx,
                               long long np, int interp, float thresh, int *count,
                               long long *index_sum, void *stream) {
    int st = check_rf(rf, false, true);
    if (st) return st;
    if (!tautx || !apodtx || !taurx || !apodrx || !count || !index_sum) return PYCBF_GB_EINVAL;
    if (np <= 0 || np >= (1LL << 31)) return np == 0 ? PYCBF_GB_OK : PYCBF_GB_ERANGE;
    if (interp < 0 || interp > 6 || std::isnan(thresh)) return PYCBF_GB_EINVAL;
    if (!das_shape_ok(GEOM_TABBED, PYCBF_GB_SUM_TX_AND_RX, rf->ntx)) return PYCBF_GB_ERANGE;
    interp = gather_kind(interp);
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.nframes = 1;
    a.tautx = tautx;
    a.apodtx = apodtx;
    a.taurx = taurx;
    a.apodrx = apodrx;
    a.np = np;
    a.thresh = thresh;
    a.census_count = count;
    a.census_isum = index_sum;
    return cuda_status(launch_das(a, GEOM_TABBED, interp, PYCBF_GB_SUM_TX_AND_RX, PYCBF_GB_F32,
                                  true, static_cast<cudaStream_t>(stream)));
}

int pycbf_gb_tap_census_synthetic(const pycbf_gb_rfinfo *rf, const pycbf_gb_synthetic *geo,
                                  int interp, int *count, long long *index_sum, void *stream) {
    int st = check_rf(rf, true, true);
    if (st) return st;
    if (!geo_ok(geo) || !count || !index_sum) return PYCBF_GB_EINVAL;
    if (interp < 0 || interp > 6) return PYCBF_GB_EINVAL;
    interp = gather_kind(interp);
    if (!das_shape_ok(GEOM_SYNTH, PYCBF_GB_SUM_TX_AND_RX, rf->ntx)) return PYCBF_GB_ERANGE;
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.nframes = 1;
    a.geo = *geo;
    a.ndim = rf->ndim;
    a.np = geo->np;
    a.thresh = 0.01f;
    a.census_count = count;
    a.census_isum = index_sum;
    return cuda_status(launch_das(a, GEOM_SYNTH, interp, PYCBF_GB_SUM_TX_AND_RX, PYCBF_GB_F32,
                                  true, static_cast<cudaStream_t>(stream)));
}

int pycbf_gb_synthetic_rx_mask(const pycbf_gb_rfinfo *rf, const pycbf_gb_synthetic *geo,
                               unsigned char *mask, void *stream) {
    int st = check_rf(rf, true, true);
    if (st) return st;
    if (!geo_ok(geo) || !mask) return PYCBF_GB_EINVAL;
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.geo = *geo;
    a.ndim = rf->ndim;
    a.np = geo->np;
    return cuda_status(launch_synth_rx_mask(a, mask, static_cast<cudaStream_t>(stream)));
}

int pycbf_gb_dmas(const float *imsep, long long nframes, long long nsep, long long np,
                  const int *lags, int nlag, int dmastype, int sumlags, float *out,
                  void *stream) {
    if (!imsep || !lags || !out) return PYCBF_GB_EINVAL;
    if (nframes <= 0 || nsep <= 0 || np <= 0 || nlag <= 0) return PYCBF_GB_EINVAL;
    if (dmastype != 0 && dmastype != 1) return PYCBF_GB_EINVAL;
    if (nframes > 65535 || np >= (1LL << 40)) return PYCBF_GB_ERANGE;
    return cuda_status(launch_dmas(imsep, nframes, nsep, np, lags, nlag, dmastype, sumlags ? 1 : 0,
                                   out, static_cast<cudaStream_t>(stream)));
}

int pycbf_gb_slsc(const float *im, const unsigned char *mask, long long nframes, int nrx, int nx,
                  int nz, int nlag, int nkern, float *out, void *stream) {
    if (!im || !mask || !out) return PYCBF_GB_EINVAL;
    if (nframes <= 0 || nrx <= 0 || nx <= 0 || nz <= 0 || nlag <= 0 || nkern < 0)
        return PYCBF_GB_EINVAL;
    if (nlag > 32 || 2 * nkern + 1 > 64 || nframes > 65535) return PYCBF_GB_ERANGE;
    return cuda_status(launch_slsc(im, mask, nullptr, nframes, nrx, nx, nz, nlag, nkern, out,
                                   static_cast<cudaStream_t>(stream)));
}

size_t pycbf_gb_slsc_kept_bytes(int nrx, int nx, int nz) {
    if (nrx <= 0 || nx <= 0 || nz <= 0) return 0;
    return sizeof(unsigned) * (size_t)((nrx + 31) / 32) * (size_t)nx * (size_t)nz;
}

int pycbf_gb_slsc_kept(const unsigned char *mask, int nrx, int nx, int nz, int nlag, int nkern,
                       unsigned *kept, size_t kept_bytes, void *stream) {
    if (!mask || !kept) return PYCBF_GB_EINVAL;
    if (nrx <= 0 || nx <= 0 || nz <= 0 || nlag <= 0 || nkern < 0) return PYCBF_GB_EINVAL;
    if (!slsc_kept_supported(nrx, nlag, nkern)) return PYCBF_GB_ERANGE;
    if (kept_bytes < pycbf_gb_slsc_kept_bytes(nrx, nx, nz)) return PYCBF_GB_ERANGE;
    return cuda_status(
        launch_slsc_kept(mask, nrx, nx, nz, nkern, kept, static_cast<cudaStream_t>(stream)));
}

int pycbf_gb_slsc_with_kept(const float *im, const unsigned *kept, long long nframes, int nrx,
                            int nx, int nz, int nlag, int nkern, float *out, void *stream) {
    if (!im || !kept || !out) return PYCBF_GB_EINVAL;
    if (nframes <= 0 || nrx <= 0 || nx <= 0 || nz <= 0 || nlag <= 0 || nkern < 0)
        return PYCBF_GB_EINVAL;
    if (!slsc_kept_supported(nrx, nlag, nkern) || nframes > 65535) return PYCBF_GB_ERANGE;
    return cuda_status(launch_slsc(im, nullptr, kept, nframes, nrx, nx, nz, nlag, nkern, out,
                                   static_cast<cudaStream_t>(stream)));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// differentiable cubic delay-and-sum
// ---------------------------------------------------------------------------
namespace {

constexpr long long kMaxAdjTx = 128;  // three shared-memory columns per transmit (192 KB)

int check_adjoint_common(const pycbf_gb_rfinfo *rf, const void *coef, int sumtype, bool synthetic) {
    int st = check_rf(rf, synthetic);
    if (st) return st;
    if (!coef || reinterpret_cast<uintptr_t>(coef) % 16) return PYCBF_GB_EINVAL;
    if (sumtype != PYCBF_GB_SUM_TX_AND_RX && sumtype != PYCBF_GB_SUM_TX_ONLY)
        return PYCBF_GB_EUNSUPPORTED;
    if (rf->ntx > kMaxAdjTx || rf->nt > kMaxNtSpline || !adjoint_rows_warps(rf->nt))
        return PYCBF_GB_ERANGE;
    return PYCBF_GB_OK;
}

int run_adjoint(const pycbf_gb_rfinfo *rf, AdjArgs &g, void *workspace, size_t workspace_bytes,
                cudaStream_t s) {
    if (g.grad_rf || g.d.pixel_index) {
        const size_t need = pycbf_gb_adjoint_workspace_bytes(rf, g.d.np);
        if (!workspace || workspace_bytes < need || reinterpret_cast<uintptr_t>(workspace) % 16)
            return PYCBF_GB_EWORKSPACE;
        g.gk_buf = static_cast<float *>(workspace);
        char *ws = static_cast<char *>(workspace);
        const size_t gb = adjoint_grad_bytes(rf->nframes, rf->nrx, g.d.np);
        g.partial = reinterpret_cast<float *>(ws + gb);
        g.live = reinterpret_cast<unsigned char *>(
            ws + gb + adjoint_partial_bytes(rf->nframes, rf->ntx, rf->nrx, g.d.np, rf->nt));
    }
    return cuda_status(launch_adjoint(g, rf->dtype, s));
}

}  // namespace

extern "C" {

int pycbf_gb_das_synthetic_slowness(const pycbf_gb_rfinfo *rf, const void *coef,
                                    const pycbf_gb_synthetic *geo, const float *slowness,
                                    const int *pixel_index, int sumtype, float *out,
                                    void *stream) {
    int st = check_adjoint_common(rf, coef, sumtype, true);
    if (st) return st;
    if (!geo_ok(geo) || !slowness || !out) return PYCBF_GB_EINVAL;
    if (!das_shape_ok(GEOM_SYNTH, sumtype, rf->ntx)) return PYCBF_GB_ERANGE;
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.data = coef;
    a.geo = *geo;
    a.ndim = rf->ndim;
    a.pixel_index = pixel_index;
    a.out = out;
    a.np = geo->np;
    a.slow = slowness;
    return cuda_status(launch_das_synth_slow(a, sumtype, rf->dtype, static_cast<cudaStream_t>(stream)));
}

size_t pycbf_gb_adjoint_workspace_bytes(const pycbf_gb_rfinfo *rf, long long np) {
    if (!rf || np <= 0 || rf->ntx <= 0 || rf->nrx <= 0 || rf->nt <= 0 || rf->nframes <= 0) return 0;
    return adjoint_workspace_bytes(rf->nframes, rf->ntx, rf->nrx, np, rf->nt);
}

int pycbf_gb_das_tabbed_adjoint(const pycbf_gb_rfinfo *rf, const void *coef,
                                const float *tautx, const float *apodtx, const float *taurx,
                                const float *apodrx, long long np, const int *pixel_index,
                                float thresh, int sumtype, const float *grad_out,
                                float *grad_rf, float *grad_tautx, float *grad_taurx,
                                void *workspace, size_t workspace_bytes, void *stream) {
    int st = check_adjoint_common(rf, coef, sumtype, false);
    if (st) return st;
    if (!tautx || !apodtx || !taurx || !apodrx || !grad_out || std::isnan(thresh))
        return PYCBF_GB_EINVAL;
    if (np <= 0 || np >= (1LL << 31)) return np == 0 ? PYCBF_GB_OK : PYCBF_GB_ERANGE;
    AdjArgs g = {};
    fill_time_axis(g.d, rf);
    g.d.data = coef;
    g.d.tautx = tautx;
    g.d.apodtx = apodtx;
    g.d.taurx = taurx;
    g.d.apodrx = apodrx;
    g.d.pixel_index = pixel_index;
    g.d.np = np;
    g.d.thresh = thresh;
    g.geom = GEOM_TABBED;
    g.sumtype = sumtype;
    g.gout = grad_out;
    g.grad_rf = grad_rf;
    g.grad_tautx = grad_tautx;
    g.grad_taurx = grad_taurx;
    return run_adjoint(rf, g, workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

int pycbf_gb_das_tabbed_adjoint_planned(const pycbf_gb_rfinfo *rf, const void *coef,
                                        const float *tautx, const float *apodtx,
                                        const float *taurx, const float *apodrx, long long np,
                                        const int *pixel_index, float thresh, int sumtype,
                                        const void *plan, const float *grad_out, float *grad_rf,
                                        float *grad_tautx, float *grad_taurx, void *workspace,
                                        size_t workspace_bytes, void *stream) {
    int st = check_adjoint_common(rf, coef, sumtype, false);
    if (st) return st;
    if (!tautx || !apodtx || !taurx || !apodrx || !grad_out || std::isnan(thresh))
        return PYCBF_GB_EINVAL;
    if (plan && reinterpret_cast<uintptr_t>(plan) % 16) return PYCBF_GB_EINVAL;
    if (np <= 0 || np >= (1LL << 31)) return np == 0 ? PYCBF_GB_OK : PYCBF_GB_ERANGE;
    AdjArgs g = {};
    fill_time_axis(g.d, rf);
    g.d.data = coef;
    g.d.tautx = tautx;
    g.d.apodtx = apodtx;
    g.d.taurx = taurx;
    g.d.apodrx = apodrx;
    g.d.pixel_index = pixel_index;
    g.d.np = np;
    g.d.thresh = thresh;
    g.geom = GEOM_TABBED;
    g.sumtype = sumtype;
    g.gout = grad_out;
    g.grad_rf = grad_rf;
    g.grad_tautx = grad_tautx;
    g.grad_taurx = grad_taurx;
    // the staged delay gradients need the plan's staged path for cubic
    // float32 records and one frame; otherwise the plan is not used
    if (plan && rf->nframes == 1 && rf->dtype == PYCBF_GB_F32 &&
        staged_ok(rf, PYCBF_GB_INTERP_CUBIC, sumtype, coef))
        g.plan = static_cast<const int *>(plan);
    return run_adjoint(rf, g, workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}


int pycbf_gb_das_synthetic_adjoint(const pycbf_gb_rfinfo *rf, const void *coef,
                                   const pycbf_gb_synthetic *geo, const float *slowness,
                                   const int *pixel_index, int sumtype, const float *grad_out,
                                   float *grad_rf, float *grad_slow, void *workspace,
                                   size_t workspace_bytes, void *stream) {
    int st = check_adjoint_common(rf, coef, sumtype, true);
    if (st) return st;
    if (!geo_ok(geo) || !slowness || !grad_out) return PYCBF_GB_EINVAL;
    AdjArgs g = {};
    fill_time_axis(g.d, rf);
    g.d.data = coef;
    g.d.geo = *geo;
    g.d.ndim = rf->ndim;
    g.d.pixel_index = pixel_index;
    g.d.np = geo->np;
    g.d.slow = slowness;
    g.geom = GEOM_SYNTH_SLOW;
    g.sumtype = sumtype;
    g.gout = grad_out;
    g.grad_rf = grad_rf;
    g.grad_slow = grad_slow;
    return run_adjoint(rf, g, workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// uneven batches
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kBatchHeader = 16;  // the work-queue head, padded

long long job_np(const pycbf_gb_batch_job &j) { return j.geom == 0 ? j.np : (j.geo ? j.geo->np : 0); }

long long job_items(const pycbf_gb_batch_job &j, int tiles_per_item) {
    const long long tiles = (job_np(j) + kBlock - 1) / kBlock;
    return (tiles + tiles_per_item - 1) / tiles_per_item;
}

int check_batch_job(const pycbf_gb_batch_job &j) {
    if (j.geom != 0 && j.geom != 1) return PYCBF_GB_EINVAL;
    int st = check_rf(&j.rf, j.geom == 1);
    if (st) return st;
    if (j.rf.nframes != 1) return PYCBF_GB_EINVAL;
    if (!j.rfdata || !j.coef || !j.out) return PYCBF_GB_EINVAL;
    if (reinterpret_cast<uintptr_t>(j.coef) % 16) return PYCBF_GB_EINVAL;
    if (j.rf.nt > kMaxNtSpline) return PYCBF_GB_ERANGE;
    if (j.geom == 0) {
        if (!j.tautx || !j.apodtx || !j.taurx || !j.apodrx || std::isnan(j.thresh))
            return PYCBF_GB_EINVAL;
        if (j.np <= 0 || j.np >= (1LL << 31)) return PYCBF_GB_ERANGE;
    } else {
        if (!geo_ok(j.geo)) return PYCBF_GB_EINVAL;
    }
    return PYCBF_GB_OK;
}

}  // namespace

extern "C" {

size_t pycbf_gb_batch_plan_bytes(const pycbf_gb_batch_job *jobs, int njobs, int tiles_per_item) {
    if (!jobs || njobs <= 0 || tiles_per_item < 1 || tiles_per_item > 8) return 0;
    long long items = 0;
    for (int k = 0; k < njobs; ++k) items += job_items(jobs[k], tiles_per_item);
    return kBatchHeader + sizeof(BatchJob) * (size_t)njobs + sizeof(int2) * (size_t)items;
}

int pycbf_gb_batch_plan(const pycbf_gb_batch_job *jobs, int njobs, int tiles_per_item, int order,
                        void *plan, size_t plan_bytes, pycbf_gb_batch_info *info, void *stream) {
    if (!jobs || njobs <= 0 || !plan || !info) return PYCBF_GB_EINVAL;
    if (tiles_per_item < 1 || tiles_per_item > 8 || (order != 0 && order != 1))
        return PYCBF_GB_EINVAL;
    for (int k = 0; k < njobs; ++k) {
        int st = check_batch_job(jobs[k]);
        if (st) return st;
    }
    const size_t need = pycbf_gb_batch_plan_bytes(jobs, njobs, tiles_per_item);
    if (plan_bytes < need || reinterpret_cast<uintptr_t>(plan) % 16) return PYCBF_GB_EWORKSPACE;

    std::vector<BatchJob> desc((size_t)njobs);
    std::vector<int2> items;
    std::vector<double> cost;
    long long ch0 = 0;
    int max_nt = 1, max_ntx = 1, dtypes = 0;
    for (int k = 0; k < njobs; ++k) {
        const pycbf_gb_batch_job &j = jobs[k];
        BatchJob &b = desc[(size_t)k];
        dtypes |= 1 << j.rf.dtype;
        b = BatchJob{};
        fill_time_axis(b.a, &j.rf);
        b.a.data = j.coef;
        b.a.pixel_index = j.pixel_index;
        b.a.out = j.out;
        b.a.np = job_np(j);
        if (j.geom == 0) {
            b.a.tautx = j.tautx;
            b.a.apodtx = j.apodtx;
            b.a.taurx = j.taurx;
            b.a.apodrx = j.apodrx;
            b.a.thresh = j.thresh;
        } else {
            b.a.geo = *j.geo;
            b.a.ndim = j.rf.ndim;
            b.a.thresh = 0.01f;
        }
        b.rf = j.rfdata;
        b.ch0 = ch0;
        b.geom = j.geom == 0 ? GEOM_TABBED : GEOM_SYNTH;
        b.dtype = j.rf.dtype;
        ch0 += j.rf.ntx * j.rf.nrx;
        max_nt = std::max(max_nt, j.rf.nt);
        max_ntx = std::max(max_ntx, (int)j.rf.ntx);
        const long long n = job_items(j, tiles_per_item);
        // relative cost of an item: its taps, synthetic delays weighted up
        const double c = (double)j.rf.ntx * (double)j.rf.nrx * (j.geom == 1 ? 1.3 : 1.0);
        for (long long t = 0; t < n; ++t) {
            items.push_back(make_int2(k, (int)t));
            cost.push_back(c);
        }
    }
    if (order == 1) {
        std::vector<size_t> idx(items.size());
        for (size_t q = 0; q < idx.size(); ++q) idx[q] = q;
        std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) { return cost[x] > cost[y]; });
        std::vector<int2> sorted(items.size());
        for (size_t q = 0; q < idx.size(); ++q) sorted[q] = items[idx[q]];
        items.swap(sorted);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char *base = static_cast<char *>(plan);
    int st = cuda_status(cudaMemsetAsync(base, 0, kBatchHeader, s));
    if (st) return st;
    st = cuda_status(cudaMemcpyAsync(base + kBatchHeader, desc.data(), sizeof(BatchJob) * desc.size(),
                                     cudaMemcpyHostToDevice, s));
    if (st) return st;
    if (!items.empty()) {
        st = cuda_status(cudaMemcpyAsync(base + kBatchHeader + sizeof(BatchJob) * desc.size(),
                                         items.data(), sizeof(int2) * items.size(),
                                         cudaMemcpyHostToDevice, s));
        if (st) return st;
    }
    info->nitems = (long long)items.size();
    info->nchannels = ch0;
    info->njobs = njobs;
    info->max_nt = max_nt;
    info->tiles_per_item = tiles_per_item;
    info->max_ntx = max_ntx;
    info->dtypes = dtypes;
    // shared-memory sizes of the batched prefilter and delay-and-sum, set outside any capture
    st = cuda_status(prepare_batch_das(max_ntx));
    if (st) return st;
    return cuda_status(launch_batch_spline(reinterpret_cast<const BatchJob *>(base + kBatchHeader),
                                           njobs, 0, max_nt, s, true));
}

int pycbf_gb_batch_run(const void *plan, const pycbf_gb_batch_info *info, int tx_chunk, int ctas,
                       void *stream) {
    if (!plan || !info || info->njobs <= 0 || info->nitems < 0 || info->max_nt <= 0)
        return PYCBF_GB_EINVAL;
    if (tx_chunk != 0 && tx_chunk != 4 && tx_chunk != 8 && tx_chunk != 12) return PYCBF_GB_EINVAL;
    if (tx_chunk == 0 && (info->max_ntx < 1 || info->max_ntx > (1 << 20))) return PYCBF_GB_EINVAL;
    if (ctas < 1 || ctas > (1 << 20) || info->tiles_per_item < 1 || info->tiles_per_item > 8)
        return PYCBF_GB_EINVAL;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const char *base = static_cast<const char *>(plan);
    const BatchJob *jobs = reinterpret_cast<const BatchJob *>(base + kBatchHeader);
    const int2 *items = reinterpret_cast<const int2 *>(base + kBatchHeader +
                                                       sizeof(BatchJob) * (size_t)info->njobs);
    unsigned long long *counter =
        reinterpret_cast<unsigned long long *>(const_cast<char *>(base));
    int st = cuda_status(launch_batch_spline(jobs, info->njobs, info->nchannels, info->max_nt, s,
                                             false));
    if (st) return st;
    return cuda_status(launch_batch_das(jobs, items, info->nitems, info->tiles_per_item, counter,
                                        tx_chunk, ctas, s, info->max_ntx, info->dtypes));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// cubic upsampling for nearest with usf > 1
// ---------------------------------------------------------------------------
extern "C" {

size_t pycbf_gb_upsampled_bytes(const pycbf_gb_rfinfo *rf, int usf) {
    if (!rf || usf < 1 || rf->ntx <= 0 || rf->nrx <= 0 || rf->nt <= 0 || rf->nframes <= 0) return 0;
    const long long ntu = (long long)usf * (rf->nt - 1) + 1;
    return sizeof(float) * (size_t)rf->nframes * (size_t)rf->ntx * (size_t)rf->nrx * (size_t)ntu;
}

int pycbf_gb_upsample(const pycbf_gb_rfinfo *rf, const void *rfdata, int usf, void *workspace,
                      size_t workspace_bytes, float *out, size_t out_bytes, void *stream) {
    int st = check_rf(rf, false);
    if (st) return st;
    if (!rfdata || !out || usf < 1) return PYCBF_GB_EINVAL;
    const long long ntu = (long long)usf * (rf->nt - 1) + 1;
    if (ntu >= kMaxNt) return PYCBF_GB_ERANGE;
    if (out_bytes < pycbf_gb_upsampled_bytes(rf, usf)) return PYCBF_GB_EWORKSPACE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const void *data = nullptr;
    pycbf_gb_rfinfo eff;
    st = prepare_data(rf, rfdata, PYCBF_GB_INTERP_CUBIC, workspace, workspace_bytes, s, &data, &eff);
    if (st) return st;
    DasArgs a = {};
    fill_time_axis(a, rf);
    a.data = data;
    const float dtu = rf->dt / (float)usf;
    return cuda_status(launch_upsample(a, rf->dtype, out, rf->nframes * rf->ntx * rf->nrx, (int)ntu,
                                       dtu, s));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// korder / akima / makima
// ---------------------------------------------------------------------------
namespace {

constexpr int kMaxKorder = 128;

bool poly_kind(int interp) {
    return interp == PYCBF_GB_INTERP_KORDER || interp == PYCBF_GB_INTERP_AKIMA ||
           interp == PYCBF_GB_INTERP_MAKIMA;
}

size_t poly_record_bytes(const pycbf_gb_rfinfo *rf) {
    return (size_t)rf->nframes * (size_t)rf->ntx * (size_t)rf->nrx * (size_t)rf->nt * 16;
}

int poly_args(const pycbf_gb_rfinfo *rf, const void *coef, int interp, int sumtype, bool synth,
              DasArgs &a) {
    int st = check_rf(rf, synth);
    if (st) return st;
    if (!poly_kind(interp) || !coef || reinterpret_cast<uintptr_t>(coef) % 16) return PYCBF_GB_EINVAL;
    if (sumtype < 0 || sumtype > 5) return PYCBF_GB_EINVAL;
    if (!das_shape_ok(synth ? GEOM_SYNTH : GEOM_TABBED, sumtype, rf->ntx)) return PYCBF_GB_ERANGE;
    a = DasArgs{};
    fill_time_axis(a, rf);
    a.data = coef;
    return PYCBF_GB_OK;
}

}  // namespace

extern "C" {

size_t pycbf_gb_poly_workspace_bytes(const pycbf_gb_rfinfo *rf, int interp, int k) {
    if (!rf || !poly_kind(interp) || rf->ntx <= 0 || rf->nrx <= 0 || rf->nt <= 0 ||
        rf->nframes <= 0 || k < 0 || k > kMaxKorder)
        return 0;
    const size_t sbytes =
        interp == PYCBF_GB_INTERP_KORDER ? ((sizeof(float) * (size_t)k * k + 15) & ~(size_t)15) : 0;
    return poly_record_bytes(rf) + sbytes;
}

int pycbf_gb_poly_coefficients(const pycbf_gb_rfinfo *rf, const void *rfdata, int interp, int k,
                               const float *S, void *coef, size_t coef_bytes, void *stream) {
    int st = check_rf(rf, false);
    if (st) return st;
    if (!rfdata || !coef || !poly_kind(interp) || reinterpret_cast<uintptr_t>(coef) % 16)
        return PYCBF_GB_EINVAL;
    if (interp == PYCBF_GB_INTERP_KORDER) {
        if (k < 0 || k > kMaxKorder || (k % 2) || k > rf->nt || (k > 0 && !S)) return PYCBF_GB_EINVAL;
        if (rf->nt < 2) return PYCBF_GB_ERANGE;
    } else {
        k = 0;
        if (rf->nt < 5) return PYCBF_GB_ERANGE;
    }
    if (coef_bytes < pycbf_gb_poly_workspace_bytes(rf, interp, k)) return PYCBF_GB_EWORKSPACE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float *dS = nullptr;
    if (interp == PYCBF_GB_INTERP_KORDER && k > 0) {
        dS = reinterpret_cast<float *>(static_cast<char *>(coef) + poly_record_bytes(rf));
        st = cuda_status(cudaMemcpyAsync(dS, S, sizeof(float) * k * k, cudaMemcpyHostToDevice, s));
        if (st) return st;
    }
    DasArgs a = {};
    fill_time_axis(a, rf);
    return cuda_status(launch_poly_records(a, rfdata, rf->dtype, interp, k, dS,
                                           static_cast<float4 *>(coef),
                                           rf->nframes * rf->ntx * rf->nrx, s));
}

int pycbf_gb_das_tabbed_poly(const pycbf_gb_rfinfo *rf, const void *coef, int interp,
                             const float *tautx, const float *apodtx, const float *taurx,
                             const float *apodrx, long long np, const int *pixel_index,
                             float thresh, int sumtype, float *out, void *stream) {
    DasArgs a;
    int st = poly_args(rf, coef, interp, sumtype, false, a);
    if (st) return st;
    if (!tautx || !apodtx || !taurx || !apodrx || !out || std::isnan(thresh)) return PYCBF_GB_EINVAL;
    if (np <= 0 || np >= (1LL << 31)) return np == 0 ? PYCBF_GB_OK : PYCBF_GB_ERANGE;
    a.tautx = tautx;
    a.apodtx = apodtx;
    a.taurx = taurx;
    a.apodrx = apodrx;
    a.pixel_index = pixel_index;
    a.out = out;
    a.np = np;
    a.thresh = thresh;
    return cuda_status(launch_das(a, GEOM_TABBED, gather_kind(interp), sumtype, PYCBF_GB_F32, false,
                                  static_cast<cudaStream_t>(stream)));
}

int pycbf_gb_das_synthetic_poly(const pycbf_gb_rfinfo *rf, const void *coef, int interp,
                                const pycbf_gb_synthetic *geo, const int *pixel_index,
                                int sumtype, float *out, void *stream) {
    DasArgs a;
    int st = poly_args(rf, coef, interp, sumtype, true, a);
    if (st) return st;
    if (!geo_ok(geo) || !out) return PYCBF_GB_EINVAL;
    a.geo = *geo;
    a.ndim = rf->ndim;
    a.pixel_index = pixel_index;
    a.out = out;
    a.np = geo->np;
    a.thresh = 0.01f;
    return cuda_status(launch_das(a, GEOM_SYNTH, gather_kind(interp), sumtype, PYCBF_GB_F32, false,
                                  static_cast<cudaStream_t>(stream)));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// delay tables of a linear array on a grid
// ---------------------------------------------------------------------------
extern "C" int pycbf_gb_tables_2d(int txkind, int ntx, const double *tx_params, int nele,
                                  const double *xele, int nx, const double *xout, int nz,
                                  const double *zout, double cm, double fnum, int hann,
                                  float *tautx, float *apodtx, float *taurx, float *apodrx,
                                  void *stream) {
    if (txkind < 0 || txkind > 2 || !tx_params || !xele || !xout || !zout || !tautx || !apodtx ||
        !taurx || !apodrx)
        return PYCBF_GB_EINVAL;
    if (ntx <= 0 || nele <= 0 || nx <= 0 || nz <= 0 || !std::isfinite(cm) || cm <= 0.0 ||
        !std::isfinite(fnum) || fnum <= 0.0)
        return PYCBF_GB_EINVAL;
    if (ntx > kTables2DMaxTx || (long long)nx * nz >= (1LL << 31)) return PYCBF_GB_ERANGE;
    Tables2D p = {};
    p.txkind = txkind;
    p.ntx = ntx;
    p.nele = nele;
    p.nx = nx;
    p.nz = nz;
    p.hann = hann ? 1 : 0;
    p.cm = cm;
    p.fnum2 = 2.0 * fnum;
    for (int t = 0; t < ntx; ++t)
        for (int k = 0; k < 6; ++k) p.tx[t][k] = tx_params[6 * t + k];
    return cuda_status(launch_tables_2d(p, xele, xout, zout, tautx, apodtx, taurx, apodrx,
                                        static_cast<cudaStream_t>(stream)));
}

// ---------------------------------------------------------------------------
// demodulation, envelope, percentile and log compression
// ---------------------------------------------------------------------------
extern "C" int pycbf_gb_demod(const float *x, long long ncols, int n, const float *W, int M,
                              float *iq, float *env, void *stream) {
    if (!x || !W || (!iq && !env) || ncols < 0 || n <= 0 || M <= 0) return PYCBF_GB_EINVAL;
    if ((ncols + 15) / 16 > 0x7fffffffLL || ((long long)M + 31) / 32 > 65535) return PYCBF_GB_ERANGE;
    return cuda_status(launch_demod(x, ncols, n, reinterpret_cast<const float2 *>(W), M,
                                    reinterpret_cast<float2 *>(iq), env,
                                    static_cast<cudaStream_t>(stream)));
}

extern "C" size_t pycbf_gb_percentile_workspace_bytes(long long nseg) {
    return nseg > 0 ? percentile_workspace_bytes(nseg) : 0;
}

extern "C" int pycbf_gb_percentile(const float *v, long long nseg, long long n, double q,
                                   float *out, void *workspace, size_t workspace_bytes,
                                   void *stream) {
    if (!v || !out || nseg < 0 || n <= 0 || !(q >= 0.0 && q <= 100.0)) return PYCBF_GB_EINVAL;
    if (n > 0x7fffffffLL || nseg > 65535) return PYCBF_GB_ERANGE;
    if (nseg == 0) return PYCBF_GB_OK;
    if (!workspace || workspace_bytes < percentile_workspace_bytes(nseg)) return PYCBF_GB_EWORKSPACE;
    return cuda_status(launch_percentile(v, nseg, n, q, out, workspace,
                                         static_cast<cudaStream_t>(stream)));
}

extern "C" int pycbf_gb_log_compress_percentile(const float *env, long long nseg, long long n,
                                                double q, float floor_add, float *out, float *ref,
                                                void *workspace, size_t workspace_bytes,
                                                void *stream) {
    if (!env || !out || !ref || nseg < 0 || n <= 0 || !(q >= 0.0 && q <= 100.0) ||
        !std::isfinite(floor_add))
        return PYCBF_GB_EINVAL;
    if (n > 0x7fffffffLL || nseg > 65535) return PYCBF_GB_ERANGE;
    if (nseg == 0) return PYCBF_GB_OK;
    if (!workspace || workspace_bytes < percentile_workspace_bytes(nseg)) return PYCBF_GB_EWORKSPACE;
    return cuda_status(launch_percentile(env, nseg, n, q, ref, workspace,
                                         static_cast<cudaStream_t>(stream), floor_add, out));
}

extern "C" int pycbf_gb_log_compress(const float *env, long long nseg, long long n,
                                     const float *ref, float floor_add, float *out, void *stream) {
    if (!env || !ref || !out || nseg < 0 || n <= 0 || !std::isfinite(floor_add)) return PYCBF_GB_EINVAL;
    if (nseg > 0 && n > std::numeric_limits<long long>::max() / nseg) return PYCBF_GB_ERANGE;
    return cuda_status(launch_log_compress(env, nseg, n, ref, floor_add, out,
                                           static_cast<cudaStream_t>(stream)));
}

extern "C" int pycbf_gb_convert_i16(const short *src, long long n, float *dst, void *stream) {
    if (!src || !dst || n < 0) return PYCBF_GB_EINVAL;
    return cuda_status(launch_convert_i16(src, n, dst, static_cast<cudaStream_t>(stream)));
}

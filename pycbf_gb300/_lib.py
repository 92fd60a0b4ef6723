"""ctypes binding of libpycbf_gb300.so (the C ABI of include/pycbf_gb300.h).

The library is loaded from this package's directory.  There is no fallback:
if it is missing or fails to load, every beamformer call raises.
"""
from __future__ import annotations

import ctypes as ct
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpycbf_gb300.so")

# status codes
OK, EINVAL, ERANGE, EWORKSPACE, EUNSUPPORTED, ECUDA = range(6)
# storage types
F32, F16, BF16, I16 = 0, 1, 2, 3
# interpolation kinds
INTERP = {"nearest": 0, "linear": 1, "cubic": 2, "linear_floor": 3, "korder_cubic": 4, "akima": 5,
          "makima": 6}
# sum types (0..3 are the reference's flag values)
SUMTYPE = {"none": 0, "tx_only": 1, "rx_only": 2, "tx_and_rx": 3, "dmas_ssr": 4, "dmas_power": 5}

EXPORTS = (
    "pycbf_gb_abi_version", "pycbf_gb_status_string", "pycbf_gb_last_cuda_error",
    "pycbf_gb_workspace_bytes", "pycbf_gb_spline_coefficients", "pycbf_gb_das_tabbed",
    "pycbf_gb_das_tabbed_prefiltered", "pycbf_gb_tabbed_plan_bytes", "pycbf_gb_tabbed_plan",
    "pycbf_gb_das_synthetic", "pycbf_gb_tap_census_tabbed", "pycbf_gb_tap_census_synthetic",
    "pycbf_gb_synthetic_rx_mask", "pycbf_gb_dmas", "pycbf_gb_slsc", "pycbf_gb_slsc_kept_bytes",
    "pycbf_gb_slsc_kept", "pycbf_gb_slsc_with_kept", "pycbf_gb_fp32_probe",
    "pycbf_gb_das_tabbed_cubic_noalloc", "pycbf_gb_das_synthetic_slowness",
    "pycbf_gb_adjoint_workspace_bytes", "pycbf_gb_das_tabbed_adjoint",
    "pycbf_gb_das_tabbed_adjoint_planned",
    "pycbf_gb_das_synthetic_adjoint", "pycbf_gb_batch_plan_bytes", "pycbf_gb_batch_plan",
    "pycbf_gb_batch_run", "pycbf_gb_upsampled_bytes", "pycbf_gb_upsample",
    "pycbf_gb_poly_workspace_bytes", "pycbf_gb_poly_coefficients", "pycbf_gb_das_tabbed_poly",
    "pycbf_gb_das_synthetic_poly", "pycbf_gb_tables_2d", "pycbf_gb_demod",
    "pycbf_gb_percentile_workspace_bytes", "pycbf_gb_percentile", "pycbf_gb_log_compress",
    "pycbf_gb_convert_i16", "pycbf_gb_log_compress_percentile", "pycbf_gb_das_tabbed_stall_test",
)
NOALLOC_SCRATCH_BYTES = 64 << 20


class RFInfo(ct.Structure):
    """pycbf_gb_rfinfo: mirrors RFInfo of pycbf/gpu/__engines__.cu:369-374."""
    _fields_ = [("ntx", ct.c_longlong), ("nrx", ct.c_longlong), ("ndim", ct.c_int),
                ("t0", ct.c_float), ("dt", ct.c_float), ("nt", ct.c_int),
                ("nframes", ct.c_longlong), ("dtype", ct.c_int)]


class SyntheticGeom(ct.Structure):
    """pycbf_gb_synthetic: device pointers of the synthetic-point geometry."""
    _fields_ = [(n, ct.c_void_p) for n in (
        "ovectx", "nvectx", "t0tx", "alatx", "doftx", "cosalatx", "secalatx", "halfdofsintx",
        "ovecrx", "nvecrx", "cosalarx", "pnts")] + [("np", ct.c_longlong), ("c0", ct.c_float)]


class BatchJob(ct.Structure):
    """pycbf_gb_batch_job: one frame of one beamformer in an uneven batch."""
    _fields_ = [("geom", ct.c_int), ("rf", RFInfo), ("rfdata", ct.c_void_p), ("coef", ct.c_void_p),
                ("tautx", ct.c_void_p), ("apodtx", ct.c_void_p), ("taurx", ct.c_void_p),
                ("apodrx", ct.c_void_p), ("np", ct.c_longlong), ("thresh", ct.c_float),
                ("geo", ct.POINTER(SyntheticGeom)), ("pixel_index", ct.c_void_p),
                ("out", ct.c_void_p)]


class BatchInfo(ct.Structure):
    """pycbf_gb_batch_info: what pycbf_gb_batch_run needs from the plan."""
    _fields_ = [("nitems", ct.c_longlong), ("nchannels", ct.c_longlong), ("njobs", ct.c_int),
                ("max_nt", ct.c_int), ("tiles_per_item", ct.c_int), ("max_ntx", ct.c_int),
                ("dtypes", ct.c_int)]


class GPUError(RuntimeError):
    pass


_lib = None
_lock = threading.Lock()


def load() -> ct.CDLL:
    """Load the library (building it first when it is absent and nvcc exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            from . import build
            build.build()
        L = ct.CDLL(LIB_PATH)
        vp, ll, i, f, sz = ct.c_void_p, ct.c_longlong, ct.c_int, ct.c_float, ct.c_size_t
        P = ct.POINTER
        L.pycbf_gb_abi_version.restype = i
        L.pycbf_gb_status_string.argtypes = [i]
        L.pycbf_gb_status_string.restype = ct.c_char_p
        L.pycbf_gb_last_cuda_error.restype = i
        L.pycbf_gb_workspace_bytes.argtypes = [P(RFInfo), i]
        L.pycbf_gb_workspace_bytes.restype = sz
        L.pycbf_gb_spline_coefficients.argtypes = [P(RFInfo), vp, vp, sz, vp]
        L.pycbf_gb_das_tabbed.argtypes = [P(RFInfo), vp, vp, vp, vp, vp, ll, vp, i, f, i, vp, vp,
                                          vp, sz, vp]
        L.pycbf_gb_tabbed_plan_bytes.argtypes = [ll, i, i]
        L.pycbf_gb_tabbed_plan_bytes.restype = sz
        L.pycbf_gb_tabbed_plan.argtypes = [P(RFInfo), vp, vp, vp, vp, ll, i, f, vp, sz, vp]
        L.pycbf_gb_das_tabbed_prefiltered.argtypes = [P(RFInfo), vp, vp, vp, vp, vp, ll, vp, f, i,
                                                      vp, vp, vp]
        L.pycbf_gb_das_synthetic.argtypes = [P(RFInfo), vp, P(SyntheticGeom), vp, i, i, vp, vp,
                                             sz, vp]
        L.pycbf_gb_tap_census_tabbed.argtypes = [P(RFInfo), vp, vp, vp, vp, ll, i, f, vp, vp, vp]
        L.pycbf_gb_tap_census_synthetic.argtypes = [P(RFInfo), P(SyntheticGeom), i, vp, vp, vp]
        L.pycbf_gb_synthetic_rx_mask.argtypes = [P(RFInfo), P(SyntheticGeom), vp, vp]
        L.pycbf_gb_dmas.argtypes = [vp, ll, ll, ll, vp, i, i, i, vp, vp]
        L.pycbf_gb_slsc.argtypes = [vp, vp, ll, i, i, i, i, i, vp, vp]
        L.pycbf_gb_slsc_kept_bytes.argtypes = [i, i, i]
        L.pycbf_gb_slsc_kept_bytes.restype = sz
        L.pycbf_gb_slsc_kept.argtypes = [vp, i, i, i, i, i, vp, sz, vp]
        L.pycbf_gb_slsc_with_kept.argtypes = [vp, vp, ll, i, i, i, i, i, vp, vp]
        L.pycbf_gb_fp32_probe.argtypes = [vp, i, i, vp]
        L.pycbf_gb_das_tabbed_cubic_noalloc.argtypes = [P(RFInfo), vp, vp, vp, vp, vp, ll, vp, f, i,
                                                        vp, vp]
        L.pycbf_gb_das_synthetic_slowness.argtypes = [P(RFInfo), vp, P(SyntheticGeom), vp, vp, i,
                                                      vp, vp]
        L.pycbf_gb_adjoint_workspace_bytes.argtypes = [P(RFInfo), ll]
        L.pycbf_gb_adjoint_workspace_bytes.restype = sz
        L.pycbf_gb_das_tabbed_adjoint.argtypes = [P(RFInfo), vp, vp, vp, vp, vp, ll, vp, f, i, vp,
                                                  vp, vp, vp, vp, sz, vp]
        L.pycbf_gb_das_tabbed_adjoint_planned.argtypes = [P(RFInfo), vp, vp, vp, vp, vp, ll, vp, f,
                                                          i, vp, vp, vp, vp, vp, vp, sz, vp]
        L.pycbf_gb_das_synthetic_adjoint.argtypes = [P(RFInfo), vp, P(SyntheticGeom), vp, vp, i,
                                                     vp, vp, vp, vp, sz, vp]
        L.pycbf_gb_batch_plan_bytes.argtypes = [P(BatchJob), i, i]
        L.pycbf_gb_batch_plan_bytes.restype = sz
        L.pycbf_gb_batch_plan.argtypes = [P(BatchJob), i, i, i, vp, sz, P(BatchInfo), vp]
        L.pycbf_gb_batch_run.argtypes = [vp, P(BatchInfo), i, i, vp]
        L.pycbf_gb_upsampled_bytes.argtypes = [P(RFInfo), i]
        L.pycbf_gb_upsampled_bytes.restype = sz
        L.pycbf_gb_upsample.argtypes = [P(RFInfo), vp, i, vp, sz, vp, sz, vp]
        L.pycbf_gb_poly_workspace_bytes.argtypes = [P(RFInfo), i, i]
        L.pycbf_gb_poly_workspace_bytes.restype = sz
        L.pycbf_gb_poly_coefficients.argtypes = [P(RFInfo), vp, i, i, vp, vp, sz, vp]
        L.pycbf_gb_das_tabbed_poly.argtypes = [P(RFInfo), vp, i, vp, vp, vp, vp, ll, vp, f, i, vp,
                                               vp]
        L.pycbf_gb_das_synthetic_poly.argtypes = [P(RFInfo), vp, i, P(SyntheticGeom), vp, i, vp,
                                                  vp]
        d = ct.c_double
        L.pycbf_gb_tables_2d.argtypes = [i, i, vp, i, vp, i, vp, i, vp, d, d, i, vp, vp, vp, vp, vp]
        L.pycbf_gb_demod.argtypes = [vp, ll, i, vp, i, vp, vp, vp]
        L.pycbf_gb_percentile_workspace_bytes.argtypes = [ll]
        L.pycbf_gb_percentile_workspace_bytes.restype = sz
        L.pycbf_gb_percentile.argtypes = [vp, ll, ll, d, vp, vp, sz, vp]
        L.pycbf_gb_log_compress.argtypes = [vp, ll, ll, vp, f, vp, vp]
        L.pycbf_gb_convert_i16.argtypes = [vp, ll, vp, vp]
        L.pycbf_gb_log_compress_percentile.argtypes = [vp, ll, ll, d, f, vp, vp, vp, sz, vp]
        L.pycbf_gb_das_tabbed_stall_test.argtypes = [P(RFInfo), vp, vp, vp, vp, vp, ll, vp, f, vp,
                                                     vp, ll, vp]
        for name in EXPORTS:
            if name not in ("pycbf_gb_abi_version", "pycbf_gb_status_string",
                            "pycbf_gb_last_cuda_error", "pycbf_gb_workspace_bytes",
                            "pycbf_gb_tabbed_plan_bytes", "pycbf_gb_adjoint_workspace_bytes",
                            "pycbf_gb_batch_plan_bytes", "pycbf_gb_upsampled_bytes",
                            "pycbf_gb_poly_workspace_bytes",
                            "pycbf_gb_percentile_workspace_bytes"):
                getattr(L, name).restype = i
        _lib = L
        return L


def check(status: int, what: str) -> None:
    if status == OK:
        return
    L = load()
    msg = L.pycbf_gb_status_string(status).decode()
    if status == ECUDA:
        msg += f" (cudaError {L.pycbf_gb_last_cuda_error()})"
    raise GPUError(f"{what}: {msg}")

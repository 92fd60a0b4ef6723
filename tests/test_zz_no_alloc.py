"""The allocation-free cubic entry point, for callers that cannot call cudaMalloc.

Such callers (a runtime reaching CUDA only through the C ABI, a service with a
device-memory budget fixed at start-up) cannot hand pycbf_gb_das_tabbed the
workspace it needs for the spline coefficients; pycbf_gb_das_tabbed_cubic_noalloc
keeps them in a device array inside the library instead.  This file runs last
(pytest collects it last) and needs nothing from the other test files.
"""
import ctypes as ct
import os

import numpy as np
import pytest
import torch

from gpu_util import assert_image_close
from pycbf_gb300 import _lib

HERE = os.path.dirname(os.path.abspath(__file__))


def _case():
    with np.load(os.path.join(HERE, "golden", "tabbed_pw_small.npz")) as z:
        return {k: z[k] for k in z.files}


def _dev(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _p(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


# storage type, frames per call
CASES = [(_lib.F32, 1), (_lib.F32, 2), (_lib.I16, 1), (_lib.F16, 1)]


def _frames(case, dtype, nframes, seed):
    """Channel data for one call: the golden frame scaled, plus seeded frames."""
    rng = np.random.default_rng(seed)
    rf = case["rf"].astype(np.float64)
    frames = [rf * (1.0 + 0.25 * seed)] + [rng.normal(size=rf.shape) * np.std(rf)
                                           for _ in range(nframes - 1)]
    rf = np.stack(frames) if nframes > 1 else frames[0]
    if dtype == _lib.I16:
        return _dev(np.round(rf / np.max(np.abs(rf)) * 20000), torch.int16)
    return _dev(rf, torch.float16 if dtype == _lib.F16 else torch.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,nframes", CASES)
def test_noalloc_matches_workspace_entry_point_twice(dtype, nframes):
    L = _lib.load()
    case = _case()
    ntx, nrx = case["tautx"].shape[0], case["taurx"].shape[0]
    np_ = case["tautx"].shape[1]
    tabs = [_dev(case[k]) for k in ("tautx", "apodtx", "taurx", "apodrx")]
    info = _lib.RFInfo(ntx, nrx, 0, float(case["t0"]), float(case["dt"]), int(case["nt"]), nframes,
                       dtype)
    need = L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["cubic"])
    assert 0 < need <= _lib.NOALLOC_SCRATCH_BYTES
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    for seed in (1, 2):  # two calls in a row, different channel data
        rf = _frames(case, dtype, nframes, seed)
        for sumtype in (_lib.SUMTYPE["tx_and_rx"], _lib.SUMTYPE["tx_only"]):
            size = nframes * (np_ if sumtype == _lib.SUMTYPE["tx_and_rx"] else nrx * np_)
            ref = torch.empty(size, device="cuda")
            out = torch.full((size,), float("nan"), device="cuda")
            st = L.pycbf_gb_das_tabbed(ct.byref(info), _p(rf), *map(_p, tabs), np_, None,
                                       _lib.INTERP["cubic"], 0.01, sumtype, None, _p(ref), _p(ws),
                                       need, stream)
            assert st == _lib.OK
            st = L.pycbf_gb_das_tabbed_cubic_noalloc(ct.byref(info), _p(rf), *map(_p, tabs), np_,
                                                     None, 0.01, sumtype, _p(out), stream)
            assert st == _lib.OK, L.pycbf_gb_status_string(st)
            torch.cuda.synchronize()
            assert_image_close(out.cpu().numpy(), ref.cpu().numpy(),
                               what=f"dtype {dtype}, {nframes} frame(s), call {seed}, sum {sumtype}")


def _noalloc_status(info, np_=0, sumtype=3, thresh=0.01):
    """Status of a call with placeholder pointers; with np_ == 0 a valid call
    queues nothing, so no placeholder is ever dereferenced."""
    L = _lib.load()
    p = ct.c_void_p(256)
    return L.pycbf_gb_das_tabbed_cubic_noalloc(ct.byref(info), p, p, p, p, p, np_, None, thresh,
                                               sumtype, p, None)


def test_noalloc_size_limit_edge():
    """Coefficients of exactly PYCBF_GB_NOALLOC_SCRATCH_BYTES are accepted; one
    16-byte record more is rejected (host checks only: no work is queued)."""
    L = _lib.load()
    at_limit = _lib.RFInfo(1, 1 << 20, 0, 0.0, 1.0, 4, 1, _lib.F32)
    assert L.pycbf_gb_workspace_bytes(ct.byref(at_limit), _lib.INTERP["cubic"]) == \
        _lib.NOALLOC_SCRATCH_BYTES
    assert _noalloc_status(at_limit) == _lib.OK
    past = _lib.RFInfo(1, 838861, 0, 0.0, 1.0, 5, 1, _lib.F32)
    assert L.pycbf_gb_workspace_bytes(ct.byref(past), _lib.INTERP["cubic"]) == \
        _lib.NOALLOC_SCRATCH_BYTES + 16
    assert _noalloc_status(past) == _lib.ERANGE
    # 16-bit storage: 8-byte records, so twice the samples fit
    half = _lib.RFInfo(2, 1 << 20, 0, 0.0, 1.0, 4, 1, _lib.F16)
    assert _noalloc_status(half) == _lib.OK
    assert _noalloc_status(_lib.RFInfo(64, 256, 0, 0.0, 1.0, 4096, 1, _lib.F32)) == _lib.ERANGE


def test_noalloc_rejects_bad_arguments_before_any_work():
    """The delay-and-sum's own checks run before the prefilter is queued."""
    ok = _lib.RFInfo(2, 4, 0, 0.0, 1.0, 16, 1, _lib.F32)
    assert _noalloc_status(ok, np_=-1) == _lib.ERANGE
    assert _noalloc_status(ok, np_=10, sumtype=9) == _lib.EINVAL
    assert _noalloc_status(ok, np_=10, thresh=float("nan")) == _lib.EINVAL
    assert _noalloc_status(_lib.RFInfo(0, 4, 0, 0.0, 1.0, 16, 1, _lib.F32)) == _lib.EINVAL
    L = _lib.load()
    p = ct.c_void_p(256)
    st = L.pycbf_gb_das_tabbed_cubic_noalloc(ct.byref(ok), p, None, p, p, p, 10, None, 0.01, 3, p,
                                             None)
    assert st == _lib.EINVAL

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

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _case():
    with np.load(os.path.join(HERE, "golden", "tabbed_pw_small.npz")) as z:
        case = {k: z[k] for k in z.files}
    rng = np.random.default_rng(17)
    # a second frame so that the array is reused with different contents
    case["rf2"] = rng.normal(size=case["rf"].shape).astype(np.float32)
    return case


def _dev(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _p(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


def test_noalloc_matches_workspace_entry_point_twice():
    L = _lib.load()
    case = _case()
    ntx, nrx = case["tautx"].shape[0], case["taurx"].shape[0]
    np_ = case["tautx"].shape[1]
    tabs = [_dev(case[k]) for k in ("tautx", "apodtx", "taurx", "apodrx")]
    info = _lib.RFInfo(ntx, nrx, 0, float(case["t0"]), float(case["dt"]), int(case["nt"]), 1,
                       _lib.F32)
    need = L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["cubic"])
    assert 0 < need <= _lib.NOALLOC_SCRATCH_BYTES
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    for key in ("rf", "rf2"):  # two calls in a row, different channel data
        rf = _dev(case[key])
        for sumtype in (_lib.SUMTYPE["tx_and_rx"], _lib.SUMTYPE["tx_only"]):
            size = np_ if sumtype == _lib.SUMTYPE["tx_and_rx"] else nrx * np_
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
            assert_image_close(out.cpu().numpy(), ref.cpu().numpy(), what=f"{key}/{sumtype}")


def test_noalloc_rejects_channel_data_beyond_its_array():
    L = _lib.load()
    info = _lib.RFInfo(64, 256, 0, 0.0, 1.0, 4096, 1, _lib.F32)  # 1 GiB of coefficients
    p = ct.c_void_p(256)
    st = L.pycbf_gb_das_tabbed_cubic_noalloc(ct.byref(info), p, p, p, p, p, 10, None, 0.01, 3, p,
                                             None)
    assert st == _lib.ERANGE

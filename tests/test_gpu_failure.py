"""The staged kernel's bounded-wait failure path, exercised without a fault.

pycbf_gb_das_tabbed_stall_test runs the cubic staged delay-and-sum with the
first receive of every tile announcing its bytes without issuing its copies,
so that receive's mbarrier wait runs out (after ~0.5 ms here).  Every CTA that gives
up writes NaN to its pixels, drains its copies (bounded) and sets the plan's
status word; the launch returns normally, the context stays usable and the
next ordinary call gives the ordinary image."""
import ctypes as ct
import time

import numpy as np
import pytest

from pycbf_gb300 import _lib


@pytest.mark.gpu
def test_wait_runs_out_and_context_survives():
    import torch

    import pycbf_gb300 as pg
    from pycbf_gb300 import phantom
    w = phantom.linear_pw_tabbed(nx=64, nz=128, n_speckle=800, device="cuda")
    bf = pg.TabbedBeamformer(tautx=w.tautx, taurx=w.taurx, apodtx=w.apodtx, apodrx=w.apodrx,
                             t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": "cubic"})
    assert bf._plan is not None
    want = bf(w.rf, out_as_numpy=False).clone()
    assert bf.kernel_status() == 0

    L = _lib.load()
    info = bf._rfinfo(1)
    rf = torch.as_tensor(np.asarray(w.rf), device="cuda").contiguous()
    need = L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["cubic"])
    coef = torch.empty(need, dtype=torch.uint8, device="cuda")
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: ct.c_void_p(t.data_ptr()) if t is not None else None
    assert L.pycbf_gb_spline_coefficients(ct.byref(info), P(rf), P(coef), need, stream) == 0
    tautx, apodtx, taurx, apodrx = bf._tables
    out = torch.zeros(bf.nop, device="cuda")
    t = time.perf_counter()
    st = L.pycbf_gb_das_tabbed_stall_test(ct.byref(info), P(coef), P(tautx), P(apodtx), P(taurx),
                                          P(apodrx), bf.nop, P(bf._pixel_index), 0.01,
                                          P(bf._plan), P(out), 1 << 20, stream)
    assert st == 0
    torch.cuda.synchronize()                       # no CUDA error: the kernel returned
    elapsed = time.perf_counter() - t
    assert bf.kernel_status() == 1
    assert torch.isnan(out).any()
    assert elapsed < 30.0

    # sticky until reset; the next ordinary call is unaffected
    again = bf(w.rf, out_as_numpy=False)
    assert torch.equal(again, want)
    assert bf.kernel_status() == 1
    bf.reset_kernel_status()
    assert bf.kernel_status() == 0
    assert torch.equal(bf(w.rf, out_as_numpy=False), want)
    assert bf.kernel_status() == 0


def test_stall_hook_validates_first():
    L = _lib.load()
    p = ct.c_void_p(16)
    info = _lib.RFInfo(2, 3, 0, 0.0, 1.0, 16, 1, _lib.F32)
    call = lambda **k: L.pycbf_gb_das_tabbed_stall_test(
        ct.byref(info), k.get("coef", p), p, p, p, p, 10, None, 0.01, k.get("plan", p), p,
        k.get("cycles", 1 << 20), None)
    assert call(plan=None) == _lib.EINVAL
    assert call(cycles=10) == _lib.ERANGE
    assert call(cycles=1 << 40) == _lib.ERANGE
    assert call(coef=ct.c_void_p(8)) == _lib.EINVAL

"""int16 channel data (raw converter counts): copied to the device as int16 and
converted exactly to float32 by the first kernel that reads it -- inside the
spline prefilter for cubic, one conversion pass for nearest/linear, and
pycbf_gb_convert_i16 ahead of the paths that take float data.  Every image
must equal, bit for bit, the image of the same counts passed as float32."""
import ctypes as ct

import numpy as np
import pytest

from pycbf_gb300 import _lib


def _info(**kw):
    base = dict(ntx=2, nrx=3, ndim=0, t0=0.0, dt=1.0, nt=16, nframes=1, dtype=_lib.I16)
    base.update(kw)
    return _lib.RFInfo(**base)


def test_i16_workspace_and_validation():
    L = _lib.load()
    info = _info()
    nsamp = 2 * 3 * 16
    assert L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["cubic"]) == nsamp * 16
    assert L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["nearest"]) == nsamp * 4
    assert L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["linear"]) == nsamp * 4
    assert L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["akima"]) == 0
    assert L.pycbf_gb_workspace_bytes(ct.byref(_info(dtype=_lib.F32)),
                                      _lib.INTERP["nearest"]) == 0
    p = ct.c_void_p(16)
    # nearest with int16 needs the conversion workspace
    assert L.pycbf_gb_das_tabbed(ct.byref(info), p, p, p, p, p, 10, None, 0, 0.01, 3, None, p,
                                 None, 0, None) == _lib.EWORKSPACE
    # entry points that take float data only
    assert L.pycbf_gb_upsample(ct.byref(info), p, 2, p, 1 << 20, p, 1 << 20, None) == _lib.EUNSUPPORTED
    assert L.pycbf_gb_poly_coefficients(ct.byref(info), p, _lib.INTERP["akima"], 0, None, p,
                                        1 << 20, None) == _lib.EUNSUPPORTED
    assert L.pycbf_gb_das_tabbed_adjoint(ct.byref(info), p, p, p, p, p, 10, None, 0.01, 3, p,
                                         None, p, p, None, 0, None) == _lib.EUNSUPPORTED
    assert L.pycbf_gb_convert_i16(None, 4, p, None) == _lib.EINVAL
    assert L.pycbf_gb_convert_i16(p, -1, p, None) == _lib.EINVAL
    assert L.pycbf_gb_convert_i16(p, 0, p, None) == _lib.OK


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _counts(rf, full=30000):
    rf = np.asarray(rf.cpu() if hasattr(rf, "cpu") else rf, np.float64)
    return np.round(rf / np.abs(rf).max() * full).astype(np.int16)


@pytest.fixture(scope="module")
def tabbed_small():
    from pycbf_gb300 import phantom
    w = phantom.linear_pw_tabbed(nx=48, nz=96, n_speckle=1000, device="cuda")
    return w


def _tabbed(w, **kw):
    import pycbf_gb300 as pg
    return pg.TabbedBeamformer(tautx=w.tautx, taurx=w.taurx, apodtx=w.apodtx, apodrx=w.apodrx,
                               t0=w.t0, dt=w.dt, nt=w.nt, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("interp", [{"kind": "cubic"}, {"kind": "nearest"}, {"kind": "linear"},
                                    {"kind": "linear", "reference_floor": True},
                                    {"kind": "nearest", "usf": 4},
                                    {"kind": "korder_cubic", "k": 8}, {"kind": "akima"}])
@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only"])
def test_tabbed_int16_equals_float_counts(tabbed_small, interp, sumtype):
    import torch
    rfi = _counts(tabbed_small.rf)
    bf = _tabbed(tabbed_small, interp=interp, sumtype=sumtype)
    a = bf(rfi, out_as_numpy=False)
    b = bf(rfi.astype(np.float32), out_as_numpy=False)
    assert torch.equal(a, b)
    assert float(b.abs().max()) > 0


@pytest.mark.gpu
def test_int16_frames_torch_and_storage(tabbed_small):
    import torch
    rfi = _counts(tabbed_small.rf)
    frames = np.stack([rfi, (rfi // 2).astype(np.int16), -rfi])
    bf = _tabbed(tabbed_small, interp={"kind": "cubic"})
    want = bf(frames.astype(np.float32), out_as_numpy=False)
    assert torch.equal(bf(frames, out_as_numpy=False), want)
    pinned = torch.from_numpy(frames).pin_memory()
    assert torch.equal(bf(pinned, out_as_numpy=False), want)
    assert torch.equal(bf(pinned.cuda(), out_as_numpy=False), want)
    # float16 storage: the counts are converted to float32, then stored as float16
    bfh = _tabbed(tabbed_small, interp={"kind": "cubic"}, storage="float16")
    assert torch.equal(bfh(rfi, out_as_numpy=False), bfh(rfi.astype(np.float32), out_as_numpy=False))


@pytest.mark.gpu
def test_int16_golden_case_vs_oracle(golden):
    import pycbf_gb300 as pg
    from gpu_util import assert_image_close
    from oracle import oracle
    case = golden("tabbed_pw_small.npz")
    rfi = _counts(case["rf"])
    for kind in ("cubic", "nearest"):
        bf = pg.TabbedBeamformer(tautx=case["tautx"], taurx=case["taurx"], apodtx=case["apodtx"],
                                 apodrx=case["apodrx"], t0=float(case["t0"]), dt=float(case["dt"]),
                                 nt=int(case["nt"]), interp={"kind": kind})
        want = oracle.das_tabbed(rfi.astype(np.float32), case["tautx"], case["apodtx"],
                                 case["taurx"], case["apodrx"], float(case["t0"]),
                                 float(case["dt"]), int(case["nt"]), interp=kind)
        assert_image_close(bf(rfi), want, what=f"int16 {kind}")


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["cubic", "nearest"])
def test_synthetic_int16_equals_float_counts(kind):
    import torch

    import pycbf_gb300 as pg
    from pycbf_gb300 import phantom
    w = phantom.linear_pw_synthetic(nele=32, nsteer=5, nt=1024, nx=32, nz=64, n_speckle=500,
                                    xlim=(-4e-3, 4e-3), zlim=(5e-3, 15e-3), device="cuda")
    g = w.geometry
    keys = ("ovectx", "nvectx", "doftx", "alatx", "t0tx", "ovecrx", "nvecrx", "alarx", "c0", "pnts")
    bf = pg.SyntheticBeamformer(**{k: g[k] for k in keys}, t0=w.t0, dt=w.dt, nt=w.nt,
                                interp={"kind": kind})
    rfi = _counts(w.rf)
    assert torch.equal(bf(rfi, out_as_numpy=False), bf(rfi.astype(np.float32), out_as_numpy=False))


@pytest.mark.gpu
def test_convert_kernel_vector_and_scalar_paths():
    import torch
    L = _lib.load()
    src = torch.randint(-32768, 32767, ((1 << 16) + 5,), dtype=torch.int16, device="cuda")
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    for off in (0, 1, 3):      # 16-byte aligned, and two misaligned starts
        s = src[off:]
        d = torch.empty(s.numel() + 4, dtype=torch.float32, device="cuda")[off % 4:][: s.numel()]
        assert L.pycbf_gb_convert_i16(ct.c_void_p(s.data_ptr()), s.numel(),
                                      ct.c_void_p(d.data_ptr()), stream) == _lib.OK
        assert torch.equal(d, s.float())

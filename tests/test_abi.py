"""The C-ABI library builds, loads and exports every symbol its header declares;
host-side validation returns status codes before any CUDA call (CPU only)."""
import ctypes as ct
import os
import re
import subprocess

import pytest

from pycbf_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(pycbf_gb_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(L, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r"\bT (pycbf_gb_\w+)", out))
    assert syms <= exported
    assert set(_lib.EXPORTS) <= syms


def test_abi_version_and_status_strings():
    L = _lib.load()
    assert L.pycbf_gb_abi_version() == 1
    assert L.pycbf_gb_status_string(0) == b"ok"
    assert b"workspace" in L.pycbf_gb_status_string(_lib.EWORKSPACE)


def _info(**kw):
    base = dict(ntx=2, nrx=3, ndim=0, t0=0.0, dt=1.0, nt=16, nframes=1, dtype=_lib.F32)
    base.update(kw)
    return _lib.RFInfo(**base)


def test_workspace_bytes():
    L = _lib.load()
    info = _info()
    assert L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["cubic"]) == 2 * 3 * 16 * 16
    assert L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["nearest"]) == 0
    half = _info(dtype=_lib.F16, nframes=4)
    assert L.pycbf_gb_workspace_bytes(ct.byref(half), _lib.INTERP["cubic"]) == 4 * 2 * 3 * 16 * 8


@pytest.mark.parametrize("bad,code", [
    (dict(ntx=0), _lib.EINVAL), (dict(nt=0), _lib.EINVAL), (dict(dt=0.0), _lib.EINVAL),
    (dict(dt=float("nan")), _lib.EINVAL), (dict(dtype=7), _lib.EINVAL),
    (dict(nframes=70000), _lib.ERANGE), (dict(nt=1 << 22), _lib.ERANGE),
])
def test_tabbed_rejects_bad_rfinfo(bad, code):
    L = _lib.load()
    info = _info(**bad)
    p = ct.c_void_p(16)  # never dereferenced: validation fails first
    st = L.pycbf_gb_das_tabbed(ct.byref(info), p, p, p, p, p, 10, None, 2, 0.01, 3, None, p, p,
                               1 << 20, None)
    assert st == code


def test_size_limits_return_erange():
    """Each limit the header lists, one past it; every call is rejected before
    any CUDA call (the pointers are never dereferenced)."""
    L = _lib.load()
    p = ct.c_void_p(16)

    def tabbed(info, interp=0, sumtype=3, ws=None, wsb=0):
        return L.pycbf_gb_das_tabbed(ct.byref(info), p, p, p, p, p, 10, None, interp, 0.01,
                                     sumtype, None, p, ws, wsb, None)

    assert tabbed(_info(ntx=(1 << 20) + 1)) == _lib.ERANGE
    assert tabbed(_info(nrx=(1 << 20) + 1)) == _lib.ERANGE
    assert tabbed(_info(ntx=455)) == _lib.ERANGE
    assert tabbed(_info(ntx=228), sumtype=2) == _lib.ERANGE
    cubic = _info(nt=18001)
    need = L.pycbf_gb_workspace_bytes(ct.byref(cubic), _lib.INTERP["cubic"])
    assert tabbed(cubic, interp=_lib.INTERP["cubic"], ws=p, wsb=need) == _lib.ERANGE

    geo = _lib.SyntheticGeom(**{n: 16 for n, _ in _lib.SyntheticGeom._fields_
                                if n not in ("np", "c0")}, np=10, c0=1540.0)
    synth = lambda info, sumtype=3: L.pycbf_gb_das_synthetic(
        ct.byref(info), p, ct.byref(geo), None, 0, sumtype, p, None, 0, None)
    assert synth(_info(ndim=2, ntx=455)) == _lib.ERANGE
    assert synth(_info(ndim=2, ntx=228), sumtype=2) == _lib.ERANGE


def test_tabbed_rejects_null_and_codes():
    L = _lib.load()
    info = _info()
    p = ct.c_void_p(16)
    call = lambda **kw: L.pycbf_gb_das_tabbed(
        ct.byref(info), kw.get("rf", p), p, p, p, p, kw.get("np", 10), None, kw.get("interp", 2),
        kw.get("thresh", 0.01), kw.get("sum", 3), None, kw.get("out", p), kw.get("ws", p),
        kw.get("wsb", 1 << 20), None)
    assert call(rf=None) == _lib.EINVAL
    assert call(out=None) == _lib.EINVAL
    assert call(interp=9) == _lib.EINVAL
    assert call(sum=6) == _lib.EINVAL
    assert call(thresh=float("nan")) == _lib.EINVAL
    assert call(np=-1) == _lib.ERANGE
    assert call(np=0) == _lib.OK          # nothing to do
    assert call(ws=None) == _lib.EWORKSPACE
    assert call(wsb=100) == _lib.EWORKSPACE
    assert call(ws=ct.c_void_p(8)) == _lib.EINVAL  # misaligned workspace


def test_plan_validation():
    L = _lib.load()
    info = _info()
    p = ct.c_void_p(16)
    # header, 8 tile records (4 words + 16 per receive), tile order, block counters,
    # (pad to 16 bytes), 8 x 2 block items (int4; receive blocks of 64), 8 x 2 x 128
    # partial sums
    head = 4 + 8 * (4 + 128 * 16) + 8 + 8
    head = (head + 3) // 4 * 4
    assert L.pycbf_gb_tabbed_plan_bytes(1000, 11, 128) == 4 * (head + 4 * 8 * 2 + 8 * 2 * 128)
    assert L.pycbf_gb_tabbed_plan_bytes(0, 11, 128) == 0
    call = lambda **kw: L.pycbf_gb_tabbed_plan(
        ct.byref(kw.get("info", info)), p, p, p, p, kw.get("np", 10), kw.get("interp", 2), 0.01,
        kw.get("plan", p), kw.get("nb", 1 << 20), None)
    assert call(plan=None) == _lib.EINVAL
    assert call(interp=3) == _lib.EINVAL
    assert call(nb=8) == _lib.EWORKSPACE
    assert call(plan=ct.c_void_p(20)) == _lib.EWORKSPACE
    assert call(info=_info(ntx=13)) == _lib.EUNSUPPORTED


def test_synthetic_and_coherence_validation():
    L = _lib.load()
    info = _info(ndim=1)
    geo = _lib.SyntheticGeom()
    p = ct.c_void_p(16)
    assert L.pycbf_gb_das_synthetic(ct.byref(info), p, ct.byref(geo), None, 2, 3, p, p, 1 << 20,
                                    None) == _lib.EINVAL
    assert L.pycbf_gb_dmas(None, 1, 4, 10, p, 2, 0, 1, p, None) == _lib.EINVAL
    assert L.pycbf_gb_dmas(p, 1, 4, 10, p, 2, 3, 1, p, None) == _lib.EINVAL
    assert L.pycbf_gb_slsc(p, p, 1, 8, 4, 4, 40, 2, p, None) == _lib.ERANGE
    assert L.pycbf_gb_slsc(p, p, 1, 8, 4, 4, 4, 40, p, None) == _lib.ERANGE
    assert L.pycbf_gb_slsc(p, None, 1, 8, 4, 4, 4, 2, p, None) == _lib.EINVAL


def test_adjoint_workspace_bytes():
    L = _lib.load()
    info = _info(ntx=2, nrx=3, nt=16, nframes=2)
    nch = 2 * 2 * 3
    # parts: enough (channel, part) blocks to fill the GPU, >= 2048 pixels per part
    lp = (16 + 1 + 3) & ~3
    grad = lambda np_: (2 * 3 * np_ * 4 + 255) // 256 * 256  # gathered upstream gradient
    live = lambda np_: (3 * ((np_ + 127) // 128) + 255) // 256 * 256  # receive x tile flags
    n = L.pycbf_gb_adjoint_workspace_bytes(ct.byref(info), 100000)
    parts = min(100000 // 2048, (11264 + nch - 1) // nch, 64)
    assert n == grad(100000) + parts * nch * 2 * lp * 4 + live(100000)
    assert L.pycbf_gb_adjoint_workspace_bytes(ct.byref(info), 100) == \
        grad(100) + nch * 2 * lp * 4 + live(100)
    assert L.pycbf_gb_adjoint_workspace_bytes(ct.byref(info), 0) == 0


def test_adjoint_entry_points_validate_first():
    L = _lib.load()
    p = ct.c_void_p(16)
    info = _info()
    tab = lambda **kw: L.pycbf_gb_das_tabbed_adjoint(
        ct.byref(kw.get("info", info)), kw.get("coef", p), p, p, p, p, 10, None, 0.01,
        kw.get("sum", 3), kw.get("gout", p), kw.get("grf", None), p, p, kw.get("ws", None),
        kw.get("wsb", 0), None)
    assert tab(sum=0) == _lib.EUNSUPPORTED
    assert tab(sum=5) == _lib.EUNSUPPORTED
    assert tab(gout=None) == _lib.EINVAL
    assert tab(coef=ct.c_void_p(8)) == _lib.EINVAL          # coefficients 16-byte aligned
    assert tab(info=_info(ntx=129)) == _lib.ERANGE
    assert tab(info=_info(nt=20000)) == _lib.ERANGE
    assert tab(grf=p) == _lib.EWORKSPACE                    # grad_rf needs the workspace
    assert tab(grf=p, ws=p, wsb=1) == _lib.EWORKSPACE
    planned = lambda **kw: L.pycbf_gb_das_tabbed_adjoint_planned(
        ct.byref(kw.get("info", info)), p, p, p, p, p, 10, None, 0.01, kw.get("sum", 3),
        kw.get("plan", None), kw.get("gout", p), None, p, p, None, 0, None)
    assert planned(plan=ct.c_void_p(8)) == _lib.EINVAL     # plans are 16-byte aligned
    assert planned(sum=0) == _lib.EUNSUPPORTED
    assert planned(gout=None) == _lib.EINVAL
    assert planned(info=_info(ntx=129)) == _lib.ERANGE
    geo = _lib.SyntheticGeom()
    sinfo = _info(ndim=2)
    assert L.pycbf_gb_das_synthetic_adjoint(ct.byref(sinfo), p, ct.byref(geo), p, None, 3, p,
                                            None, p, None, 0, None) == _lib.EINVAL
    assert L.pycbf_gb_das_synthetic_slowness(ct.byref(_info(ndim=4)), p, ct.byref(geo), p, None,
                                             3, p, None) == _lib.EINVAL


def test_batch_plan_validates_jobs():
    L = _lib.load()
    p = ct.c_void_p(16)
    j = _lib.BatchJob()
    j.geom = 0
    j.rf = _info()
    j.rfdata = j.coef = j.out = 16
    j.tautx = j.apodtx = j.taurx = j.apodrx = 16
    j.np = 300
    j.thresh = 0.01
    jobs = (_lib.BatchJob * 2)(j, j)
    # 300 pixels = 3 tiles of 128: 3 items, or 2 of two tiles
    hdr, desc = 16, None
    n1 = L.pycbf_gb_batch_plan_bytes(jobs, 2, 1)
    n2 = L.pycbf_gb_batch_plan_bytes(jobs, 2, 2)
    assert n1 - n2 == 2 * 8 * (3 - 2)
    assert L.pycbf_gb_batch_plan_bytes(jobs, 2, 9) == 0
    info = _lib.BatchInfo()
    plan = lambda js, n=2, tpi=1, order=1, nbytes=n1: L.pycbf_gb_batch_plan(
        js, n, tpi, order, p, nbytes, ct.byref(info), None)
    assert plan(jobs, nbytes=n1 - 1) == _lib.EWORKSPACE
    assert plan(jobs, order=2) == _lib.EINVAL
    bad = _lib.BatchJob.from_buffer_copy(j)
    bad.rf.nframes = 2
    assert plan((_lib.BatchJob * 2)(j, bad)) == _lib.EINVAL
    bad = _lib.BatchJob.from_buffer_copy(j)
    bad.coef = 8
    assert plan((_lib.BatchJob * 2)(j, bad)) == _lib.EINVAL
    bad = _lib.BatchJob.from_buffer_copy(j)
    bad.rf.dtype = _lib.I16  # int16 counts: not a storage type of the batch
    assert plan((_lib.BatchJob * 2)(j, bad)) == _lib.EUNSUPPORTED
    bad = _lib.BatchJob.from_buffer_copy(j)
    bad.geom = 1  # synthetic without geometry
    assert plan((_lib.BatchJob * 2)(j, bad)) == _lib.EINVAL
    assert L.pycbf_gb_batch_run(p, ct.byref(info), 6, 10, None) == _lib.EINVAL


def test_slsc_kept_limits():
    """Host checks only: the kept-set entry points refuse what the register
    kernel cannot run (ERANGE) and missing pointers (EINVAL)."""
    L = _lib.load()
    p = 256
    assert L.pycbf_gb_slsc_kept(p, 257, 4, 4, 16, 3, p, 1 << 20, None) == _lib.ERANGE
    assert L.pycbf_gb_slsc_kept(p, 64, 4, 4, 17, 3, p, 1 << 20, None) == _lib.ERANGE
    assert L.pycbf_gb_slsc_kept(p, 64, 4, 4, 16, 4, p, 1 << 20, None) == _lib.ERANGE
    assert L.pycbf_gb_slsc_kept(None, 64, 4, 4, 16, 3, p, 1 << 20, None) == _lib.EINVAL
    assert L.pycbf_gb_slsc_with_kept(p, None, 1, 64, 4, 4, 16, 3, p, None) == _lib.EINVAL
    assert L.pycbf_gb_slsc_with_kept(p, p, 1, 64, 4, 4, 17, 3, p, None) == _lib.ERANGE
    assert L.pycbf_gb_slsc_kept_bytes(0, 4, 4) == 0

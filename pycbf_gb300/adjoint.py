"""Differentiable cubic delay-and-sum (no counterpart in the reference, whose
beamformers are forward-only).

Two ``torch.autograd.Function``s over the adjoint kernels of the C ABI
(``pycbf_gb_das_tabbed_adjoint``, ``pycbf_gb_das_synthetic_adjoint``):

``das_tabbed(rf, tautx, taurx, apodtx, apodrx, t0=, dt=, ...)``
    the Tabbed delay-and-sum of the reference's float32 C path
    (pycbf/cpu/pycbf.c:179-207 per channel), differentiable with respect to
    the channel data and both delay tables;
``das_synthetic_slowness(rf, slowness, geometry, ...)``
    the Synthetic delay-and-sum with every delay written as path length x
    slowness of the pixel (s = 1/c for a uniform medium), differentiable with
    respect to the channel data and the per-pixel slowness.

Gradients with respect to the channel data are the transpose of the
interpolation followed by the adjoint of the spline prefilter, accumulated
without atomics in a fixed order (bitwise reproducible).  Gradients with
respect to the delays use the analytic derivative of the cubic interpolant;
delays are recomputed in the backward pass, never stored per tap.  The
apodization is not differentiated, and the tap decisions (range, threshold,
knot) are those of the forward pass.

Pixel order: the tables / slowness are in the order the kernels walk them;
``pixel_index`` (int32, optional) maps that order to the image order, as for
the forward entry points.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

__all__ = ["das_tabbed", "das_synthetic_slowness", "SUMTYPES"]

SUMTYPES = ("tx_and_rx", "tx_only")
_DTYPE = {torch.float32: _lib.F32, torch.float16: _lib.F16, torch.bfloat16: _lib.BF16}


def _ptr(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass(frozen=True)
class _Spec:
    t0: float
    dt: float
    thresh: float
    sumtype: int
    ndim: int = 0


def _check_rf(rf: torch.Tensor):
    if not (isinstance(rf, torch.Tensor) and rf.is_cuda):
        raise ValueError("rf must be a CUDA tensor")
    if rf.dtype not in _DTYPE:
        raise ValueError(f"rf dtype must be one of {list(_DTYPE)}, got {rf.dtype}")
    if rf.ndim not in (3, 4):
        raise ValueError("rf must be (ntx, nrx, nt) or (nframes, ntx, nrx, nt)")


def _info(rf4: torch.Tensor, spec: _Spec) -> _lib.RFInfo:
    nf, ntx, nrx, nt = rf4.shape
    return _lib.RFInfo(ntx, nrx, spec.ndim, float(np.float32(spec.t0)), float(np.float32(spec.dt)),
                       nt, nf, _DTYPE[rf4.dtype])


def _coefficients(L, rf4: torch.Tensor, info) -> torch.Tensor:
    need = L.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["cubic"])
    coef = torch.empty(need, dtype=torch.uint8, device=rf4.device)
    _lib.check(L.pycbf_gb_spline_coefficients(ct.byref(info), _ptr(rf4), _ptr(coef), need,
                                              _stream()), "pycbf_gb_spline_coefficients")
    return coef


def _out_shape(rf4, np_, sumtype):
    nf, _, nrx, _ = rf4.shape
    return (nf, np_) if sumtype == _lib.SUMTYPE["tx_and_rx"] else (nf, nrx, np_)


class _TabbedDAS(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rf4, tautx, taurx, apodtx, apodrx, pixel_index, spec, plan=None):
        L = _lib.load()
        info = _info(rf4, spec)
        coef = _coefficients(L, rf4, info)
        np_ = tautx.shape[1]
        out = torch.empty(_out_shape(rf4, np_, spec.sumtype), dtype=torch.float32,
                          device=rf4.device)
        st = L.pycbf_gb_das_tabbed_prefiltered(
            ct.byref(info), _ptr(coef), _ptr(tautx), _ptr(apodtx), _ptr(taurx), _ptr(apodrx), np_,
            _ptr(pixel_index), float(np.float32(spec.thresh)), spec.sumtype, _ptr(plan), _ptr(out),
            _stream())
        _lib.check(st, "pycbf_gb_das_tabbed_prefiltered")
        ctx.save_for_backward(coef, tautx, taurx, apodtx, apodrx)
        ctx.plan = plan
        ctx.pixel_index = pixel_index
        ctx.spec = spec
        ctx.rf_meta = (tuple(rf4.shape), rf4.dtype)
        return out

    @staticmethod
    def backward(ctx, gout):
        coef, tautx, taurx, apodtx, apodrx = ctx.saved_tensors
        shape, dtype = ctx.rf_meta
        spec = ctx.spec
        need_rf, need_ttx, need_trx = ctx.needs_input_grad[0:3]
        L = _lib.load()
        info = _lib.RFInfo(shape[1], shape[2], 0, float(np.float32(spec.t0)),
                           float(np.float32(spec.dt)), shape[3], shape[0], _DTYPE[dtype])
        np_ = tautx.shape[1]
        dev = coef.device
        gout = gout.to(torch.float32).contiguous()
        g_rf = torch.empty(shape, dtype=torch.float32, device=dev) if need_rf else None
        g_ttx = torch.empty_like(tautx) if need_ttx else None
        g_trx = torch.empty_like(taurx) if need_trx else None
        ws, nws = None, 0
        if need_rf or ctx.pixel_index is not None:
            nws = L.pycbf_gb_adjoint_workspace_bytes(ct.byref(info), np_)
            ws = torch.empty(nws, dtype=torch.uint8, device=dev)
        if need_rf or need_ttx or need_trx:
            st = L.pycbf_gb_das_tabbed_adjoint_planned(
                ct.byref(info), _ptr(coef), _ptr(tautx), _ptr(apodtx), _ptr(taurx), _ptr(apodrx),
                np_, _ptr(ctx.pixel_index), float(np.float32(spec.thresh)), spec.sumtype,
                _ptr(ctx.plan), _ptr(gout), _ptr(g_rf), _ptr(g_ttx), _ptr(g_trx), _ptr(ws), nws,
                _stream())
            _lib.check(st, "pycbf_gb_das_tabbed_adjoint_planned")
        if g_rf is not None and dtype != torch.float32:
            g_rf = g_rf.to(dtype)
        return g_rf, g_ttx, g_trx, None, None, None, None, None


class _SyntheticDAS(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rf4, slowness, geom_struct, keepalive, pixel_index, spec):
        L = _lib.load()
        info = _info(rf4, spec)
        coef = _coefficients(L, rf4, info)
        np_ = slowness.shape[0]
        out = torch.empty(_out_shape(rf4, np_, spec.sumtype), dtype=torch.float32,
                          device=rf4.device)
        st = L.pycbf_gb_das_synthetic_slowness(ct.byref(info), _ptr(coef), ct.byref(geom_struct),
                                               _ptr(slowness), _ptr(pixel_index), spec.sumtype,
                                               _ptr(out), _stream())
        _lib.check(st, "pycbf_gb_das_synthetic_slowness")
        ctx.save_for_backward(coef, slowness)
        ctx.geom = (geom_struct, keepalive)
        ctx.pixel_index = pixel_index
        ctx.spec = spec
        ctx.rf_meta = (tuple(rf4.shape), rf4.dtype)
        return out

    @staticmethod
    def backward(ctx, gout):
        coef, slowness = ctx.saved_tensors
        geom_struct, _ = ctx.geom
        shape, dtype = ctx.rf_meta
        spec = ctx.spec
        need_rf, need_s = ctx.needs_input_grad[0:2]
        L = _lib.load()
        info = _lib.RFInfo(shape[1], shape[2], spec.ndim, float(np.float32(spec.t0)),
                           float(np.float32(spec.dt)), shape[3], shape[0], _DTYPE[dtype])
        dev = coef.device
        gout = gout.to(torch.float32).contiguous()
        g_rf = torch.empty(shape, dtype=torch.float32, device=dev) if need_rf else None
        g_s = torch.empty_like(slowness) if need_s else None
        ws, nws = None, 0
        if need_rf or ctx.pixel_index is not None:
            nws = L.pycbf_gb_adjoint_workspace_bytes(ct.byref(info), slowness.shape[0])
            ws = torch.empty(nws, dtype=torch.uint8, device=dev)
        if need_rf or need_s:
            st = L.pycbf_gb_das_synthetic_adjoint(
                ct.byref(info), _ptr(coef), ct.byref(geom_struct), _ptr(slowness),
                _ptr(ctx.pixel_index), spec.sumtype, _ptr(gout), _ptr(g_rf), _ptr(g_s), _ptr(ws),
                nws, _stream())
            _lib.check(st, "pycbf_gb_das_synthetic_adjoint")
        if g_rf is not None and dtype != torch.float32:
            g_rf = g_rf.to(dtype)
        return g_rf, g_s, None, None, None, None


def _sumtype_code(sumtype: str) -> int:
    if sumtype not in SUMTYPES:
        raise ValueError(f"sumtype must be one of {SUMTYPES} for the differentiable path")
    return _lib.SUMTYPE[sumtype]


def _as4(rf):
    return (rf.unsqueeze(0) if rf.ndim == 3 else rf).contiguous(), rf.ndim == 3


def das_tabbed(rf: torch.Tensor, tautx: torch.Tensor, taurx: torch.Tensor, apodtx: torch.Tensor,
               apodrx: torch.Tensor, *, t0: float, dt: float, thresh: float = 1e-2,
               sumtype: str = "tx_and_rx", pixel_index: torch.Tensor | None = None,
               plan: torch.Tensor | None = None) -> torch.Tensor:
    """Differentiable cubic Tabbed delay-and-sum.

    rf (ntx, nrx, nt) or (nframes, ntx, nrx, nt), float32/float16/bfloat16 on
    CUDA; tautx/apodtx (ntx, np), taurx/apodrx (nrx, np) float32.  Returns
    (np,) / (nframes, np) for 'tx_and_rx', (nrx, np) / (nframes, nrx, np) for
    'tx_only'.  Values equal TabbedBeamformer(interp cubic) on the same inputs.
    plan: a staging plan built for exactly these tables and thresh
    (pycbf_gb_tabbed_plan): the forward then runs the staged kernel, and so
    do the delay gradients for one frame of float32 channel data.
    """
    _check_rf(rf)
    rf4, squeeze = _as4(rf)
    ntx, nrx = rf4.shape[1], rf4.shape[2]
    tables = [t.to(device=rf.device, dtype=torch.float32).contiguous()
              for t in (tautx, taurx, apodtx, apodrx)]
    if tables[0].shape[0] != ntx or tables[2].shape[0] != ntx or tables[1].shape[0] != nrx or \
            tables[3].shape[0] != nrx or len({t.shape[1] for t in tables}) != 1:
        raise ValueError("tables must be tautx/apodtx (ntx, np) and taurx/apodrx (nrx, np)")
    if pixel_index is not None:
        pixel_index = pixel_index.to(device=rf.device, dtype=torch.int32).contiguous()
    spec = _Spec(float(t0), float(dt), float(thresh), _sumtype_code(sumtype))
    out = _TabbedDAS.apply(rf4, *tables, pixel_index, spec, plan)
    return out[0] if squeeze else out


def das_synthetic_slowness(rf: torch.Tensor, slowness: torch.Tensor, geometry, *,
                           sumtype: str = "tx_and_rx") -> torch.Tensor:
    """Differentiable cubic Synthetic delay-and-sum with a slowness per pixel.

    geometry: a SyntheticBeamformer (its element geometry, points, time axis
    and pixel order are used; its c0 is not).  slowness: (np,) float32 in the
    beamformer's point order (s/m; 1/c for a uniform medium).
    """
    _check_rf(rf)
    rf4, squeeze = _as4(rf)
    if geometry._interp_code != _lib.INTERP["cubic"]:
        raise ValueError("the differentiable path interpolates with the cubic spline only")
    if tuple(rf4.shape[1:]) != (geometry.ntx, geometry.nrx, geometry.nt):
        raise ValueError("rf shape does not match the beamformer")
    s = slowness.to(device=rf.device, dtype=torch.float32)
    if s.shape != (geometry.nop,):
        raise ValueError(f"slowness must have shape ({geometry.nop},)")
    pidx = geometry._pixel_index
    if pidx is not None:
        s = s[pidx.long()]
    s = s.contiguous()
    spec = _Spec(float(geometry.t0), float(geometry.dt), 0.0, _sumtype_code(sumtype),
                 int(geometry.ndimp))
    out = _SyntheticDAS.apply(rf4, s, geometry._geom, geometry._dev, pidx, spec)
    return out[0] if squeeze else out

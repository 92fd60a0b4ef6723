"""Beamformer classes: the drop-in for pycbf's Tabbed / Synthetic x DAS / DMAS
path, plus SLSC, running on hand-written sm_103a kernels through the C ABI.

Constructor arguments, validation, sumtype/interp vocabulary, output shapes and
``__call__(txrxt, out_as_numpy=True, buffer=None)`` follow the reference:
  - base classes        pycbf/__bf_base_classes__.py:18-219
  - DMAS mixin          pycbf/__advanced_bf_classes__.py:7-25
  - GPU classes         pycbf/gpu/__core_bf_classes__.py:8-364,
                        pycbf/gpu/__advanced_bf_classes__.py:10-109
  - CPU Tabbed class    pycbf/cpu/__core_bf_classes__.py:6-253 (thresh field)

Differences, all deliberate:
  - inputs may be NumPy arrays or torch tensors (CPU or CUDA); outputs are
    float32 NumPy arrays (out_as_numpy=True) or CUDA torch tensors;
  - ``buffer`` may be a preallocated CUDA float32 tensor of the output shape
    (the reference raises for any buffer);
  - tap selection uses the CPU rule |apodtx*apodrx| >= thresh (thresh default
    1e-2, pycbf/cpu/__core_bf_classes__.py:14) for Tabbed and the GPU rule
    (both masks on) for Synthetic;
  - interp kinds: 'cubic' (natural spline, the reference C path), 'nearest',
    'linear' (two-point interpolation; {'kind': 'linear', 'reference_floor':
    True} reproduces the reference CUDA linear_interp, which returns the floor
    sample).  nearest with usf > 1 upsamples each
    channel by the cubic spline first (pycbf.c:223-253); 'korder_cubic'
    (k-point derivative estimates; {'zero_slopes': True} reproduces the
    reference's Synthetic korder kernel, whose k arrives as 0), 'akima' and
    'makima' follow the reference's CUDA interpolators;
  - DMAS uses the values in ``lags`` (the reference kernel uses positions
    0..nlag-1; both agree when lags = arange(nlag)), takes nsep = ntx for
    lagaxis='tx', and handles 4-D input per frame;
  - there is no global parameter registry; ``id`` is still assigned.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass, field
from typing import ClassVar, Literal

import numpy as np
import torch

from . import _lib, helpers

__all__ = ["BeamformerException", "Beamformer", "Tabbed", "Synthetic", "TabbedBeamformer",
           "SyntheticBeamformer", "TabbedDMASBeamformer", "SyntheticDMASBeamformer",
           "TabbedSLSCBeamformer", "SyntheticSLSCBeamformer", "DMASBeamformer"]

_POLY = (_lib.INTERP["korder_cubic"], _lib.INTERP["akima"], _lib.INTERP["makima"])
STORAGE = {"float32": (_lib.F32, torch.float32), "float16": (_lib.F16, torch.float16),
           "bfloat16": (_lib.BF16, torch.bfloat16)}


class BeamformerException(Exception):
    pass


def _require_cuda():
    if not torch.cuda.is_available():
        raise BeamformerException("pycbf_gb300 needs a CUDA device; none is available")


def _stream_ptr():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


def _to_host(out: torch.Tensor) -> np.ndarray:
    """A CUDA result as a NumPy array: copied into page-locked host memory on
    the current stream (a direct DMA, several times faster than a copy into
    pageable memory), then the stream is synchronised.  The array owns its
    page-locked block, which returns to torch's host cache when it is freed."""
    host = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
    host.copy_(out, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    return host.numpy()


def _to_dev(a, dtype=torch.float32, device="cuda"):
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=device).contiguous()


def _morton(coords: torch.Tensor, bits: int = 21) -> torch.Tensor:
    """Morton (Z-order) key of points given as (n, d) float coordinates."""
    lo = coords.min(dim=0).values
    hi = coords.max(dim=0).values
    span = torch.clamp(hi - lo, min=1e-30)
    q = ((coords - lo) / span * ((1 << bits) - 1)).round().long().clamp(0, (1 << bits) - 1)
    d = q.shape[1]
    key = torch.zeros(q.shape[0], dtype=torch.long, device=q.device)
    for b in range(bits):
        for k in range(d):
            key |= ((q[:, k] >> b) & 1) << (b * d + k)
    return key


# ---------------------------------------------------------------------------
# base dataclasses (validation mirrors the reference)
# ---------------------------------------------------------------------------
@dataclass(kw_only=True)
class Beamformer:
    """Common fields: ``interp`` (dict with 'kind') and ``sumtype``.

    pycbf/__bf_base_classes__.py:18-95.
    """
    nbf: ClassVar[int] = 0
    id: int = field(init=False)
    interp: dict = field(default_factory=lambda: {"kind": "cubic"})
    sumtype: Literal["none", "tx_only", "rx_only", "tx_and_rx"] = "tx_and_rx"

    def __post_init__(self):
        self.id = Beamformer.nbf
        Beamformer.nbf += 1
        self.__check_interp__()
        self.__check_sumtype__()

    def __check_sumtype__(self):
        valid = ["none", "tx_only", "rx_only", "tx_and_rx"]
        if self.sumtype not in valid:
            raise BeamformerException(
                f"sumtype was {self.sumtype} but must be one of the following: " + ", ".join(valid))

    def __check_interp__(self):
        valid = ["nearest", "linear", "akima", "makima", "korder_cubic", "cubic"]
        kind = self.interp.get("kind", None)
        if kind is None or kind not in valid:
            raise BeamformerException(
                f"interp['kind'] was {kind} but must be one of the following: " + ", ".join(valid))
        if kind == "korder_cubic":
            k = self.interp.get("k", None)
            if k is None:
                k = self.interp["k"] = 4
            if k < 4 or k % 2 != 0:
                raise BeamformerException("'k' for interp kind 'korder_cubic' must be at least four and even")
        elif kind != "cubic":
            usf = self.interp.get("usf", None)
            if usf is None:
                self.interp["usf"] = 1
            elif usf < 1:
                raise BeamformerException(
                    f"'usf' for interp kind '{kind}' must be an interger greater than 1")


@dataclass(kw_only=True)
class Tabbed:
    """tautx, apodtx: (Ntx, Np); taurx, apodrx: (Nrx, Np).  __bf_base_classes__.py:97-139."""
    tautx: object = field(init=True)
    taurx: object = field(init=True)
    apodtx: object = field(init=True)
    apodrx: object = field(init=True)
    ntx: int = field(init=False)
    nrx: int = field(init=False)
    nop: int = field(init=False)

    def __post_init__(self):
        shapes = [tuple(np.shape(a)) for a in (self.tautx, self.taurx, self.apodtx, self.apodrx)]
        if not all(len(s) == 2 for s in shapes):
            raise BeamformerException("all delay tabs and apodizations must be 2D matrices")
        (ntx, nop), (nrx, _), _, _ = shapes
        if shapes[2][0] != ntx:
            raise BeamformerException(
                f"tautx and apodtx must have the same shape in dim 0 but were {ntx} and {shapes[2][0]}")
        if shapes[3][0] != nrx:
            raise BeamformerException(
                f"taurx and apodrx must have the same shape in dim 0 but were {nrx} and {shapes[3][0]}")
        if not (shapes[1][1] == nop and shapes[2][1] == nop and shapes[3][1] == nop):
            raise BeamformerException(
                "tautx, taurx, apodtx, and apodrx must have the same shape in dim 1 but were "
                f"{shapes[0][1]}, {shapes[1][1]}, {shapes[2][1]}, and {shapes[3][1]}")
        self.ntx, self.nrx, self.nop = ntx, nrx, nop


@dataclass(kw_only=True)
class Synthetic:
    """Synthetic-point geometry.  __bf_base_classes__.py:141-219."""
    ovectx: object = field(init=True)
    nvectx: object = field(init=True)
    doftx: object = field(init=True)
    alatx: object = field(init=True)
    t0tx: object = field(init=True)
    ovecrx: object = field(init=True)
    nvecrx: object = field(init=True)
    alarx: object = field(init=True)
    c0: float = field(init=True)
    pnts: object = field(init=True)
    ntx: int = field(init=False)
    nrx: int = field(init=False)
    nop: int = field(init=False)
    ndimp: int = field(init=False)

    def __post_init__(self):
        nd = np.ndim
        if not (nd(self.doftx) == 1 and nd(self.alatx) == 1 and nd(self.t0tx) == 1 and nd(self.alarx) == 1):
            raise BeamformerException("all acceptance angle, depth of field, and t0 vectors must be 1D")
        if not (nd(self.ovectx) == 2 and nd(self.nvectx) == 2 and nd(self.ovecrx) == 2 and nd(self.nvecrx) == 2):
            raise BeamformerException("all origin and normal vector matrices must be 2D")
        sh = np.shape
        ntx, nrx = sh(self.ovectx)[0], sh(self.ovecrx)[0]
        nop, ndimp = sh(self.pnts)[0], sh(self.pnts)[1]
        if not (sh(self.nvectx)[0] == ntx and sh(self.doftx)[0] == ntx and sh(self.alatx)[0] == ntx
                and sh(self.t0tx)[0] == ntx):
            raise BeamformerException("All tx variables must have the same shape in the first dimension")
        if not (sh(self.nvecrx)[0] == nrx and sh(self.alarx)[0] == nrx):
            raise BeamformerException("All rx variables must have the same shame in the first variable")
        if not (sh(self.ovectx)[1] == ndimp and sh(self.nvectx)[1] == ndimp and sh(self.ovecrx)[1] == ndimp
                and sh(self.nvecrx)[1] == ndimp):
            raise BeamformerException("All matrix variables must have the same number of dimensions")
        if ndimp not in (2, 3):
            raise BeamformerException("points must be 2-D or 3-D")
        self.ntx, self.nrx, self.nop, self.ndimp = ntx, nrx, nop, ndimp


@dataclass(kw_only=True)
class DMASBeamformer:
    """Delay-multiply-and-sum settings.  pycbf/__advanced_bf_classes__.py:7-25."""
    lags: object = field(init=True)
    lagaxis: Literal["tx", "rx"] = "rx"
    nlags: int = field(init=False)
    sumlags: bool = True
    sumtype: str = field(init=False)
    dmastype: Literal["ssr", "power"] = "ssr"

    def __post_init__(self):
        if self.lagaxis == "rx":
            self.sumtype = "tx_only"
        elif self.lagaxis == "tx":
            self.sumtype = "rx_only"
        else:
            raise BeamformerException("lagaxis keyword can only be 'tx' or 'rx'")
        if self.dmastype not in ("ssr", "power"):
            raise BeamformerException("dmastype keyword must be 'ssr' (signed-square-root) or 'power'")
        self.nlags = len(self.lags)


# ---------------------------------------------------------------------------
# GPU beamformer core
# ---------------------------------------------------------------------------
@dataclass(kw_only=True)
class _GPUBeamformer(Beamformer):
    """Time axis, threshold, storage type and launch helpers.

    pycbf/gpu/__core_bf_classes__.py:8-118.
    """
    t0: float = field(init=True)
    dt: float = field(init=True)
    nt: int = field(init=True)
    nthread: int = 512                      # accepted for compatibility; launch shapes are fixed
    thresh: float = 1e-2
    storage: Literal["float32", "float16", "bfloat16"] = "float32"
    pixel_order: Literal["auto", "natural"] = "auto"
    stage_channels: bool = True             # Tabbed: TMA-staged kernel where it applies

    def __post_init__(self):
        Beamformer.__post_init__(self)
        if self.storage not in STORAGE:
            raise BeamformerException(f"storage must be one of {list(STORAGE)}")
        kind = self.interp["kind"]
        self._usf = int(self.interp.get("usf", 1)) if kind == "nearest" else 1
        if kind == "linear" and self.interp.get("reference_floor", False):
            self._interp_code = _lib.INTERP["linear_floor"]
        else:
            self._interp_code = _lib.INTERP[kind]
        if not (int(self.nt) >= 1 and float(self.dt) > 0):
            raise BeamformerException("nt must be >= 1 and dt > 0")
        self._k, self._S = 0, None
        if kind == "korder_cubic":
            k = int(self.interp["k"])
            if k > 128 or k > int(self.nt):
                raise BeamformerException("'k' for korder_cubic must be at most 128 and at most nt")
            self._S = helpers.korder_matrix(k)
            # zero_slopes: the reference Synthetic korder kernel, whose k arrives as 0
            self._k = 0 if self.interp.get("zero_slopes", False) else k
        if kind in ("akima", "makima") and int(self.nt) < 5:
            raise BeamformerException(f"interp kind '{kind}' needs nt >= 5")
        self._dtype_code, self._torch_dtype = STORAGE[self.storage]
        self._workspace = None

    def _init_device(self):
        _require_cuda()
        self._lib = _lib.load()

    def __check_indexing_limits__(self):
        if self.ntx * self.nrx * self.nt > 2**31 - 1:
            raise BeamformerException(
                f"Product of ntx * nrx * nt must be less than {2**31 - 1} but was "
                f"{self.ntx * self.nrx * self.nt}.")

    # -- shapes ------------------------------------------------------------
    def _out_shape(self, nframes, sumtype=None):
        st = sumtype or self.sumtype
        core = {"none": (self.ntx, self.nrx, self.nop), "tx_only": (self.nrx, self.nop),
                "rx_only": (self.ntx, self.nop), "tx_and_rx": (self.nop,),
                "dmas_ssr": (self.nop,), "dmas_power": (self.nop,)}[st]
        return core if nframes is None else (nframes,) + core

    def _prepare_input(self, txrxt):
        if isinstance(txrxt, np.ndarray):
            t = torch.from_numpy(np.ascontiguousarray(txrxt))
        elif isinstance(txrxt, torch.Tensor):
            t = txrxt
        else:
            raise BeamformerException(
                f"txrxt must be a numpy ndarray or a torch tensor but was {type(txrxt)}")
        if t.ndim == 3:
            if tuple(t.shape) != (self.ntx, self.nrx, self.nt):
                raise BeamformerException(
                    f"'txrxt' must be ({self.ntx}, {self.nrx}, {self.nt}) based on input parameters "
                    f"but was {tuple(t.shape)}")
            nframes = None
        elif t.ndim == 4:
            if tuple(t.shape[1:]) != (self.ntx, self.nrx, self.nt):
                raise BeamformerException(
                    f"'txrxt' must be ({self.ntx}, {self.nrx}, {self.nt}) based on input parameters "
                    f"but was {tuple(t.shape)}")
            nframes = int(t.shape[0])
        else:
            raise BeamformerException("txrxt must be 3-D (ntx, nrx, nt) or 4-D (nframes, ntx, nrx, nt)")
        if t.dtype == torch.int16:
            # raw converter counts: copied as int16, converted on the device
            return t.to(device="cuda", non_blocking=True).contiguous(), nframes
        if not (t.is_floating_point()):
            raise BeamformerException("txrxt must hold floating-point or int16 samples")
        t = t.to(device="cuda", dtype=self._torch_dtype, non_blocking=True).contiguous()
        return t, nframes

    def _ingest_i16(self, rf, info):
        """int16 channel data: passed as PYCBF_GB_I16 where the call converts
        it itself (nearest/linear/cubic, usf 1, float32 storage), else
        converted to float32 by pycbf_gb_convert_i16 and cast to the storage."""
        if self._interp_code <= _lib.INTERP["linear_floor"] and self._usf <= 1 \
                and self._dtype_code == _lib.F32:
            info.dtype = _lib.I16
            return rf
        f = torch.empty(rf.shape, dtype=torch.float32, device=rf.device)
        st = self._lib.pycbf_gb_convert_i16(_ptr(rf), rf.numel(), _ptr(f), _stream_ptr())
        _lib.check(st, "pycbf_gb_convert_i16")
        return f.to(self._torch_dtype)

    def _rfinfo(self, nframes, ndim=0):
        return _lib.RFInfo(self.ntx, self.nrx, ndim, float(np.float32(self.t0)),
                           float(np.float32(self.dt)), int(self.nt), nframes or 1, self._dtype_code)

    def _workspace_for(self, info):
        need = self._lib.pycbf_gb_workspace_bytes(ct.byref(info), self._interp_code)
        if need == 0:
            return None, 0
        if self._workspace is None or self._workspace.numel() < need:
            self._workspace = torch.empty(need, dtype=torch.uint8, device="cuda")
        return self._workspace, need

    def _usf_info(self, info):
        """The rfinfo of the cubic-upsampled channel data (nearest, usf > 1):
        usf*(nt-1)+1 samples at the float32 quotient dt/usf, float32."""
        u = self._usf
        return _lib.RFInfo(info.ntx, info.nrx, info.ndim, info.t0,
                           float(np.float32(info.dt) / np.float32(u)), u * (info.nt - 1) + 1,
                           info.nframes, _lib.F32)

    def _prepare_channels(self, rf, info):
        """(data, rfinfo, workspace, bytes) for the delay-and-sum call: for
        nearest with usf > 1 the channels upsampled by the cubic spline
        (pycbf.c:223-253), else the input and the interp's own workspace."""
        if self._interp_code in _POLY:
            need = self._lib.pycbf_gb_poly_workspace_bytes(ct.byref(info), self._interp_code,
                                                           self._k)
            if self._workspace is None or self._workspace.numel() < need:
                self._workspace = torch.empty(need, dtype=torch.uint8, device="cuda")
            S = self._S.ctypes.data_as(ct.c_void_p) if self._k > 0 else None
            st = self._lib.pycbf_gb_poly_coefficients(ct.byref(info), _ptr(rf), self._interp_code,
                                                      self._k, S, _ptr(self._workspace), need,
                                                      _stream_ptr())
            _lib.check(st, "pycbf_gb_poly_coefficients")
            return self._workspace, info, None, 0
        if self._usf <= 1:
            ws, nws = self._workspace_for(info)
            return rf, info, ws, nws
        need = self._lib.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["cubic"])
        if self._workspace is None or self._workspace.numel() < need:
            self._workspace = torch.empty(need, dtype=torch.uint8, device="cuda")
        nbytes = self._lib.pycbf_gb_upsampled_bytes(ct.byref(info), self._usf)
        up = getattr(self, "_upsampled", None)
        if up is None or up.numel() * 4 < nbytes:
            up = self._upsampled = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda")
        st = self._lib.pycbf_gb_upsample(ct.byref(info), _ptr(rf), self._usf, _ptr(self._workspace),
                                         need, _ptr(up), nbytes, _stream_ptr())
        _lib.check(st, "pycbf_gb_upsample")
        return up, self._usf_info(info), None, 0

    def _output(self, shape, buffer):
        if buffer is None:
            return torch.empty(shape, dtype=torch.float32, device="cuda")
        if not (isinstance(buffer, torch.Tensor) and buffer.is_cuda and buffer.dtype == torch.float32
                and tuple(buffer.shape) == tuple(shape) and buffer.is_contiguous()):
            raise BeamformerException(f"buffer must be a contiguous CUDA float32 tensor of shape {shape}")
        return buffer

    def _launch(self, rf, info, out, sumtype_code):
        raise NotImplementedError

    def _autograd_input(self, txrxt):
        if not isinstance(txrxt, torch.Tensor):
            raise BeamformerException("the differentiable path takes torch tensors")
        if txrxt.ndim not in (3, 4) or tuple(txrxt.shape[-3:]) != (self.ntx, self.nrx, self.nt):
            raise BeamformerException(
                f"'txrxt' must be ({self.ntx}, {self.nrx}, {self.nt}) or 4-D with those last axes")
        return txrxt.to(device="cuda", dtype=self._torch_dtype)

    def _beamform(self, txrxt, buffer=None, sumtype=None):
        rf, nframes = self._prepare_input(txrxt)
        info = self._rfinfo(nframes, getattr(self, "ndimp", 0) if isinstance(self, Synthetic) else 0)
        if rf.dtype == torch.int16:
            rf = self._ingest_i16(rf, info)
        out = self._output(self._out_shape(nframes, sumtype), buffer)
        self._launch(rf, info, out, _lib.SUMTYPE[sumtype or self.sumtype])
        return out

    def __call__(self, txrxt, out_as_numpy: bool = True, buffer=None):
        """Beamform channel data (ntx, nrx, nt) or (nframes, ntx, nrx, nt).

        The work is queued on the current CUDA stream.  With out_as_numpy=True
        the call returns when the image is in host memory.  With False it
        returns the CUDA tensor at once; a pinned host input may then still be
        in flight and must not be overwritten before the stream reaches it.
        The calls of one beamformer share its workspace and staging plan, so
        they must not run on two streams at the same time.
        """
        out = self._beamform(txrxt, buffer)
        return _to_host(out) if out_as_numpy else out

    def beamform_stream(self, frames, sumtype=None):
        """Beamform a sequence of frames held in host memory; yields NumPy
        images in order (the images of __call__).

        While frame k is beamformed, frame k+1 is copied to the device and the
        image of frame k-1 back to the host, each direction on a stream of its
        own (an image copy waits for its beamform, and must not hold up the
        next frame's input copy): two device slots for inputs and outputs,
        pinned host slots for the images (pinned host frames make the input
        copies asynchronous too).  Each frame is
        (ntx, nrx, nt) or (nframes, ntx, nrx, nt), NumPy or CPU torch, float or
        int16.  Sustained throughput is that of the GPU work alone once the
        copies are shorter than the beamform.
        """
        main = torch.cuda.current_stream()
        copy, back = torch.cuda.Stream(), torch.cuda.Stream()
        dev_in, dev_out, host_out = [None, None], [None, None], [None, None]
        in_free = [None, None]    # main is done reading the input slot
        out_home = [None, None]   # the slot's image has reached host memory
        pending = None
        for k, fr in enumerate(frames):
            s = k % 2
            t = fr if isinstance(fr, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(fr))
            if t.is_cuda:
                raise BeamformerException("beamform_stream takes frames in host memory")
            if dev_in[s] is None or dev_in[s].shape != t.shape or dev_in[s].dtype != t.dtype:
                torch.cuda.synchronize()  # no copy may still use a slot being replaced
                dev_in[s] = torch.empty(t.shape, dtype=t.dtype, device="cuda")
            with torch.cuda.stream(copy):
                if in_free[s] is not None:
                    copy.wait_event(in_free[s])
                dev_in[s].copy_(t, non_blocking=True)
                ready = torch.cuda.Event()
                ready.record(copy)
            main.wait_event(ready)
            if out_home[s] is not None:
                main.wait_event(out_home[s])  # frame k-2's image has left the output slot
            nframes = t.shape[0] if t.ndim == 4 else None
            shape = self._out_shape(nframes, sumtype)
            if dev_out[s] is None or tuple(dev_out[s].shape) != tuple(shape):
                dev_out[s] = torch.empty(shape, dtype=torch.float32, device="cuda")
                host_out[s] = torch.empty(shape, dtype=torch.float32, pin_memory=True)
            out = self._beamform(dev_in[s], dev_out[s], sumtype)
            done = torch.cuda.Event()
            done.record(main)
            in_free[s] = done
            with torch.cuda.stream(back):
                back.wait_event(done)
                host_out[s].copy_(out, non_blocking=True)
                home = torch.cuda.Event()
                home.record(back)
                out_home[s] = home
            if pending is not None:
                ps, pev = pending
                pev.synchronize()
                yield host_out[ps].numpy().copy()
            pending = (s, out_home[s])
        if pending is not None:
            ps, pev = pending
            pev.synchronize()
            yield host_out[ps].numpy().copy()


# ---------------------------------------------------------------------------
# Tabbed
# ---------------------------------------------------------------------------
@dataclass(kw_only=True)
class TabbedBeamformer(Tabbed, _GPUBeamformer):
    """Beamformer reading precomputed delay tables and apodizations.

    pycbf/gpu/__core_bf_classes__.py:255-364 and pycbf/cpu/__core_bf_classes__.py:63-253.
    The tables are copied to the device once; with pixel_order='auto' their
    columns are stored in Morton order of the delays to a few elements, so a
    warp's pixels sit close together in every channel.
    """

    def __post_init__(self):
        _GPUBeamformer.__post_init__(self)
        Tabbed.__post_init__(self)
        self.__check_indexing_limits__()
        self._init_device()
        tautx, taurx = _to_dev(self.tautx), _to_dev(self.taurx)
        apodtx, apodrx = _to_dev(self.apodtx), _to_dev(self.apodrx)
        self._pixel_index = None
        if self.pixel_order == "auto" and self.nop > 1:
            rows = [taurx[0], taurx[self.nrx - 1], tautx[self.ntx // 2]]
            key = _morton(torch.stack(rows, dim=1).double())
            perm = torch.argsort(key, stable=True)
            tautx, taurx = tautx[:, perm].contiguous(), taurx[:, perm].contiguous()
            apodtx, apodrx = apodtx[:, perm].contiguous(), apodrx[:, perm].contiguous()
            self._pixel_index = perm.to(torch.int32).contiguous()
        self._tables = (tautx, apodtx, taurx, apodrx)
        self._plan = None
        if (self.stage_channels and self.ntx <= 12 and self._interp_code <= _lib.INTERP["cubic"]
                and self._usf == 1):
            self._plan = self._build_plan(tautx, apodtx, taurx, apodrx)

    def _build_plan(self, tautx, apodtx, taurx, apodrx):
        """The staging plan of these (kernel-order) tables, on the current stream."""
        nbytes = self._lib.pycbf_gb_tabbed_plan_bytes(self.nop, self.ntx, self.nrx)
        plan = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
        info = self._rfinfo(1)
        st = self._lib.pycbf_gb_tabbed_plan(
            ct.byref(info), _ptr(tautx), _ptr(apodtx), _ptr(taurx), _ptr(apodrx), self.nop,
            self._interp_code, float(np.float32(self.thresh)), _ptr(plan), nbytes, _stream_ptr())
        _lib.check(st, "pycbf_gb_tabbed_plan")
        return plan

    def _launch(self, rf, info, out, sumtype_code):
        tautx, apodtx, taurx, apodrx = self._tables
        rf, info, ws, nws = self._prepare_channels(rf, info)
        if self._interp_code in _POLY:
            st = self._lib.pycbf_gb_das_tabbed_poly(
                ct.byref(info), _ptr(rf), self._interp_code, _ptr(tautx), _ptr(apodtx),
                _ptr(taurx), _ptr(apodrx), self.nop, _ptr(self._pixel_index),
                float(np.float32(self.thresh)), sumtype_code, _ptr(out), _stream_ptr())
            _lib.check(st, "pycbf_gb_das_tabbed_poly")
            return
        st = self._lib.pycbf_gb_das_tabbed(
            ct.byref(info), _ptr(rf), _ptr(tautx), _ptr(apodtx), _ptr(taurx), _ptr(apodrx),
            self.nop, _ptr(self._pixel_index), self._interp_code, float(np.float32(self.thresh)),
            sumtype_code, _ptr(self._plan), _ptr(out), _ptr(ws), nws, _stream_ptr())
        _lib.check(st, "pycbf_gb_das_tabbed")

    def differentiable(self, txrxt, tautx=None, taurx=None, sumtype=None):
        """Cubic delay-and-sum through torch autograd (pycbf_gb300.adjoint.das_tabbed).

        txrxt: torch CUDA tensor (ntx, nrx, nt) or (nframes, ntx, nrx, nt);
        tautx / taurx: optional (ntx, nop) / (nrx, nop) tensors in the
        original pixel order replacing the constructor's tables (e.g.
        learnable delays).  sumtype 'tx_and_rx' or 'tx_only'.  Returns a CUDA
        float32 tensor of the usual output shape, differentiable with respect
        to txrxt and the given delay tables.
        """
        from . import adjoint
        if self._interp_code != _lib.INTERP["cubic"]:
            raise BeamformerException("the differentiable path interpolates with the cubic spline")
        rf = self._autograd_input(txrxt)
        if tautx is None and taurx is None:
            ktx, kap_tx, krx, kap_rx = self._tables
            return adjoint.das_tabbed(rf, ktx, krx, kap_tx, kap_rx, t0=self.t0, dt=self.dt,
                                      thresh=self.thresh, sumtype=sumtype or self.sumtype,
                                      pixel_index=self._pixel_index, plan=self._plan)
        # caller-owned delay tables: run in the caller's pixel order, so that
        # no permutation (and no scatter of its gradient) is needed
        ntx_, nap_tx, nrx_, nap_rx = self._natural_tables()
        ktx = ntx_ if tautx is None else tautx.to(device="cuda", dtype=torch.float32)
        krx = nrx_ if taurx is None else taurx.to(device="cuda", dtype=torch.float32)
        return adjoint.das_tabbed(rf, ktx, krx, nap_tx, nap_rx, t0=self.t0, dt=self.dt,
                                  thresh=self.thresh, sumtype=sumtype or self.sumtype)

    def _natural_tables(self):
        """The tables in the caller's pixel order (kept after the first use)."""
        if getattr(self, "_nat_tables", None) is None:
            if self._pixel_index is None:
                self._nat_tables = self._tables
            else:
                perm = self._pixel_index.long()
                nat = []
                for t in self._tables:
                    u = torch.empty_like(t)
                    u[:, perm] = t
                    nat.append(u)
                self._nat_tables = tuple(nat)
        return self._nat_tables

    def kernel_status(self) -> int:
        """0, or 1 if a staged launch gave up a bounded wait (its outputs are
        NaN).  Sticky until reset_kernel_status()."""
        if self._plan is None:
            return 0
        return int(self._plan[:4].view(torch.int32)[0].item())

    def reset_kernel_status(self) -> None:
        if self._plan is not None:
            self._plan[:4].zero_()

    def tap_census(self):
        """Per pixel (original order): contributing taps and the sum of their sample indices."""
        tautx, apodtx, taurx, apodrx = self._tables
        info = self._rfinfo(1)
        if self._usf > 1:
            info = self._usf_info(info)
        cnt = torch.empty(self.nop, dtype=torch.int32, device="cuda")
        isum = torch.empty(self.nop, dtype=torch.int64, device="cuda")
        st = self._lib.pycbf_gb_tap_census_tabbed(
            ct.byref(info), _ptr(tautx), _ptr(apodtx), _ptr(taurx), _ptr(apodrx), self.nop,
            self._interp_code, float(np.float32(self.thresh)), _ptr(cnt), _ptr(isum), _stream_ptr())
        _lib.check(st, "pycbf_gb_tap_census_tabbed")
        return self._unpermute(cnt), self._unpermute(isum)

    def _unpermute(self, v):
        if self._pixel_index is None:
            return v
        out = torch.empty_like(v)
        out[self._pixel_index.long()] = v
        return out

    def rx_mask(self):
        """(nrx, nop) uint8: 1 where |apodrx| >= thresh (original pixel order)."""
        m = (self._tables[3].abs() >= np.float32(self.thresh)).to(torch.uint8)
        if self._pixel_index is None:
            return m
        out = torch.empty_like(m)
        out[:, self._pixel_index.long()] = m
        return out


# ---------------------------------------------------------------------------
# Synthetic
# ---------------------------------------------------------------------------
@dataclass(kw_only=True)
class SyntheticBeamformer(Synthetic, _GPUBeamformer):
    """Beamformer computing delays and masks per pixel from synthetic points.

    pycbf/gpu/__core_bf_classes__.py:120-253.  With pixel_order='auto' the
    points are processed in Morton order of their positions.
    """

    def __post_init__(self):
        _GPUBeamformer.__post_init__(self)
        Synthetic.__post_init__(self)
        self.__check_indexing_limits__()
        self._init_device()
        f32 = lambda a: np.asarray(a, dtype=np.float32)
        alatx, doftx, alarx = f32(self.alatx).astype(np.float64), f32(self.doftx).astype(np.float64), \
            f32(self.alarx).astype(np.float64)
        # per-element constants of the cosine-compare form of the acos tests
        consts = dict(cosalatx=np.cos(alatx), secalatx=np.sqrt(1.0 + np.tan(alatx) ** 2),
                      halfdofsintx=doftx * np.sin(alatx) / 2.0, cosalarx=np.cos(alarx))
        dev = {k: _to_dev(v) for k, v in consts.items()}
        for k in ("ovectx", "nvectx", "t0tx", "alatx", "doftx", "ovecrx", "nvecrx"):
            dev[k] = _to_dev(getattr(self, k))
        pnts = _to_dev(self.pnts)
        self._pixel_index = None
        if self.pixel_order == "auto" and self.nop > 1:
            perm = torch.argsort(_morton(pnts.double()), stable=True)
            pnts = pnts[perm].contiguous()
            self._pixel_index = perm.to(torch.int32).contiguous()
        dev["pnts"] = pnts
        self._dev = dev
        self._geom = _lib.SyntheticGeom(
            **{k: _ptr(dev[k]).value for k in ("ovectx", "nvectx", "t0tx", "alatx", "doftx",
                                                "cosalatx", "secalatx", "halfdofsintx", "ovecrx",
                                                "nvecrx", "cosalarx", "pnts")},
            np=self.nop, c0=float(np.float32(self.c0)))

    def _launch(self, rf, info, out, sumtype_code):
        rf, info, ws, nws = self._prepare_channels(rf, info)
        if self._interp_code in _POLY:
            st = self._lib.pycbf_gb_das_synthetic_poly(
                ct.byref(info), _ptr(rf), self._interp_code, ct.byref(self._geom),
                _ptr(self._pixel_index), sumtype_code, _ptr(out), _stream_ptr())
            _lib.check(st, "pycbf_gb_das_synthetic_poly")
            return
        st = self._lib.pycbf_gb_das_synthetic(
            ct.byref(info), _ptr(rf), ct.byref(self._geom), _ptr(self._pixel_index),
            self._interp_code, sumtype_code, _ptr(out), _ptr(ws), nws, _stream_ptr())
        _lib.check(st, "pycbf_gb_das_synthetic")

    def differentiable(self, txrxt, slowness=None, sumtype=None):
        """Cubic delay-and-sum with a slowness per pixel, through torch autograd
        (pycbf_gb300.adjoint.das_synthetic_slowness).

        slowness: (nop,) tensor in the original point order, s/m; default
        1/c0 everywhere.  Every delay is path length x slowness (plus t0tx
        for focused transmits).  Returns a CUDA float32 tensor of the usual
        output shape for sumtype 'tx_and_rx' or 'tx_only', differentiable with
        respect to txrxt and slowness.
        """
        from . import adjoint
        if self._interp_code != _lib.INTERP["cubic"]:
            raise BeamformerException("the differentiable path interpolates with the cubic spline")
        rf = self._autograd_input(txrxt)
        if slowness is None:
            slowness = torch.full((self.nop,), 1.0 / float(self.c0), dtype=torch.float32,
                                  device="cuda")
        return adjoint.das_synthetic_slowness(rf, slowness, self, sumtype=sumtype or self.sumtype)

    def tap_census(self):
        info = self._rfinfo(1, self.ndimp)
        if self._usf > 1:
            info = self._usf_info(info)
        cnt = torch.empty(self.nop, dtype=torch.int32, device="cuda")
        isum = torch.empty(self.nop, dtype=torch.int64, device="cuda")
        st = self._lib.pycbf_gb_tap_census_synthetic(ct.byref(info), ct.byref(self._geom),
                                                     self._interp_code, _ptr(cnt), _ptr(isum),
                                                     _stream_ptr())
        _lib.check(st, "pycbf_gb_tap_census_synthetic")
        return self._unpermute(cnt), self._unpermute(isum)

    _unpermute = TabbedBeamformer._unpermute

    def rx_mask(self):
        info = self._rfinfo(1, self.ndimp)
        m = torch.empty((self.nrx, self.nop), dtype=torch.uint8, device="cuda")
        st = self._lib.pycbf_gb_synthetic_rx_mask(ct.byref(info), ct.byref(self._geom), _ptr(m),
                                                  _stream_ptr())
        _lib.check(st, "pycbf_gb_synthetic_rx_mask")
        if self._pixel_index is None:
            return m
        out = torch.empty_like(m)
        out[:, self._pixel_index.long()] = m
        return out


# ---------------------------------------------------------------------------
# DMAS
# ---------------------------------------------------------------------------
class _DMASMixin:
    """DMAS on top of a Tabbed/Synthetic beamformer.

    pycbf/gpu/__advanced_bf_classes__.py:10-67.  When the lags are every
    receive lag (1..nrx-1, lagaxis='rx', summed) the pairwise sum is fused into
    the delay-and-sum kernel and the (nrx, np) intermediate never exists.
    """

    def beamform_stream(self, frames, sumtype=None):
        raise BeamformerException("beamform_stream is available for delay-and-sum beamformers")

    def _dmas_setup(self):
        self._lags_host = np.asarray(self.lags, dtype=np.int64).ravel()
        self._lags_dev = torch.as_tensor(self._lags_host.astype(np.int32), device="cuda")
        nsep = self.nrx if self.lagaxis == "rx" else self.ntx
        self._fused = (self.lagaxis == "rx" and self.sumlags and len(self._lags_host) == nsep - 1
                       and np.array_equal(np.sort(self._lags_host), np.arange(1, nsep)))

    def _dmas_out_shape(self, nframes):
        core = (self.nop,) if self.sumlags else (self.nlags, self.nop)
        return core if nframes is None else (nframes,) + core

    def __call__(self, txrxt, out_as_numpy: bool = True, buffer=None):
        if self._fused:
            code = "dmas_ssr" if self.dmastype == "ssr" else "dmas_power"
            out = self._beamform(txrxt, buffer, sumtype=code)
        else:
            sep = self._beamform(txrxt, None)
            nframes = sep.shape[0] if sep.ndim == 3 else None
            nsep = sep.shape[-2]
            out = self._output(self._dmas_out_shape(nframes), buffer)
            st = self._lib.pycbf_gb_dmas(_ptr(sep), nframes or 1, nsep, self.nop, _ptr(self._lags_dev),
                                         len(self._lags_host), 0 if self.dmastype == "ssr" else 1,
                                         int(bool(self.sumlags)), _ptr(out), _stream_ptr())
            _lib.check(st, "pycbf_gb_dmas")
        return _to_host(out) if out_as_numpy else out


@dataclass(kw_only=True)
class TabbedDMASBeamformer(_DMASMixin, TabbedBeamformer, DMASBeamformer):
    """DMAS with precomputed delay tables.  gpu/__advanced_bf_classes__.py:69-88."""

    def __post_init__(self):
        DMASBeamformer.__post_init__(self)
        TabbedBeamformer.__post_init__(self)
        self._dmas_setup()


@dataclass(kw_only=True)
class SyntheticDMASBeamformer(_DMASMixin, SyntheticBeamformer, DMASBeamformer):
    """DMAS with synthetic-point delays.  gpu/__advanced_bf_classes__.py:90-109."""

    def __post_init__(self):
        DMASBeamformer.__post_init__(self)
        SyntheticBeamformer.__post_init__(self)
        self._dmas_setup()


# ---------------------------------------------------------------------------
# SLSC (no reference class: the notebook algorithm, advanced_beamforming.ipynb)
# ---------------------------------------------------------------------------
class _SLSCMixin:
    """Short-lag spatial coherence over the transmit-summed per-element image.

    The pixels must form a grid_shape = (nx, nz) grid in meshgrid('ij') order
    (z fastest).  An element takes part at pixel (ix, iz) when its receive
    mask is on for the whole axial kernel [iz-nkern, iz+nkern]; the result is
    the mean over lags 1..nlag of the nan-mean pair correlation.
    """

    def beamform_stream(self, frames, sumtype=None):
        raise BeamformerException("beamform_stream is available for delay-and-sum beamformers")

    def _slsc_setup(self):
        nx, nz = (int(v) for v in self.grid_shape)
        if nx * nz != self.nop:
            raise BeamformerException(f"grid_shape {self.grid_shape} does not match {self.nop} points")
        if not (1 <= int(self.nlag) <= 32) or not (0 <= int(self.nkern) <= 31):
            raise BeamformerException("nlag must be in 1..32 and nkern in 0..31")
        self._mask = self.rx_mask().contiguous()
        # the kept-element bit sets depend on the mask and nkern only: once here
        self._kept = None
        nbytes = self._lib.pycbf_gb_slsc_kept_bytes(self.nrx, nx, nz)
        kept = torch.empty(max(nbytes, 4), dtype=torch.uint8, device="cuda")
        st = self._lib.pycbf_gb_slsc_kept(_ptr(self._mask), self.nrx, nx, nz, int(self.nlag),
                                          int(self.nkern), _ptr(kept), nbytes, _stream_ptr())
        if st == _lib.OK:
            self._kept = kept
        elif st != _lib.ERANGE:  # ERANGE: outside the register kernel's limits
            _lib.check(st, "pycbf_gb_slsc_kept")

    def __call__(self, txrxt, out_as_numpy: bool = True, buffer=None):
        sep = self._beamform(txrxt, None, sumtype="tx_only")
        nframes = sep.shape[0] if sep.ndim == 3 else None
        nx, nz = (int(v) for v in self.grid_shape)
        shape = (nx, nz) if nframes is None else (nframes, nx, nz)
        out = self._output(shape, buffer)
        if self._kept is not None:
            st = self._lib.pycbf_gb_slsc_with_kept(_ptr(sep), _ptr(self._kept), nframes or 1,
                                                   self.nrx, nx, nz, int(self.nlag),
                                                   int(self.nkern), _ptr(out), _stream_ptr())
            _lib.check(st, "pycbf_gb_slsc_with_kept")
        else:
            st = self._lib.pycbf_gb_slsc(_ptr(sep), _ptr(self._mask), nframes or 1, self.nrx, nx,
                                         nz, int(self.nlag), int(self.nkern), _ptr(out),
                                         _stream_ptr())
            _lib.check(st, "pycbf_gb_slsc")
        return _to_host(out) if out_as_numpy else out


@dataclass(kw_only=True)
class TabbedSLSCBeamformer(_SLSCMixin, TabbedBeamformer):
    grid_shape: tuple = field(init=True)
    nlag: int = 16
    nkern: int = 2

    def __post_init__(self):
        TabbedBeamformer.__post_init__(self)
        self._slsc_setup()


@dataclass(kw_only=True)
class SyntheticSLSCBeamformer(_SLSCMixin, SyntheticBeamformer):
    grid_shape: tuple = field(init=True)
    nlag: int = 16
    nkern: int = 2

    def __post_init__(self):
        SyntheticBeamformer.__post_init__(self)
        self._slsc_setup()

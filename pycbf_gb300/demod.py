"""IQ demodulation, envelope and log compression of beamformed images on the GPU
(the step after the delay-and-sum).

``fft_tukey_demod`` and ``zout_fft_tukey_demod`` keep the signatures of the
helpers the reference's examples define and call after every beamform
(examples/SyntheticPointBeamforming.ipynb cell 1; the same functions in
SyntheticVsTabbed.ipynb cell 1 and develop_dmas_class.ipynb cell 7): real FFT
along ``axis``, bins [ikmin, ikmax) kept and weighted by a Tukey window,
ifftshift to base band, inverse FFT.  The chain is linear, so ``Demodulator``
builds it once as an (n, M) complex matrix (NumPy float64 applied to the
identity, stored as complex64 on the device) and ``pycbf_gb_demod`` applies it
to every line in one float32 kernel, writing IQ and/or the envelope.
``Demodulator.bmode`` adds the examples' display line
20*log10(env/percentile(env, 99) + 1e-10) (SyntheticPointBeamforming.ipynb
cell 11): an exact percentile selection and the log compression on the
device, with no host round trip.
"""
from __future__ import annotations

import ctypes as ct
from collections import OrderedDict

import numpy as np
import torch

from . import _lib

__all__ = ["Demodulator", "fft_tukey_demod", "zout_fft_tukey_demod", "percentile",
           "log_compress", "bmode_compress", "tukey", "demod_matrix"]


def _stream():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


def tukey(M: int, alpha: float = 0.25) -> np.ndarray:
    """Symmetric tapered-cosine (Tukey) window of M points, float64: 1 in the
    middle, half-cosine lobes over a fraction alpha (0 rectangular, 1 Hann)."""
    if M <= 0:
        return np.zeros(0)
    if M == 1 or alpha <= 0:
        return np.ones(M)
    n = np.arange(M, dtype=np.float64)
    if alpha >= 1.0:
        return 0.5 - 0.5 * np.cos(2 * np.pi * n / (M - 1))
    width = int(np.floor(alpha * (M - 1) / 2.0))
    w = np.ones(M)
    a, b = n[: width + 1], n[M - width - 1:]
    w[: width + 1] = 0.5 * (1 + np.cos(np.pi * (-1 + 2.0 * a / alpha / (M - 1))))
    w[M - width - 1:] = 0.5 * (1 + np.cos(np.pi * (-2.0 / alpha + 1 + 2.0 * b / alpha / (M - 1))))
    return w


def _bins(n, ks, kmin, kmax):
    f = np.fft.rfftfreq(n, 1 / ks)
    return int(np.argmin(np.abs(f - kmin))), int(np.argmin(np.abs(f - kmax))) + 1


def demod_matrix(n: int, kmin: float, kmax: float, ks: float, alpha: float = 0.25,
                 shiftit: bool = True) -> np.ndarray:
    """(n, M) complex128 W with iq = x @ W for lines x of n samples: the rows
    are the demodulated unit impulses."""
    lo, hi = _bins(n, ks, kmin, kmax)
    if hi <= lo:
        raise ValueError(f"empty band: bins [{lo}, {hi}) for kmin={kmin}, kmax={kmax}")
    spec = np.fft.rfft(np.eye(n), axis=1)[:, lo:hi] * tukey(hi - lo, alpha)[None, :]
    if shiftit:
        spec = np.fft.ifftshift(spec, axes=1)
    return np.fft.ifft(spec, axis=1)


def zout_fft_tukey_demod(zout, kmin, kmax):
    """Axial positions of the demodulated samples, as the examples compute them."""
    zout = np.asarray(zout, np.float64)
    dz = zout[1] - zout[0]
    k = np.fft.rfftfreq(len(zout), dz)
    dk = k[1] - k[0]
    lo = np.argmin(np.abs(k - kmin))
    hi = np.argmin(np.abs(k - kmax))
    return zout[0] + np.arange(hi - lo + 1) / (dk * (hi - lo))


def _as_cuda_f32(x):
    if isinstance(x, torch.Tensor):
        if not x.is_cuda:
            raise ValueError("torch input must be a CUDA tensor (or pass a NumPy array)")
        return x.to(torch.float32)
    return torch.as_tensor(np.asarray(x, np.float32), device="cuda")


def percentile(v: torch.Tensor, q: float = 99.0, segments: int = 1) -> torch.Tensor:
    """NumPy's percentile (method 'linear') of each of `segments` equal
    contiguous parts of v, on the device: a float32 tensor of `segments`."""
    v = _as_cuda_f32(v).contiguous().reshape(-1)
    if segments <= 0 or v.numel() % segments:
        raise ValueError("v must split into `segments` equal parts")
    n = v.numel() // segments
    L = _lib.load()
    ws = torch.empty(max(1, L.pycbf_gb_percentile_workspace_bytes(segments)), dtype=torch.uint8,
                     device=v.device)
    out = torch.empty(segments, dtype=torch.float32, device=v.device)
    st = L.pycbf_gb_percentile(_p(v), segments, n, float(q), _p(out), _p(ws), ws.numel(), _stream())
    _lib.check(st, "pycbf_gb_percentile")
    return out


def log_compress(env: torch.Tensor, ref: torch.Tensor, floor: float = 1e-10,
                 out: torch.Tensor | None = None) -> torch.Tensor:
    """20 log10(env / ref[s] + floor), env split into len(ref) equal segments."""
    env = _as_cuda_f32(env).contiguous()
    ref = ref.to(device=env.device, dtype=torch.float32).contiguous().reshape(-1)
    nseg = ref.numel()
    if nseg == 0 or env.numel() % nseg:
        raise ValueError("env must split into len(ref) equal parts")
    out = torch.empty_like(env) if out is None else out
    st = _lib.load().pycbf_gb_log_compress(_p(env), nseg, env.numel() // nseg, _p(ref),
                                           float(np.float32(floor)), _p(out), _stream())
    _lib.check(st, "pycbf_gb_log_compress")
    return out


def bmode_compress(env: torch.Tensor, q: float = 99.0, floor: float = 1e-10, segments: int = 1,
                   out: torch.Tensor | None = None):
    """(20 log10(env / percentile(env, q) + floor), percentiles) per segment,
    the percentile and the compression in one launch for images of up to
    425,984 values (a cluster of 8 CTAs holds each image in shared memory)."""
    env = _as_cuda_f32(env).contiguous()
    if segments <= 0 or env.numel() % segments:
        raise ValueError("env must split into `segments` equal parts")
    L = _lib.load()
    ws = torch.empty(max(1, L.pycbf_gb_percentile_workspace_bytes(segments)), dtype=torch.uint8,
                     device=env.device)
    ref = torch.empty(segments, dtype=torch.float32, device=env.device)
    out = torch.empty_like(env) if out is None else out
    st = L.pycbf_gb_log_compress_percentile(_p(env), segments, env.numel() // segments, float(q),
                                            float(np.float32(floor)), _p(out), _p(ref), _p(ws),
                                            ws.numel(), _stream())
    _lib.check(st, "pycbf_gb_log_compress_percentile")
    return out, ref


class Demodulator:
    """fft_tukey_demod for lines of n samples, its matrix kept on the device.

    iq(x, axis)        complex64 IQ, the band's M samples along `axis`
    envelope(x, axis)  |IQ| as float32, without writing the IQ
    bmode(x, axis, q, floor, image_ndim)
                       20 log10(env / percentile(env, q) + floor); the
                       percentile is taken over the last `image_ndim` axes
                       of the envelope (None: the whole array, as the
                       examples do for one image)
    """

    def __init__(self, n: int, kmin: float, kmax: float, ks: float, alpha: float = 0.25,
                 shiftit: bool = True, device="cuda"):
        self.n = int(n)
        self.kmin, self.kmax, self.ks, self.alpha = float(kmin), float(kmax), float(ks), float(alpha)
        self.shiftit = bool(shiftit)
        W = demod_matrix(self.n, kmin, kmax, ks, alpha, shiftit)
        self.M = W.shape[1]
        self._W = torch.view_as_real(torch.as_tensor(W.astype(np.complex64))).contiguous().to(device)
        self._lib = _lib.load()

    def _lines(self, x, axis):
        x = _as_cuda_f32(x)
        axis = axis % x.ndim
        if x.shape[axis] != self.n:
            raise ValueError(f"axis {axis} has {x.shape[axis]} samples, the demodulator {self.n}")
        xm = x.movedim(axis, -1).contiguous()
        return xm, axis

    def _run(self, xm, want_iq, want_env):
        lead = xm.shape[:-1]
        ncols = int(np.prod(lead)) if lead else 1
        iq = torch.empty((*lead, self.M, 2), dtype=torch.float32, device=xm.device) if want_iq else None
        env = torch.empty((*lead, self.M), dtype=torch.float32, device=xm.device) if want_env else None
        st = self._lib.pycbf_gb_demod(_p(xm), ncols, self.n, _p(self._W), self.M, _p(iq), _p(env),
                                      _stream())
        _lib.check(st, "pycbf_gb_demod")
        return iq, env

    def iq(self, x, axis: int = -1) -> torch.Tensor:
        xm, axis = self._lines(x, axis)
        iq, _ = self._run(xm, True, False)
        return torch.view_as_complex(iq).movedim(-1, axis)

    def envelope(self, x, axis: int = -1) -> torch.Tensor:
        xm, axis = self._lines(x, axis)
        _, env = self._run(xm, False, True)
        return env.movedim(-1, axis)

    def bmode(self, x, axis: int = -1, q: float = 99.0, floor: float = 1e-10,
              image_ndim: int | None = None) -> torch.Tensor:
        env = self.envelope(x, axis).contiguous()
        nseg = 1 if image_ndim is None else int(np.prod(env.shape[: env.ndim - image_ndim]))
        return bmode_compress(env, q, floor, nseg, out=env)[0]


_CACHE: "OrderedDict[tuple, Demodulator]" = OrderedDict()


def fft_tukey_demod(rfdata, kmin: float, kmax: float, ks: float, alpha: float = 0.25,
                    axis: int = -1, shiftit: bool = True):
    """Demodulate rfdata along `axis` to complex IQ (the examples' helper).

    CUDA tensors give a complex64 CUDA tensor; NumPy arrays give a NumPy
    complex64 array.  The matrix of each (n, band, window) is cached."""
    is_np = not isinstance(rfdata, torch.Tensor)
    shape = np.shape(rfdata) if is_np else tuple(rfdata.shape)
    n = shape[axis % len(shape)]
    key = (n, float(kmin), float(kmax), float(ks), float(alpha), bool(shiftit))
    dm = _CACHE.get(key)
    if dm is None:
        dm = _CACHE[key] = Demodulator(n, kmin, kmax, ks, alpha, shiftit)
        while len(_CACHE) > 16:
            _CACHE.popitem(last=False)
    else:
        _CACHE.move_to_end(key)
    iq = dm.iq(rfdata, axis)
    return iq.cpu().numpy() if is_np else iq

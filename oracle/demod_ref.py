"""CPU oracle of the IQ demodulation and log compression (test infrastructure).

Restates in NumPy float64 the examples' fft_tukey_demod and
zout_fft_tukey_demod (examples/SyntheticPointBeamforming.ipynb cell 1; the
same function in SyntheticVsTabbed.ipynb cell 1 and develop_dmas_class.ipynb
cell 7) and their display line 20*log10(env/percentile(env, 99) + 1e-10)
(SyntheticPointBeamforming.ipynb cell 11).  The Tukey window is the tapered
cosine of scipy.signal.windows.tukey (symmetric form), restated from its
definition.  Pinned against tests/golden/demod.npz, which the reference's own
notebook code produced.  Only tests, smoke() and the bench's CPU leg use this.
"""
from __future__ import annotations

import numpy as np


def tukey(M: int, alpha: float = 0.25) -> np.ndarray:
    """Symmetric tapered-cosine window of M points: flat top, cosine lobes
    over a fraction alpha of the window."""
    if M <= 0:
        return np.zeros(0)
    if M == 1:
        return np.ones(1)
    if alpha <= 0:
        return np.ones(M)
    n = np.arange(M, dtype=np.float64)
    if alpha >= 1.0:
        return 0.5 - 0.5 * np.cos(2 * np.pi * n / (M - 1))
    width = int(np.floor(alpha * (M - 1) / 2.0))
    w = np.ones(M)
    n1 = n[: width + 1]
    n3 = n[M - width - 1:]
    w[: width + 1] = 0.5 * (1 + np.cos(np.pi * (-1 + 2.0 * n1 / alpha / (M - 1))))
    w[M - width - 1:] = 0.5 * (1 + np.cos(np.pi * (-2.0 / alpha + 1 + 2.0 * n3 / alpha / (M - 1))))
    return w


def band_bins(n: int, ks: float, kmin: float, kmax: float):
    """[ikmin, ikmax) of the kept rfft bins (cell 1: argmin |f - kmin|,
    argmin |f - kmax| + 1)."""
    freqs = np.fft.rfftfreq(n, 1 / ks)
    return int(np.argmin(np.abs(freqs - kmin))), int(np.argmin(np.abs(freqs - kmax))) + 1


def fft_tukey_demod(rfdata, kmin, kmax, ks, alpha=0.25, axis=-1, shiftit=True):
    """rfft -> bins [ikmin, ikmax) -> Tukey window -> (ifftshift) -> ifft, float64."""
    x = np.asarray(rfdata, np.float64)
    lo, hi = band_bins(x.shape[axis], ks, kmin, kmax)
    shape = [1] * x.ndim
    shape[axis] = hi - lo
    win = tukey(hi - lo, alpha).reshape(shape)
    spec = np.take(np.fft.rfft(x, axis=axis), np.arange(lo, hi), axis=axis) * win
    if shiftit:
        spec = np.fft.ifftshift(spec, axes=axis)
    return np.fft.ifft(spec, axis=axis)


def zout_fft_tukey_demod(zout, kmin, kmax):
    """Axial positions of the demodulated samples (cell 1)."""
    zout = np.asarray(zout, np.float64)
    dz = zout[1] - zout[0]
    ks = np.fft.rfftfreq(len(zout), dz)
    dk = ks[1] - ks[0]
    lo = np.argmin(np.abs(ks - kmin))
    hi = np.argmin(np.abs(ks - kmax))
    return zout[0] + np.arange(hi - lo + 1) / (dk * (hi - lo))


def log_compress(env, q=99.0, floor=1e-10):
    """20 log10(env / percentile(env, q) + floor) over the whole array (cell 11)."""
    env = np.asarray(env, np.float64)
    return 20 * np.log10(env / np.percentile(env, q) + floor)

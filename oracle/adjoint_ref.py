"""Float64 autograd restatement of the cubic delay-and-sum (test infrastructure).

Only the tests import this module.  It is the reference the adjoint kernels
are checked against: the same piecewise-cubic function of the channel data
and the delays, evaluated in float64 and differentiated by torch autograd.

What "the same function" means:
  - the natural cubic spline of each channel, z = 1/2 T^-1 D y
    (pycbf/cpu/pycbf.c:114-166: tie_knots1D_fixed's Thomas solve of
    0.5 y2_i-1 + 2 y2_i + 0.5 y2_i+1 = 3 (y_i+1 - 2 y_i + y_i-1) / dx^2,
    y2_0 = y2_n-1 = 0, with z = y2 dx^2 / 6), here a dense float64 solve;
  - the tap decisions of the float32 path: x32 = fl(tautx + taurx),
    apod = fl(apodtx * apodrx) >= thresh, t0 <= x32 <= fl(t0 + fl(dt (nt-1))),
    j = (int) fl(fl(x32 - t0) / dt) (pycbf.c:68-105, 179-207);
  - the knot positions xlo = fl(t0 + fl(dt j)), xhi = fl(t0 + fl(dt (j+1)))
    of the float32 path, a = (xhi - x) / dt, b = (x - xlo) / dt in float64,
    S = a y_j + b y_j+1 + (a^3 - a) z_j + (b^3 - b) z_j+1 (pycbf.c:93-104);
  - x is the float32 sum x32 in value, with derivative 1 with respect to each
    delay (the rounding of the sum has no derivative).
For the Synthetic slowness form (plane-wave transmits, element receives:
pycbf/gpu/__engines__.cu:382-470 with 1/c0 replaced by a slowness per pixel)
the float32 path is x32 = fl(fl(proj s) + fl(mag s)) and the float64 value
x = (proj + mag) s carries the derivative dx/ds = proj + mag.
"""
from __future__ import annotations

import numpy as np
import torch

__all__ = ["spline_z", "das_tabbed_ref", "das_synth_pw_ref", "synth_pw_paths32"]

_TINV: dict = {}


def _tinv(n: int) -> torch.Tensor:
    if n not in _TINV:
        m = n - 2
        T = torch.zeros((m, m), dtype=torch.float64)
        idx = torch.arange(m)
        T[idx, idx] = 2.0
        T[idx[:-1], idx[:-1] + 1] = 0.5
        T[idx[1:], idx[1:] - 1] = 0.5
        _TINV[n] = torch.linalg.inv(T)
    return _TINV[n]


def spline_z(y: torch.Tensor) -> torch.Tensor:
    """z = 1/2 T^-1 D y along the last axis (natural ends), float64."""
    n = y.shape[-1]
    if n < 3:
        return torch.zeros_like(y)
    d = y[..., 2:] - 2.0 * y[..., 1:-1] + y[..., :-2]
    zi = 0.5 * d @ _tinv(n)  # T symmetric
    return torch.nn.functional.pad(zi, (1, 1))


def _f32(v):
    return np.float32(v)


def _decide(x32: np.ndarray, t0: float, dt: float, nt: int):
    """In-range flag, knot j and float32 knot positions of the float32 path."""
    t0f, dtf = _f32(t0), _f32(dt)
    xmax = _f32(t0f + _f32(dtf * _f32(nt - 1)))
    with np.errstate(invalid="ignore", over="ignore"):
        inr = (x32 >= t0f) & (x32 <= xmax)
        q = ((x32 - t0f) / dtf).astype(np.float32)
        j = np.where(inr, np.floor(q), 0).astype(np.int64)
    j = np.minimum(j, nt - 1)
    jf = j.astype(np.float32)
    xlo = (t0f + (dtf * jf).astype(np.float32)).astype(np.float32)
    xhi = (t0f + (dtf * (jf + np.float32(1))).astype(np.float32)).astype(np.float32)
    return inr, j, xlo, xhi


def _interp(y, z, ch, j, x, xlo, xhi, dt):
    """Cubic value at float64 x of the records (y, z) gathered at channel ch, knot j."""
    nt = y.shape[-1]
    yp = torch.nn.functional.pad(y, (0, 1)).reshape(-1)
    zp = torch.nn.functional.pad(z, (0, 1)).reshape(-1)
    base = ch * (nt + 1) + j
    a = (xhi - x) / dt
    b = (x - xlo) / dt
    return a * yp[base] + b * yp[base + 1] + (a ** 3 - a) * zp[base] + (b ** 3 - b) * zp[base + 1]


def das_tabbed_ref(rf, tautx, taurx, apodtx, apodrx, t0, dt, thresh=1e-2, sumtype="tx_and_rx"):
    """rf (nf, ntx, nrx, nt), tables (ntx|nrx, np): float64 tensors (may require grad)
    holding float32 values.  Returns (nf, np) or (nf, nrx, np) float64."""
    nf, ntx, nrx, nt = rf.shape
    np_ = tautx.shape[1]
    ttx32 = tautx.detach().numpy().astype(np.float32)
    trx32 = taurx.detach().numpy().astype(np.float32)
    atx32 = apodtx.detach().numpy().astype(np.float32)
    arx32 = apodrx.detach().numpy().astype(np.float32)
    x32 = (ttx32[:, None, :] + trx32[None, :, :]).astype(np.float32)        # (ntx, nrx, np)
    apod32 = (atx32[:, None, :] * arx32[None, :, :]).astype(np.float32)
    inr, j, xlo, xhi = _decide(x32, t0, dt, nt)
    hit = inr & (np.abs(apod32) >= _f32(thresh))
    t_i, r_i, p_i = np.nonzero(hit)
    tt, rr, pp = (torch.from_numpy(v) for v in (t_i, r_i, p_i))
    x = (torch.from_numpy(x32[hit].astype(np.float64))
         + (tautx[tt, pp] - tautx[tt, pp].detach()) + (taurx[rr, pp] - taurx[rr, pp].detach()))
    w = torch.from_numpy(apod32[hit].astype(np.float64))
    z = spline_z(rf)
    jj = torch.from_numpy(j[hit])
    lo = torch.from_numpy(xlo[hit].astype(np.float64))
    hi = torch.from_numpy(xhi[hit].astype(np.float64))
    dt64 = float(_f32(dt))
    if sumtype == "tx_and_rx":
        out = torch.zeros((nf, np_), dtype=torch.float64)
    else:
        out = torch.zeros((nf, nrx, np_), dtype=torch.float64)
    for f in range(nf):
        ch = (f * ntx + tt) * nrx + rr
        v = w * _interp(rf, z, ch, jj, x, lo, hi, dt64)
        if sumtype == "tx_and_rx":
            out = out.index_put((torch.full_like(pp, f), pp), v, accumulate=True)
        else:
            out = out.index_put((torch.full_like(pp, f), rr, pp), v, accumulate=True)
    return out


def synth_pw_paths32(pnts32, ovectx32, nvectx32, ovecrx32, nvecrx32, cosalarx32):
    """Float32 path lengths of the kernels' arithmetic (sequential sums, IEEE ops):
    proj (ntx, np) for plane-wave transmits, mag (nrx, np) and the receive mask."""
    nd = pnts32.shape[1]

    def dist(o, n):
        m2 = np.zeros((o.shape[0], pnts32.shape[0]), np.float32)
        pr = np.zeros_like(m2)
        for k in range(nd):
            d = (pnts32[None, :, k] - o[:, None, k]).astype(np.float32)
            m2 = (m2 + (d * d).astype(np.float32)).astype(np.float32)
            pr = (pr + (d * n[:, None, k]).astype(np.float32)).astype(np.float32)
        return np.sqrt(m2).astype(np.float32), pr

    _, proj = dist(ovectx32, nvectx32)
    mag, prr = dist(ovecrx32, nvecrx32)
    with np.errstate(invalid="ignore", divide="ignore"):
        off = (mag > np.float32(1e-12)) & ((prr / mag).astype(np.float32) < cosalarx32[:, None])
    return proj, mag, ~off


def das_synth_pw_ref(rf, slowness, pnts32, ovectx32, nvectx32, ovecrx32, nvecrx32, cosalarx32,
                     t0, dt, sumtype="tx_and_rx"):
    """Plane-wave Synthetic delay-and-sum with slowness per pixel (float64 tensor
    holding float32 values, may require grad).  Geometry arrays are float32 numpy."""
    nf, ntx, nrx, nt = rf.shape
    np_ = slowness.shape[0]
    proj, mag, rx_ok = synth_pw_paths32(pnts32, ovectx32, nvectx32, ovecrx32, nvecrx32,
                                        cosalarx32)
    s32 = slowness.detach().numpy().astype(np.float32)
    tautx32 = (proj * s32[None, :]).astype(np.float32)
    taurx32 = np.where(rx_ok, (mag * s32[None, :]).astype(np.float32), np.float32(np.inf))
    with np.errstate(invalid="ignore"):
        x32 = (tautx32[:, None, :] + taurx32[None, :, :]).astype(np.float32)
    inr, j, xlo, xhi = _decide(x32, t0, dt, nt)
    hit = inr & rx_ok[None, :, :]
    t_i, r_i, p_i = np.nonzero(hit)
    tt, rr, pp = (torch.from_numpy(v) for v in (t_i, r_i, p_i))
    D = torch.from_numpy((proj[t_i, p_i].astype(np.float64) + mag[r_i, p_i].astype(np.float64)))
    x = torch.from_numpy(x32[hit].astype(np.float64)) + D * (slowness[pp] - slowness[pp].detach())
    z = spline_z(rf)
    jj = torch.from_numpy(j[hit])
    lo = torch.from_numpy(xlo[hit].astype(np.float64))
    hi = torch.from_numpy(xhi[hit].astype(np.float64))
    dt64 = float(_f32(dt))
    if sumtype == "tx_and_rx":
        out = torch.zeros((nf, np_), dtype=torch.float64)
    else:
        out = torch.zeros((nf, nrx, np_), dtype=torch.float64)
    for f in range(nf):
        ch = (f * ntx + tt) * nrx + rr
        v = _interp(rf, z, ch, jj, x, lo, hi, dt64)
        if sumtype == "tx_and_rx":
            out = out.index_put((torch.full_like(pp, f), pp), v, accumulate=True)
        else:
            out = out.index_put((torch.full_like(pp, f), rr, pp), v, accumulate=True)
    return out

"""Delay tables and apodizations of a linear array on a pixel grid, built on
the GPU (the step before the Tabbed path).

``make_tabs_and_apods_2d`` takes the arguments of the reference's
``pycbf.helpers.make_tabs_and_apods_2D`` (pycbf/helpers/__full_aperture_2D__.py
:170-203) and returns the same four tables as float32 CUDA tensors, built by
``pycbf_gb_tables_2d``: the per-transmit constants are computed here with
NumPy exactly as the reference's helper functions compute them, every
per-pixel value on the device in float64 in NumPy's order of operations, then
rounded to float32 (what the reference's classes do with its float64
tables).  The tables can be handed to ``TabbedBeamformer`` without a trip
through host memory.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

from . import _lib

__all__ = ["make_tabs_and_apods_2d", "transmit_params_2d"]


def transmit_params_2d(steers, r0, ctx, cm, xele):
    """(txkind, params (ntx, 6) float64) of pycbf_gb_tables_2d.

    r0 > 0 focused (calc_tx_synthetic_points_focused_2D, :270-314), r0 == 0
    plane waves (calc_tx_tabs_and_apods_pw_2D, :129-168), r0 < 0 diverging
    (calc_tx_tabs_and_apods_divergent_2D, :37-84)."""
    steers = np.atleast_1d(np.asarray(steers, np.float64))
    xele = np.asarray(xele, np.float64)
    p = np.zeros((len(steers), 6))
    if r0 > 0:
        if ctx != cm:
            raise NotImplementedError("speed-of-sound correction is not defined for focused waves")
        ovectx = r0 * np.array([np.sin(steers), np.cos(steers)]).T
        dxmax = np.max(np.hypot(xele[None, :] - ovectx[:, 0, None], ovectx[:, 1, None]), axis=1)
        t0tx = dxmax / cm
        alneg = np.arctan2(ovectx[:, 0] - xele[0], ovectx[:, 1])
        alpos = np.arctan2(ovectx[:, 0] - xele[-1], ovectx[:, 1])
        alatx = -(alpos - alneg) / 2
        alsteers = (alpos + alneg) / 2
        p[:, 0:2] = ovectx
        p[:, 2], p[:, 3] = np.sin(alsteers), np.cos(alsteers)
        p[:, 4], p[:, 5] = t0tx, alatx
        return 2, p
    if r0 == 0:
        orig = np.array([xele[-1] if s <= 0 else xele[0] for s in steers])
        s2 = np.arcsin(cm * np.sin(steers) / ctx)
        p[:, 0] = orig
        p[:, 2], p[:, 3] = np.sin(s2), np.cos(s2)
        return 0, p
    if ctx != cm:
        raise NotImplementedError("speed-of-sound correction is not defined for diverging waves")
    r = -np.abs(r0)
    O = np.array([r * np.sin(steers), r * np.cos(steers)]).T
    E = np.stack([xele, np.zeros_like(xele)], axis=1)
    tau0 = np.min(np.linalg.norm(E[None, :, :] - O[:, None, :], axis=-1) / ctx, axis=1)
    p[:, 0:2] = O
    p[:, 4] = tau0
    return 1, p


def make_tabs_and_apods_2d(steers, r0, ctx, cm, xele, xout, zout, fnum, hann=False,
                           device="cuda"):
    """{'tautx', 'taurx', 'apodtx', 'apodrx'}: float32 CUDA tensors of shape
    (ntx, nx*nz) / (nele, nx*nz), pixels meshgrid(xout, zout, 'ij') flattened.
    hann=True weights the receive F-number mask by a Hann window across the
    active aperture (the reference's mask is 0/1)."""
    L = _lib.load()
    kind, params = transmit_params_2d(steers, r0, ctx, cm, xele)
    params = np.ascontiguousarray(params, np.float64)
    d64 = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float64), device=device)
    xe, xo, zo = d64(xele), d64(xout), d64(zout)
    ntx, nele, nx, nz = params.shape[0], xe.numel(), xo.numel(), zo.numel()
    npix = nx * nz
    out = {k: torch.empty((n, npix), dtype=torch.float32, device=device)
           for k, n in (("tautx", ntx), ("apodtx", ntx), ("taurx", nele), ("apodrx", nele))}
    P = lambda t: ct.c_void_p(t.data_ptr())
    st = L.pycbf_gb_tables_2d(kind, ntx, params.ctypes.data_as(ct.c_void_p), nele, P(xe), nx, P(xo),
                              nz, P(zo), float(cm), float(fnum), int(bool(hann)), P(out["tautx"]),
                              P(out["apodtx"]), P(out["taurx"]), P(out["apodrx"]),
                              ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "pycbf_gb_tables_2d")
    return out

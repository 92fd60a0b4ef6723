"""Geometry helpers for linear arrays: delay tables, synthetic-point parameters, grids.

These build the constructor inputs of the beamformers, following the formulas
of the reference's helper module (pycbf/helpers/__full_aperture_2D__.py).
They run once per geometry, in float64 NumPy, off the timed path.
"""
from __future__ import annotations

import numpy as np


def element_positions(nele: int, pitch: float) -> np.ndarray:
    """Lateral centres of a linear array, symmetric about x = 0."""
    return pitch * (np.arange(nele) - (nele - 1) / 2.0)


def pixel_grid(xout: np.ndarray, zout: np.ndarray) -> np.ndarray:
    """(Np, 2) pixel positions in meshgrid('ij') order: z varies fastest.

    Same ordering as pycbf/helpers/__full_aperture_2D__.py:148-149, 387-388.
    """
    X, Z = np.meshgrid(xout, zout, indexing="ij")
    return np.ascontiguousarray(np.stack([X.ravel(), Z.ravel()], axis=1))


def rx_tables(cm, xele, xout, zout, fnum, hann: bool = False):
    """Receive delays |p - e| / c and the F-number mask (helpers :3-35).

    The mask is |dx| - dz / (2 fnum) < 0.  With hann=True the mask is weighted
    by a Hann window across the active aperture of each pixel:
    cos^2(pi/2 * dx / a), a = z / (2 fnum).
    """
    P = pixel_grid(xout, zout)
    dX = P[None, :, :] - np.stack([xele, np.zeros_like(xele)], axis=1)[:, None, :]
    taurx = np.linalg.norm(dX, axis=-1) / cm
    inside = np.abs(dX[..., 0]) - dX[..., 1] / (2 * fnum) < 0
    if not hann:
        return taurx, inside.astype(np.float64)
    half = np.maximum(dX[..., 1] / (2 * fnum), 1e-30)
    w = np.cos(0.5 * np.pi * np.clip(dX[..., 0] / half, -1.0, 1.0)) ** 2
    return taurx, np.where(inside, w, 0.0)


def pw_tx_tables(steers, ctx, cm, xele, xout, zout, ones: bool = False):
    """Plane-wave transmit delays and masks (helpers :129-168).

    The wave is timed from the array edge it leaves first: origin xele[-1]
    for steer <= 0, xele[0] otherwise.  ones=True gives an all-ones apodization.
    """
    steers = np.asarray(steers, np.float64)
    P = pixel_grid(xout, zout)
    O = np.stack([np.where(steers <= 0, xele[-1], xele[0]), np.zeros_like(steers)], axis=1)
    th = np.arcsin(cm * np.sin(steers) / ctx)
    N = np.stack([np.sin(th), np.cos(th)], axis=1)
    tautx = np.sum((P[None] - O[:, None]) * N[:, None], axis=-1) / cm
    if ones:
        return tautx, np.ones_like(tautx)
    Nperp = np.stack([-np.cos(th), np.sin(th)], axis=1)
    dneg = np.sum((P[None] - np.array([xele[0], 0.0])[None, None]) * Nperp[:, None], axis=-1)
    dpos = np.sum((P[None] - np.array([xele[-1], 0.0])[None, None]) * Nperp[:, None], axis=-1)
    return tautx, ((dneg <= 0) & (dpos >= 0)).astype(np.float64)


def pw_synthetic_points(steers, ctx, cm, xele, fnum, rpw: float = -10.0):
    """Synthetic-point parameters of plane waves approximated by far virtual
    sources, plus the receive points (helpers :205-268)."""
    steers = np.arcsin(cm * np.sin(np.asarray(steers, np.float64)) / ctx)
    orig = np.stack([np.where(steers <= 0, xele[-1], xele[0]), np.zeros_like(steers)], axis=1)
    nvectx = np.stack([np.sin(steers), np.cos(steers)], axis=1)
    ovectx = rpw * nvectx
    t0tx = np.sum(nvectx * (ovectx - orig), axis=-1) / cm
    doftx = np.zeros(len(t0tx))
    dxo = orig - ovectx
    alatx = np.arccos(np.abs(np.sum(dxo * nvectx, axis=-1)) / np.linalg.norm(dxo, axis=-1))
    nrx = len(xele)
    ovecrx = np.stack([xele, np.zeros(nrx)], axis=1)
    nvecrx = np.stack([np.zeros(nrx), np.ones(nrx)], axis=1)
    alarx = np.arctan2(0.5, fnum) * np.ones(nrx)
    return dict(ovectx=ovectx, nvectx=nvectx, t0tx=t0tx, doftx=doftx, alatx=alatx,
                ovecrx=ovecrx, nvecrx=nvecrx, alarx=alarx)


def pw_synthetic_planewaves(steers, xele, fnum):
    """True plane waves in the synthetic-point form: alatx = 0, so a transmit
    delay is (p - o) . n / c with o the array edge the wave leaves first (the
    geometry of pw_tx_tables), and receive elements with the F-number mask
    (pycbf/gpu/__engines__.cu:382-470: the ala == 0 branch of
    calc_tautx_apodtx has no mask and no t0)."""
    steers = np.asarray(steers, np.float64)
    orig = np.stack([np.where(steers <= 0, xele[-1], xele[0]), np.zeros_like(steers)], axis=1)
    nvectx = np.stack([np.sin(steers), np.cos(steers)], axis=1)
    z = np.zeros(len(steers))
    nrx = len(xele)
    ovecrx = np.stack([xele, np.zeros(nrx)], axis=1)
    nvecrx = np.stack([np.zeros(nrx), np.ones(nrx)], axis=1)
    alarx = np.arctan2(0.5, fnum) * np.ones(nrx)
    return dict(ovectx=orig, nvectx=nvectx, t0tx=z, doftx=z.copy(), alatx=z.copy(),
                ovecrx=ovecrx, nvecrx=nvecrx, alarx=alarx)


def korder_matrix(k: int) -> np.ndarray:
    """S = C^-1 P of k-point cubic interpolation (the published method of
    Praesius and Jensen, 2024), as pycbf/gpu/__core_bf_classes__.py:366-395
    builds it: C tridiagonal with 4 inside and 1 at the ends (2 beside them),
    P the matching difference operator.  float64 inverse, float32 result."""
    c00 = np.ones(k)
    c00[1:-1] = 4.0
    cp1 = np.ones(k - 1)
    cp1[0] = 2.0
    C = np.diag(c00) + np.diag(cp1, 1) + np.diag(cp1[::-1], -1)
    pp1 = 3.0 * np.ones(k - 1)
    pp1[0] = 2.0
    P = np.diag(pp1, 1) + np.diag(-pp1[::-1], -1)
    P[0, 0] = -2.5
    P[-1, -1] = 2.5
    P[0, 2] = 0.5
    P[-1, -3] = -0.5
    return np.ascontiguousarray(np.linalg.inv(C) @ P, dtype=np.float32)

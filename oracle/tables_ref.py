"""NumPy restatement of the reference's table helpers (test infrastructure).

Follows pycbf/helpers/__full_aperture_2D__.py: receive tables (:3-35),
diverging (:37-84), focused (:86-127, with the synthetic points of
:270-314) and plane-wave (:129-168) transmit tables, dispatched as
make_tabs_and_apods_2D (:170-203).  float64, masks as booleans, like the
reference; pinned against the reference's own output in
tests/golden/tables_2d.npz.
"""
import numpy as np

__all__ = ["make_tabs_and_apods_2d"]


def _grid(xout, zout):
    X, Z = np.meshgrid(xout, zout, indexing="ij")
    return np.array([X.flatten(), Z.flatten()]).T


def _rx(cm, xele, xout, zout, fnum):
    P = _grid(xout, zout)
    E = np.array([xele, np.zeros(len(xele))]).T
    d = P[None, :, :] - E[:, None, :]
    return np.linalg.norm(d, axis=-1) / cm, np.abs(d[..., 0]) - d[..., 1] / (2 * fnum) < 0


def _pw(steers, ctx, cm, xele, xout, zout):
    P = _grid(xout, zout)
    O = np.array([[xele[-1] if s <= 0 else xele[0] for s in steers], np.zeros(steers.shape)]).T
    s2 = np.arcsin(cm * np.sin(steers) / ctx)
    N = np.array([np.sin(s2), np.cos(s2)]).T
    tautx = np.sum((P[None] - O[:, None]) * N[:, None, :], axis=-1) / cm
    Np = np.array([-np.cos(s2), np.sin(s2)]).T
    dneg = np.sum((P[None] - np.array([xele[0], 0])[None, None]) * Np[:, None, :], axis=-1)
    dpos = np.sum((P[None] - np.array([xele[-1], 0])[None, None]) * Np[:, None, :], axis=-1)
    return tautx, (dneg <= 0) & (dpos >= 0)


def _div(steers, r0, cm, xele, xout, zout):
    r0 = -np.abs(r0)
    O = np.array([r0 * np.sin(steers), r0 * np.cos(steers)]).T
    E = np.array([xele, np.zeros(len(xele))]).T
    tau0 = np.min(np.linalg.norm(E[None] - O[:, None], axis=-1) / cm, axis=1, keepdims=True)
    P = _grid(xout, zout)
    tautx = np.linalg.norm(P[None] - O[:, None], axis=-1) / cm - tau0
    return tautx, np.ones(tautx.shape)


def _foc(steers, r0, cm, xele, xout, zout):
    ovectx = r0 * np.array([np.sin(steers), np.cos(steers)]).T
    dxmax = np.max(np.hypot(xele[None, :] - ovectx[:, 0, None], ovectx[:, 1, None]), axis=1)
    t0tx = dxmax / cm
    alneg = np.arctan2(ovectx[:, 0] - xele[0], ovectx[:, 1])
    alpos = np.arctan2(ovectx[:, 0] - xele[-1], ovectx[:, 1])
    alatx = -(alpos - alneg) / 2
    als = (alpos + alneg) / 2
    nvectx = np.array([np.sin(als), np.cos(als)]).T
    P = _grid(xout, zout)
    d = P[None] - ovectx[:, None]
    proj = np.sum(d * nvectx[:, None, :], axis=-1)
    mag = np.linalg.norm(d, axis=-1)
    tautx = np.sign(proj) * mag / cm + t0tx[:, None]
    mag[mag < 1e-12] = 1e-12
    return tautx, np.arccos(np.abs(proj) / mag) < alatx[:, None]


def make_tabs_and_apods_2d(steers, r0, ctx, cm, xele, xout, zout, fnum):
    steers = np.asarray(steers, np.float64)
    if r0 > 0:
        tautx, apodtx = _foc(steers, r0, cm, xele, xout, zout)
    elif r0 == 0:
        tautx, apodtx = _pw(steers, ctx, cm, xele, xout, zout)
    else:
        tautx, apodtx = _div(steers, r0, cm, xele, xout, zout)
    taurx, apodrx = _rx(cm, xele, xout, zout, fnum)
    return {"tautx": tautx, "taurx": taurx, "apodtx": apodtx, "apodrx": apodrx}

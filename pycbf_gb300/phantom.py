"""Seeded synthetic channel data and the named workloads.

Channel data are sums of Gaussian-modulated pulses (the pulse of
scipy.signal.gausspulse: exp(-a t^2) cos(2 pi fc t), a set by the fractional
bandwidth at -6 dB) at the two-way delays of point scatterers, plus white
noise at a fixed level below the signal RMS.  Each echo is evaluated only on
the samples where its envelope exceeds 1e-9, with torch on the given device.

Workloads (the defaults of the builders below):

* ``linear_pw_tabbed``: 128-element linear array, 0.3 mm pitch, 11 plane waves over
  -10..+10 deg, fs 25 MHz, 5 MHz pulse at 60 % bandwidth, Nt 2048, c 1540 m/s,
  20 bright points + 5000 N(0,1) speckle in x in [-19, 19] mm, z in [5, 45] mm,
  -40 dB noise; grid 256 x 512; tautx/taurx from the plane-wave geometry,
  apodtx all ones, apodrx a Hann window inside an F#1.5 mask.
* ``linear_pw_synthetic``: 192 elements, 0.2 mm pitch, 75 plane waves over -18..+18
  deg, fs 31.25 MHz, f0 6.25 MHz, Nt 4096, 40 000 speckle + 30 points, grid
  512 x 1024 over x in [-19.2, 19.2] mm, z in [5, 45] mm, synthetic-point
  geometry (virtual sources 10 m behind the array), F#1.5 receive.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import helpers


def gauss_pulse_a(fc: float, bw: float, bwr_db: float = -6.0) -> float:
    ref = 10.0 ** (bwr_db / 20.0)
    return -((math.pi * fc * bw) ** 2) / (4.0 * math.log(ref))


def simulate_channels(tau_tx: torch.Tensor, tau_rx: torch.Tensor, amp: torch.Tensor,
                      t0: float, dt: float, nt: int, fc: float, bw: float,
                      noise_db: float | None, seed: int) -> torch.Tensor:
    """rf[tx, rx, t] = sum_s amp[s] * pulse(t - tau_tx[tx, s] - tau_rx[rx, s]).

    tau_tx: (ntx, ns), tau_rx: (nrx, ns), amp: (ns,) on one device (float64).
    Returns float32 (ntx, nrx, nt) on that device.
    """
    dev = tau_tx.device
    ntx, ns = tau_tx.shape
    nrx = tau_rx.shape[0]
    a = gauss_pulse_a(fc, bw)
    half = int(math.ceil(math.sqrt(math.log(1e9) / a) / dt)) + 1
    offs = torch.arange(-half, half + 1, device=dev, dtype=torch.float64)
    chunk = max(1, int(2e7 // (ntx * nrx * offs.numel())))
    rf = torch.zeros(ntx * nrx * nt, dtype=torch.float64, device=dev)
    for s0 in range(0, ns, chunk):
        s1 = min(ns, s0 + chunk)
        tt = tau_tx[:, None, s0:s1] + tau_rx[None, :, s0:s1]            # (ntx, nrx, S)
        centre = torch.round((tt - t0) / dt)                            # nearest sample
        idx = centre[..., None] + offs                                  # (ntx, nrx, S, K)
        tloc = t0 + idx * dt - tt[..., None]
        val = amp[None, None, s0:s1, None] * torch.exp(-a * tloc * tloc) * torch.cos(
            2 * math.pi * fc * tloc)
        ok = (idx >= 0) & (idx < nt)
        base = (torch.arange(ntx * nrx, device=dev, dtype=torch.float64).view(ntx, nrx, 1, 1)
                * nt)
        flat = (base + idx.clamp(0, nt - 1)).long()
        rf.index_add_(0, flat[ok], val[ok])
    rf = rf.view(ntx, nrx, nt)
    if noise_db is not None:
        g = torch.Generator(device="cpu").manual_seed(seed + 1)
        rms = torch.sqrt(torch.mean(rf * rf)).item()
        noise = torch.randn(rf.shape, generator=g, dtype=torch.float64) * (
            rms * 10 ** (noise_db / 20.0))
        rf = rf + noise.to(dev)
    return rf.to(torch.float32)


def scatterers(seed: int, n_speckle: int, n_points: int, xlim, zlim, bright: float = 10.0,
               ndim: int = 2, ylim=None):
    """(positions (ns, ndim), amplitudes (ns,)) -- speckle N(0,1), points `bright`."""
    rng = np.random.default_rng(seed)
    ns = n_speckle + n_points
    pos = np.empty((ns, ndim))
    pos[:, 0] = rng.uniform(xlim[0], xlim[1], ns)
    if ndim == 3:
        pos[:, 1] = rng.uniform(ylim[0], ylim[1], ns)
    pos[:, -1] = rng.uniform(zlim[0], zlim[1], ns)
    amp = np.concatenate([rng.normal(0.0, 1.0, n_speckle), np.full(n_points, bright)])
    return pos, amp


@dataclass
class TabbedWorkload:
    name: str
    rf: np.ndarray            # (ntx, nrx, nt) float32
    tautx: np.ndarray         # (ntx, np) float32
    apodtx: np.ndarray
    taurx: np.ndarray         # (nrx, np) float32
    apodrx: np.ndarray
    t0: float
    dt: float
    nt: int
    grid: tuple = ()
    meta: dict = field(default_factory=dict)


@dataclass
class SyntheticWorkload:
    name: str
    rf: np.ndarray
    geometry: dict            # ovectx, nvectx, t0tx, doftx, alatx, ovecrx, nvecrx, alarx, c0, pnts
    t0: float
    dt: float
    nt: int
    grid: tuple = ()
    meta: dict = field(default_factory=dict)


def _device(device):
    if device is None:
        return torch.device("cuda" if torch.cuda.is_available() else "cpu")
    return torch.device(device)


def linear_pw_tabbed(nele=128, pitch=0.3e-3, nsteer=11, max_deg=10.0, fs=25e6, fc=5e6, bw=0.6,
                     nt=2048, c=1540.0, nx=256, nz=512, xlim=(-19e-3, 19e-3),
                     zlim=(5e-3, 45e-3), n_speckle=5000, n_points=20, fnum=1.5,
                     noise_db=-40.0, seed=1234, device=None, name="tabbed") -> TabbedWorkload:
    """Plane-wave Tabbed workload (defaults: the 128-element, 11-angle case)."""
    dev = _device(device)
    xele = helpers.element_positions(nele, pitch)
    steers = np.radians(np.linspace(-max_deg, max_deg, nsteer))
    xout = np.linspace(xlim[0], xlim[1], nx)
    zout = np.linspace(zlim[0], zlim[1], nz)
    tautx, _ = helpers.pw_tx_tables(steers, c, c, xele, xout, zout, ones=True)
    taurx, apodrx = helpers.rx_tables(c, xele, xout, zout, fnum, hann=True)
    pos, amp = scatterers(seed, n_speckle, n_points, xlim, zlim)
    # scatterer delays with the same formulas as the tables
    sx = pos[:, 0]
    sz = pos[:, 1]
    O = np.where(steers <= 0, xele[-1], xele[0])
    tt = ((sx[None] - O[:, None]) * np.sin(steers)[:, None] + sz[None] * np.cos(steers)[:, None]) / c
    tr = np.hypot(sx[None] - xele[:, None], sz[None]) / c
    t0, dt = 0.0, 1.0 / fs
    rf = simulate_channels(torch.tensor(tt, device=dev), torch.tensor(tr, device=dev),
                           torch.tensor(amp, device=dev), t0, dt, nt, fc, bw, noise_db, seed)
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    return TabbedWorkload(name, rf.cpu().numpy(), f32(tautx), np.ones_like(f32(tautx)), f32(taurx),
                          f32(apodrx), t0, dt, nt, (nx, nz),
                          dict(nele=nele, pitch=pitch, nsteer=nsteer, fs=fs, fc=fc, bw=bw, c=c,
                               fnum=fnum, seed=seed, xout=xout, zout=zout))


def linear_pw_synthetic(nele=192, pitch=0.2e-3, nsteer=75, max_deg=18.0, fs=31.25e6, fc=6.25e6,
                        bw=0.6, nt=4096, c=1540.0, nx=512, nz=1024, xlim=(-19.2e-3, 19.2e-3),
                        zlim=(5e-3, 45e-3), n_speckle=40000, n_points=30, fnum=1.5,
                        noise_db=-40.0, seed=4321, device=None,
                        name="synthetic") -> SyntheticWorkload:
    """Plane waves as far virtual sources (defaults: the 192-element, 75-angle case)."""
    dev = _device(device)
    xele = helpers.element_positions(nele, pitch)
    steers = np.radians(np.linspace(-max_deg, max_deg, nsteer))
    xout = np.linspace(xlim[0], xlim[1], nx)
    zout = np.linspace(zlim[0], zlim[1], nz)
    geo = helpers.pw_synthetic_points(steers, c, c, xele, fnum)
    pnts = helpers.pixel_grid(xout, zout)
    pos, amp = scatterers(seed, n_speckle, n_points, xlim, zlim)
    # echo delays from the same virtual-source model: sign(proj)|s-o|/c + t0tx
    d = pos[None, :, :] - geo["ovectx"][:, None, :]
    proj = np.sum(d * geo["nvectx"][:, None, :], axis=-1)
    tt = np.sign(proj) * np.linalg.norm(d, axis=-1) / c + geo["t0tx"][:, None]
    tr = np.linalg.norm(pos[None, :, :] - geo["ovecrx"][:, None, :], axis=-1) / c
    t0, dt = 0.0, 1.0 / fs
    rf = simulate_channels(torch.tensor(tt, device=dev), torch.tensor(tr, device=dev),
                           torch.tensor(amp, device=dev), t0, dt, nt, fc, bw, noise_db, seed)
    geo = dict(geo)
    geo["c0"] = c
    geo["pnts"] = pnts
    return SyntheticWorkload(name, rf.cpu().numpy(), geo, t0, dt, nt, (nx, nz),
                             dict(nele=nele, pitch=pitch, nsteer=nsteer, fs=fs, fc=fc, c=c,
                                  fnum=fnum, seed=seed, xout=xout, zout=zout))


def layered_slowness(z, c_top=1450.0, c_bottom=1560.0, z_interface=15e-3):
    """Mean slowness (s/m) along a straight path from depth 0 to depth z through
    a layer of speed c_top above z_interface and c_bottom below it."""
    z = np.maximum(np.asarray(z, np.float64), 1e-9)
    return (np.minimum(z, z_interface) / c_top + np.maximum(z - z_interface, 0.0) / c_bottom) / z


def two_layer_pw_synthetic(nele=128, pitch=0.3e-3, nsteer=11, max_deg=10.0, fs=25e6, fc=5e6,
                           bw=0.6, nt=2048, nx=256, nz=512, xlim=(-19e-3, 19e-3),
                           zlim=(5e-3, 45e-3), n_speckle=5000, n_points=20, fnum=1.5,
                           noise_db=-40.0, c_top=1450.0, c_bottom=1560.0, z_interface=15e-3,
                           c_nominal=1540.0, seed=2468, device=None,
                           name="two_layer") -> SyntheticWorkload:
    """Plane-wave synthetic workload in a two-layer medium (defaults: the
    128-element, 11-angle geometry; 1450 m/s to 15 mm, 1560 m/s below).

    Every echo delay is its straight path length times the mean slowness of
    the layers down to the scatterer's depth (layered_slowness), the model the
    slowness form of the delay-and-sum inverts.  meta['slowness_true'] holds
    that slowness at every pixel; geometry['c0'] is the nominal speed.
    """
    dev = _device(device)
    xele = helpers.element_positions(nele, pitch)
    steers = np.radians(np.linspace(-max_deg, max_deg, nsteer))
    xout = np.linspace(xlim[0], xlim[1], nx)
    zout = np.linspace(zlim[0], zlim[1], nz)
    geo = helpers.pw_synthetic_planewaves(steers, xele, fnum)
    pnts = helpers.pixel_grid(xout, zout)
    pos, amp = scatterers(seed, n_speckle, n_points, xlim, zlim)
    s_true = layered_slowness(pos[:, 1], c_top, c_bottom, z_interface)
    proj = np.sum((pos[None, :, :] - geo["ovectx"][:, None, :]) * geo["nvectx"][:, None, :], -1)
    tt = proj * s_true[None, :]
    tr = np.linalg.norm(pos[None, :, :] - geo["ovecrx"][:, None, :], axis=-1) * s_true[None, :]
    t0, dt = 0.0, 1.0 / fs
    rf = simulate_channels(torch.tensor(tt, device=dev), torch.tensor(tr, device=dev),
                           torch.tensor(amp, device=dev), t0, dt, nt, fc, bw, noise_db, seed)
    geo = dict(geo)
    geo["c0"] = c_nominal
    geo["pnts"] = pnts
    return SyntheticWorkload(name, rf.cpu().numpy(), geo, t0, dt, nt, (nx, nz),
                             dict(nele=nele, pitch=pitch, nsteer=nsteer, fs=fs, fc=fc, c=c_nominal,
                                  fnum=fnum, seed=seed, xout=xout, zout=zout,
                                  slowness_true=layered_slowness(pnts[:, 1], c_top, c_bottom,
                                                                 z_interface)))


def pw_tabbed_tables_torch(steers, xele, xout, zout, c, fnum, device):
    """The plane-wave tables of helpers.pw_tx_tables(ones=True) / rx_tables(hann=True),
    built with torch on the device (float32 results, float64 arithmetic)."""
    dev = _device(device)
    f64 = dict(dtype=torch.float64, device=dev)
    st = torch.as_tensor(np.asarray(steers, np.float64), **f64)
    xe = torch.as_tensor(np.asarray(xele, np.float64), **f64)
    X, Z = torch.meshgrid(torch.as_tensor(xout, **f64), torch.as_tensor(zout, **f64), indexing="ij")
    X, Z = X.reshape(-1), Z.reshape(-1)
    O = torch.where(st <= 0, xe[-1], xe[0])
    tautx = ((X[None] - O[:, None]) * torch.sin(st)[:, None] + Z[None] * torch.cos(st)[:, None]) / c
    dx = X[None] - xe[:, None]
    taurx = torch.sqrt(dx * dx + Z[None] * Z[None]) / c
    half = torch.clamp(Z[None] / (2 * fnum), min=1e-30)
    inside = dx.abs() - Z[None] / (2 * fnum) < 0
    w = torch.cos(0.5 * math.pi * torch.clamp(dx / half, -1.0, 1.0)) ** 2
    apodrx = torch.where(inside, w, torch.zeros_like(w))
    f32 = lambda t: t.to(torch.float32).contiguous()
    return f32(tautx), torch.ones_like(f32(tautx)), f32(taurx), f32(apodrx)


BATCH_NTX = (1, 5, 11, 31, 75)
BATCH_NRX = (64, 128, 192)
BATCH_NT = (1024, 2048, 4096)
BATCH_NX = (128, 256, 512)
BATCH_NZ = (128, 256, 512, 1024)


def batch_frames(n=64, seed=64, n_speckle=300, n_points=5, pitch=0.2e-3, max_deg=16.0,
                 window_s=64e-6, fnum=1.5, c=1540.0, device=None):
    """Seeded uneven frames: kind (tabbed / synthetic), ntx from BATCH_NTX, nrx
    from BATCH_NRX, nt from BATCH_NT, grid nx x nz from BATCH_NX x BATCH_NZ
    (128 x 128 .. 512 x 1024).  The record window is window_s for every nt
    (fs = nt / window_s, pulse centre fs / 5).  Returns dicts with the
    beamformer arguments (tables as CUDA tensors for Tabbed frames) and rf."""
    dev = _device(device)
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        kind = "tabbed" if rng.uniform() < 0.5 else "synthetic"
        ntx = int(rng.choice(BATCH_NTX))
        nrx = int(rng.choice(BATCH_NRX))
        nt = int(rng.choice(BATCH_NT))
        nx, nz = int(rng.choice(BATCH_NX)), int(rng.choice(BATCH_NZ))
        fs = nt / window_s
        fc = fs / 5.0
        xele = helpers.element_positions(nrx, pitch)
        half = 0.5 * nrx * pitch
        steers = np.radians(np.linspace(-max_deg, max_deg, ntx)) if ntx > 1 else np.zeros(1)
        xout = np.linspace(-half, half, nx)
        zout = np.linspace(5e-3, 45e-3, nz)
        pos, amp = scatterers(seed * 1000 + k, n_speckle, n_points, (-half, half), (5e-3, 45e-3))
        entry = dict(kind=kind, ntx=ntx, nrx=nrx, nt=nt, nx=nx, nz=nz, t0=0.0, dt=1.0 / fs)
        if kind == "tabbed":
            tautx, apodtx, taurx, apodrx = pw_tabbed_tables_torch(steers, xele, xout, zout, c,
                                                                  fnum, dev)
            O = np.where(steers <= 0, xele[-1], xele[0])
            tt = ((pos[None, :, 0] - O[:, None]) * np.sin(steers)[:, None]
                  + pos[None, :, 1] * np.cos(steers)[:, None]) / c
            entry.update(tautx=tautx, apodtx=apodtx, taurx=taurx, apodrx=apodrx)
        else:
            geo = helpers.pw_synthetic_points(steers, c, c, xele, fnum)
            d = pos[None, :, :] - geo["ovectx"][:, None, :]
            proj = np.sum(d * geo["nvectx"][:, None, :], axis=-1)
            tt = np.sign(proj) * np.linalg.norm(d, axis=-1) / c + geo["t0tx"][:, None]
            geo = dict(geo, c0=c, pnts=helpers.pixel_grid(xout, zout))
            entry.update(geometry=geo)
        tr = np.hypot(pos[None, :, 0] - xele[:, None], pos[None, :, 1]) / c
        entry["rf"] = simulate_channels(torch.tensor(tt, device=dev), torch.tensor(tr, device=dev),
                                        torch.tensor(amp, device=dev), 0.0, 1.0 / fs, nt, fc, 0.6,
                                        -40.0, seed * 1000 + k)
        out.append(entry)
    return out


def matrix_dw_synthetic(nside=32, pitch=0.3e-3, nvs=5, vs_behind=10e-3, fs=20e6, fc=3.5e6,
                        bw=0.6, nt=2048, c=1540.0, nvox=(128, 128, 256),
                        lims=((-10e-3, 10e-3), (-10e-3, 10e-3), (5e-3, 65e-3)), n_speckle=200_000,
                        n_points=50, fnum=1.5, noise_db=-40.0, seed=5353, device=None,
                        name="matrix_3d") -> SyntheticWorkload:
    """3-D diverging waves from a matrix array (defaults: 32 x 32 elements at
    0.3 mm, 25 virtual sources on a 5 x 5 grid 10 mm behind the array, fs 20
    MHz, 3.5 MHz pulse, Nt 2048, 128 x 128 x 256 voxels over 20 x 20 x 60 mm).

    Transmits are virtual sources (synthetic-point form with dof = 0): delay
    |p - v| / c - |v| ... written as sign(proj) |p - v| / c + t0tx with t0tx
    = -(distance from the source to the array plane) / c, acceptance angle
    covering the aperture; receives take the F-number mask."""
    dev = _device(device)
    e1 = helpers.element_positions(nside, pitch)
    ex, ey = np.meshgrid(e1, e1, indexing="ij")
    nele = nside * nside
    ovecrx = np.stack([ex.ravel(), ey.ravel(), np.zeros(nele)], axis=1)
    nvecrx = np.tile(np.array([0.0, 0.0, 1.0]), (nele, 1))
    alarx = np.arctan2(0.5, fnum) * np.ones(nele)
    half = 0.5 * nside * pitch
    v1 = np.linspace(-half, half, nvs)
    vx, vy = np.meshgrid(v1, v1, indexing="ij")
    ntx = nvs * nvs
    ovectx = np.stack([vx.ravel(), vy.ravel(), -vs_behind * np.ones(ntx)], axis=1)
    nvectx = np.tile(np.array([0.0, 0.0, 1.0]), (ntx, 1))
    t0tx = -vs_behind / c * np.ones(ntx)
    # the cone from each source through the whole aperture and beyond
    alatx = np.arctan2(2.0 * half, vs_behind) * np.ones(ntx)
    doftx = np.zeros(ntx)
    axes = [np.linspace(lo, hi, n) for (lo, hi), n in zip(lims, nvox)]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    pnts = np.ascontiguousarray(np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1))
    rng = np.random.default_rng(seed)
    ns = n_speckle + n_points
    pos = np.stack([rng.uniform(lo, hi, ns) for lo, hi in lims], axis=1)
    amp = np.concatenate([rng.normal(0.0, 1.0, n_speckle), np.full(n_points, 10.0)])
    d = pos[None, :, :] - ovectx[:, None, :]
    proj = np.sum(d * nvectx[:, None, :], axis=-1)
    tt = np.sign(proj) * np.linalg.norm(d, axis=-1) / c + t0tx[:, None]
    tr = np.linalg.norm(pos[None, :, :] - ovecrx[:, None, :], axis=-1) / c
    t0, dt = 0.0, 1.0 / fs
    rf = simulate_channels(torch.tensor(tt, device=dev), torch.tensor(tr, device=dev),
                           torch.tensor(amp, device=dev), t0, dt, nt, fc, bw, noise_db, seed)
    geo = dict(ovectx=ovectx, nvectx=nvectx, t0tx=t0tx, doftx=doftx, alatx=alatx, ovecrx=ovecrx,
               nvecrx=nvecrx, alarx=alarx, c0=c, pnts=pnts)
    return SyntheticWorkload(name, rf.cpu().numpy(), geo, t0, dt, nt, tuple(nvox),
                             dict(nside=nside, pitch=pitch, fs=fs, fc=fc, c=c, seed=seed))

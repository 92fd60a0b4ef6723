"""Generate the golden fixtures of tests/golden/ by running the reference itself.

Runs only where the reference checkout exists ($PYCBF_REF, else the default of
oracle/Makefile):

* the reference's own ``pycbf.cpu.TabbedBeamformer`` (pycbf/cpu/__core_bf_classes__.py)
  calling its own ``pycbf.c`` -- compiled by oracle/Makefile into a temporary
  copy of the package, since the checkout is read-only -- gives the Tabbed
  cubic / nearest outputs for every sumtype on small seeded cases, including
  edge cases (delays at t0, at t_max, past it, apodization exactly at the
  threshold, negative weights, 2- and 3-sample channels);
* the reference notebook's own SLSC function (calc_lagn_coherence, cell 2 of
  examples/advanced_beamforming.ipynb) and pixel loop (cell 6) run on a small
  per-element image, and its DMAS loop (cell 9, first statements);
* the known answer of examples/compare_interpolation_methods.ipynb (CPU nearest
  vs CPU cubic RMSE, printed at :571 as 35.48316740429086) is recomputed from
  data regenerated by tests/kat_interp.py, through the reference's classes.

Usage:  python tests/golden/make_golden.py [--ref CHECKOUT]
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))


def import_reference(ref_root: str):
    """Import the reference package from a temporary copy with its C library built in."""
    tmp = tempfile.mkdtemp(prefix="pycbf_ref_")
    shutil.copytree(os.path.join(ref_root, "pycbf"), os.path.join(tmp, "pycbf"))
    subprocess.run(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-shared",
                    "-I", os.path.join(tmp, "pycbf", "cpu"), "-o",
                    os.path.join(tmp, "pycbf", "cpu", "pycbf.so"),
                    os.path.join(tmp, "pycbf", "cpu", "pycbf.c"), "-lm"], check=True)
    sys.path.insert(0, tmp)
    import pycbf.cpu as refcpu  # noqa: E402
    return refcpu, tmp


def notebook_cells(path):
    with open(path) as fp:
        nb = json.load(fp)
    return ["".join(c["source"]) for c in nb["cells"] if c["cell_type"] == "code"]


def small_pw_case(seed=7, nele=16, nsteer=3, nt=256, nx=24, nz=32):
    from pycbf_gb300 import phantom
    w = phantom.linear_pw_tabbed(nele=nele, pitch=0.3e-3, nsteer=nsteer, max_deg=8.0, fs=25e6,
                                 fc=5e6, bw=0.6, nt=nt, nx=nx, nz=nz, xlim=(-2.4e-3, 2.4e-3),
                                 zlim=(3e-3, 7e-3), n_speckle=60, n_points=3, fnum=1.0,
                                 noise_db=-40, seed=seed, device="cpu")
    # apodtx: a taper so that the transmit weights are not all ones
    x = np.linspace(-1, 1, w.tautx.shape[1], dtype=np.float32)
    apodtx = np.stack([np.float32(0.5) + np.float32(0.5) * np.cos(np.float32(k) * x) ** 2
                       for k in range(nsteer)]).astype(np.float32)
    return dict(rf=w.rf, tautx=w.tautx, apodtx=apodtx, taurx=w.taurx, apodrx=w.apodrx,
                t0=np.float32(w.t0), dt=np.float32(w.dt), nt=np.int32(nt))


def edge_case(nt=64):
    """Hand-placed delays and weights that sit on every decision boundary."""
    rng = np.random.default_rng(11)
    dt = np.float32(1 / 20e6)
    t0 = np.float32(2e-6)
    xmax = np.float32(t0 + np.float32(dt * np.float32(nt - 1)))
    ntx, nrx = 2, 3
    taus = [t0, xmax, np.nextafter(xmax, np.float32(1)), np.nextafter(t0, np.float32(0)),
            np.float32(t0 + dt * np.float32(10)), np.float32(t0 + dt * np.float32(10.5)),
            np.float32(t0 - dt * np.float32(0.5)), np.float32(t0 - dt * np.float32(1.4)),
            np.float32(t0 - dt * np.float32(1.6)), np.float32(t0 + dt * np.float32(nt - 0.5)),
            np.float32(t0 + dt * np.float32(nt - 0.6)), np.float32(0.0)]
    npix = len(taus) * 3
    tautx = np.zeros((ntx, npix), np.float32)
    taurx = np.zeros((nrx, npix), np.float32)
    for p in range(npix):
        tautx[:, p] = taus[p % len(taus)]
    apodtx = np.ones((ntx, npix), np.float32)
    apodrx = np.ones((nrx, npix), np.float32)
    # weights: exactly at the threshold, just below, negative, zero
    apodrx[0, len(taus):2 * len(taus)] = np.float32(0.01)
    apodrx[1, len(taus):2 * len(taus)] = np.nextafter(np.float32(0.01), np.float32(0))
    apodrx[2, 2 * len(taus):] = np.float32(-0.5)
    apodtx[1, 2 * len(taus):] = np.float32(0.0)
    rf = rng.normal(size=(ntx, nrx, nt)).astype(np.float32)
    return dict(rf=rf, tautx=tautx, apodtx=apodtx, taurx=taurx, apodrx=apodrx, t0=t0, dt=dt,
                nt=np.int32(nt))


def short_case(nt):
    rng = np.random.default_rng(100 + nt)
    dt, t0 = np.float32(1.0), np.float32(0.0)
    npix = 40
    tautx = rng.uniform(-0.5, nt - 0.5, size=(1, npix)).astype(np.float32)
    taurx = np.zeros((2, npix), np.float32)
    apodtx = np.ones((1, npix), np.float32)
    apodrx = np.ones((2, npix), np.float32)
    rf = rng.normal(size=(1, 2, nt)).astype(np.float32)
    return dict(rf=rf, tautx=tautx, apodtx=apodtx, taurx=taurx, apodrx=apodrx, t0=t0, dt=dt,
                nt=np.int32(nt))


def run_reference(refcpu, case, kind, usf=1, sumtype="tx_and_rx"):
    interp = {"kind": kind} if kind == "cubic" else {"kind": kind, "usf": usf}
    bf = refcpu.TabbedBeamformer(tautx=case["tautx"], taurx=case["taurx"], apodtx=case["apodtx"],
                                 apodrx=case["apodrx"], t0=float(case["t0"]), dt=float(case["dt"]),
                                 nt=int(case["nt"]), interp=interp, sumtype=sumtype)
    out = np.asarray(bf(case["rf"]), dtype=np.float64)
    del bf
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--skip-kat", action="store_true")
    args = ap.parse_args()
    from oracle.oracle import ref_root
    refcpu, tmp = import_reference(args.ref or ref_root())

    # ---- Tabbed cases through the reference's own CPU class ----------------
    cases = {"pw_small": small_pw_case(), "edge": edge_case(), "short2": short_case(2),
             "short3": short_case(3)}
    for name, case in cases.items():
        outs = {}
        for sumtype in ("tx_and_rx", "tx_only", "rx_only", "none"):
            outs[f"cubic_{sumtype}"] = run_reference(refcpu, case, "cubic", sumtype=sumtype)
        outs["nearest_tx_and_rx"] = run_reference(refcpu, case, "nearest")
        outs["nearest_rx_only"] = run_reference(refcpu, case, "nearest", sumtype="rx_only")
        outs["nearest_usf4_tx_and_rx"] = run_reference(refcpu, case, "nearest", usf=4)
        for k, v in outs.items():
            if not np.all(np.isfinite(v)):
                raise SystemExit(f"{name}/{k}: the reference produced non-finite values")
        np.savez_compressed(os.path.join(HERE, f"tabbed_{name}.npz"), **case,
                            **{f"ref_{k}": v for k, v in outs.items()})
        print(f"tabbed_{name}.npz", {k: v.shape for k, v in outs.items()})

    # ---- SLSC and DMAS with the notebook's own code -------------------------
    cells = notebook_cells(os.path.join(args.ref, "examples", "advanced_beamforming.ipynb"))
    pick = lambda needle: next(c for c in cells if needle in c)
    ns = {"np": np}
    exec(pick("def calc_lagn_coherence"), ns)    # cell 2: calc_coherence, calc_lagn_coherence
    rng = np.random.default_rng(5)
    nrx, nx, nz, nlag, nkern = 20, 6, 40, 4, 2
    # a smooth correlated per-element image with a noisy patch and a dead element
    base = rng.normal(size=(nx, nz)).astype(np.float32)
    im = (base[None] + 0.4 * rng.normal(size=(nrx, nx, nz))).astype(np.float32)
    im[3] = 0.0
    mask = np.ones((nrx, nx, nz), bool)
    for e in range(nrx):                      # an aperture that grows with depth
        half = 2 + (np.arange(nz) * 8) // nz
        for ix in range(nx):
            centre = 3 * ix
            mask[e, ix] = np.abs(e - centre) <= half
    ns.update(dict(xout=np.arange(nx), zout=np.arange(nz), dsfx=1, dsfz=1, nkern=nkern, nlag=nlag,
                   apodrx_coherence=mask, im_txsum=im.astype(np.float64), time=lambda: 0.0,
                   tqdm=lambda it, **kw: it, print=lambda *a, **k: None))
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        exec(pick("locpeak = np.zeros"), ns)     # cell 6: the pixel loop -> locpeak
    locpeak = ns["locpeak"][:nx, :nz]
    # DMAS loop of cell 9 (its first statements, before the plotting)
    src9 = pick("dmas = 0").split("dz = zout")[0]
    ns2 = {"np": np, "im_txsum": im.astype(np.float64)}
    exec(src9, ns2)
    np.savez_compressed(os.path.join(HERE, "coherence_small.npz"), im=im, mask=mask.astype(np.uint8),
                        nlag=np.int32(nlag), nkern=np.int32(nkern), ref_slsc=locpeak,
                        ref_dmas=ns2["dmas"], ref_das=ns2["das"], dmas_nlag=np.int32(10))
    print("coherence_small.npz", locpeak.shape, np.asarray(ns2["dmas"]).shape)

    # ---- the interpolation known answer ------------------------------------
    if not args.skip_kat:
        import kat_interp
        d = kat_interp.make_data()
        bf = lambda kind: refcpu.TabbedBeamformer(
            tautx=d["tautxrx"], taurx=d["tautxrx"], apodtx=d["apod"], apodrx=d["apod"],
            t0=d["t"][0], dt=d["t"][1] - d["t"][0], nt=len(d["t"]), interp={"kind": kind})
        im_cubic = bf("cubic")(d["rf"])
        im_near = bf("nearest")(d["rf"])
        rmse = kat_interp.rmse_roi(im_near, im_cubic, d)
        with open(os.path.join(HERE, "kat_interp.json"), "w") as fp:
            json.dump({"rmse_cpu_nearest_vs_cubic": rmse, "notebook_value": 35.48316740429086,
                       "rmse_norm": kat_interp.rms_roi(im_cubic, d),
                       "checksum_cubic": float(np.sum(np.asarray(im_cubic, np.float64))),
                       "checksum_nearest": float(np.sum(np.asarray(im_near, np.float64)))}, fp,
                      indent=1)
        print("kat", rmse)
    shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()

"""How much the reference's Synthetic image depends on float rounding, per
geometry (test infrastructure; run where the reference checkout exists).

The reference accepts a transmit tap when acos(|proj/mag|) <= ala in float
(pycbf/gpu/__engines__.cu:412,427).  For plane waves modelled as virtual
sources far behind the array the acceptance angle is ~4.5e-4 rad, so
proj/mag lies within a few float steps of 1 and the decision depends on how
mag and proj were rounded.  This script beamforms each geometry with the
reference's kernels built two ways (every operation rounded alone, and with
multiply-adds contracted as NVRTC's default does) and with the oracle's
cosine compare, and prints the tap-mask flips and image differences.

    make -C oracle refgpu refgpu-fused
    python oracle/synthetic_mask_sensitivity.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from pycbf_gb300 import phantom  # noqa: E402

KEYS = ("ovectx", "nvectx", "doftx", "alatx", "t0tx", "ovecrx", "nvecrx", "alarx", "c0", "pnts")


def geometries():
    w = phantom.linear_pw_synthetic(nele=48, nsteer=9, nt=1536, nx=48, nz=96, n_speckle=2000,
                                    xlim=(-4.8e-3, 4.8e-3), zlim=(5e-3, 20e-3), device="cpu")
    yield "plane waves as virtual sources 10 m behind (48 el, 9 tx)", w
    w = phantom.matrix_dw_synthetic(nside=8, nvs=2, nt=1024, nvox=(12, 12, 24), n_speckle=300,
                                    lims=((-2e-3, 2e-3), (-2e-3, 2e-3), (5e-3, 15e-3)),
                                    device="cpu")
    yield "3-D diverging waves (8x8 el, 4 tx)", w


def main():
    if oracle.refgpu_lib() is None or oracle.refgpu_lib(contracted=True) is None:
        raise SystemExit("build the reference's kernels first: make -C oracle refgpu refgpu-fused")
    for name, w in geometries():
        g = w.geometry
        run = lambda contracted: oracle.das_synthetic_refgpu(w.rf, g, w.t0, w.dt, w.nt, "linear",
                                                             sumtype="none", contracted=contracted)
        plain, fused = run(False), run(True)
        tabs = oracle.synth_tables(*(g[k] for k in KEYS))
        orc = oracle.das_tabbed(w.rf, *tabs, w.t0, w.dt, w.nt, interp="linear_floor", thresh=0.01,
                                sumtype="none")
        ntx, nrx = np.shape(g["ovectx"])[0], np.shape(g["ovecrx"])[0]
        img = lambda a: a.reshape(ntx, nrx, -1).sum((0, 1))
        flips = lambda a, b: int(((a != 0) != (b != 0)).sum())
        print(name)
        print(f"  reference, contracted vs not: {flips(plain, fused)} of {plain.size} taps flip, "
              f"image rel-L2 {oracle.rel_l2(img(fused), img(plain)):.3g}")
        print(f"  oracle (cosine compare) vs reference: {flips(plain, orc)} taps flip, "
              f"image rel-L2 {oracle.rel_l2(img(orc), img(plain)):.3g}")


if __name__ == "__main__":
    main()

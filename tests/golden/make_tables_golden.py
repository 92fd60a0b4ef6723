"""Golden tables from the reference's own helper (run where the reference
checkout exists): pycbf.helpers.make_tabs_and_apods_2D for plane-wave,
diverging and focused transmits on a small grid, rounded to float32 as the
reference's classes round them before beamforming.

    python tests/golden/make_tables_golden.py /path/to/reference
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = {"pw": 0.0, "diverging": -20e-3, "focused": 30e-3}


def inputs():
    xele = 0.3e-3 * (np.arange(24) - 11.5)
    xout = np.linspace(-5e-3, 5e-3, 16)
    zout = np.linspace(2e-3, 30e-3, 32)
    steers = np.radians(np.linspace(-12, 12, 5))
    return steers, 1500.0, 1540.0, xele, xout, zout, 1.5


def main(ref):
    sys.path.insert(0, ref)
    from pycbf.helpers.__full_aperture_2D__ import make_tabs_and_apods_2D
    steers, ctx, cm, xele, xout, zout, fnum = inputs()
    out = {}
    for name, r0 in CASES.items():
        c = ctx if r0 == 0 else cm
        t = make_tabs_and_apods_2D(steers, r0, c, cm, xele, xout, zout, fnum)
        for k, v in t.items():
            out[f"{name}_{k}"] = np.asarray(v, np.float64).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "tables_2d.npz"), **out)


def oracle_ref_root() -> str:
    """The reference checkout: $PYCBF_REF, else the default of oracle/Makefile."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from oracle.oracle import ref_root
    return ref_root()


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else oracle_ref_root())

"""Golden synthetic-point parameters from the reference's own helpers (run
where the reference checkout exists): calc_tx_synthetic_points_pw_2D and
calc_rx_synthetic_points for plane waves with a speed-of-sound correction.

    python tests/golden/make_synth_points_golden.py /path/to/reference
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def inputs():
    xele = 0.2e-3 * (np.arange(32) - 15.5)
    steers = np.radians(np.linspace(-18, 18, 7))
    return steers, 1500.0, 1540.0, xele, 1.5, -10.0


def main(ref):
    sys.path.insert(0, ref)
    from pycbf.helpers.__full_aperture_2D__ import (calc_rx_synthetic_points,
                                                     calc_tx_synthetic_points_pw_2D)
    steers, ctx, cm, xele, fnum, rpw = inputs()
    ovectx, nvectx, t0tx, doftx, alatx = calc_tx_synthetic_points_pw_2D(steers, ctx, cm, xele, rpw)
    ovecrx, nvecrx, alarx = calc_rx_synthetic_points(xele, fnum)
    np.savez_compressed(os.path.join(HERE, "synth_points.npz"), ovectx=ovectx, nvectx=nvectx,
                        t0tx=t0tx, doftx=doftx, alatx=alatx, ovecrx=ovecrx, nvecrx=nvecrx,
                        alarx=alarx)


def oracle_ref_root() -> str:
    """The reference checkout: $PYCBF_REF, else the default of oracle/Makefile."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from oracle.oracle import ref_root
    return ref_root()


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else oracle_ref_root())

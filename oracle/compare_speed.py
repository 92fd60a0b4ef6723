"""Times the oracle's C restatement against the compiled reference (oracle/_ref)
on the same slice of the 11 x 128 x 2048 / 256 x 512 plane-wave workload:
the first 3 transmits, all receives and pixels, cubic interpolation.  Test
infrastructure: it shows that the port, which stands in for the reference
where the reference is not built, runs at the reference's speed.

Usage (from the repository root, after `make -C oracle all ref`):

    python oracle/compare_speed.py [--ntx 3] [--threads 1 3]
"""
import argparse
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from pycbf_gb300 import phantom  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ntx", type=int, default=3)
    ap.add_argument("--threads", type=int, nargs="+", default=[1, 3])
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    if oracle.ref_lib() is None:
        raise SystemExit("the compiled reference (oracle/_ref) is not built here")
    w = phantom.linear_pw_tabbed(device="cpu")
    sl = slice(0, a.ntx)
    c = np.ascontiguousarray
    args = (c(w.rf[sl]), c(w.tautx[sl]), c(w.apodtx[sl]), w.taurx, w.apodrx, w.t0, w.dt, w.nt)
    taps = a.ntx * w.taurx.shape[0] * w.tautx.shape[1]
    for threads in a.threads:
        for use_ref in (False, True):
            best = float("inf")
            for _ in range(a.reps):
                t = time.perf_counter()
                oracle.das_tabbed(*args, interp="cubic", threads=threads, use_ref=use_ref)
                best = min(best, time.perf_counter() - t)
            name = "reference" if use_ref else "port"
            print(f"threads={threads} {name:9s} {best:.3f} s  {taps / best:.3e} samples/s")


if __name__ == "__main__":
    main()

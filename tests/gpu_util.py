"""Helpers shared by the GPU parity tests."""
import json
import os

import numpy as np

from oracle import oracle

# The parity bar for float32 images: rel-L2 <= 1e-5 and max-abs <= 1e-4 of the peak.
REL_L2 = 1e-5
MAX_ABS_PEAK = 1e-4


def assert_image_close(out, ref, rel=REL_L2, peak=MAX_ABS_PEAK, what=""):
    out = np.asarray(out, np.float64).ravel()
    ref = np.asarray(ref, np.float64).ravel()
    assert out.shape == ref.shape, (out.shape, ref.shape)
    pk = np.max(np.abs(ref))
    if pk == 0:
        assert np.max(np.abs(out)) == 0, what
        return 0.0, 0.0
    r = oracle.rel_l2(out, ref)
    m = oracle.max_abs_rel_peak(out, ref)
    assert r <= rel and m <= peak, f"{what}: rel-L2 {r:.3e} (<= {rel}), max-abs/peak {m:.3e} (<= {peak})"
    return r, m


def report(name, **values):
    """Append a parity record to $PYCBF_PARITY_REPORT (JSON lines) when set."""
    path = os.environ.get("PYCBF_PARITY_REPORT")
    if not path:
        return
    with open(path, "a") as fp:
        fp.write(json.dumps({"case": name, **{k: float(v) for k, v in values.items()}}) + "\n")

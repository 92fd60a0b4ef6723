"""Golden IQ demodulation and log-compression vectors from the reference's
own example code (run where the reference checkout exists).

fft_tukey_demod and zout_fft_tukey_demod are defined in a notebook cell, not
in the package (examples/SyntheticPointBeamforming.ipynb cell 1); this script
takes that cell's source from the notebook file and executes it with a stand-in
`cupy` module (the function imports cupy but only uses it for CuPy inputs), so
the golden outputs are the reference's own code run on NumPy arrays.  The
display line of cell 11 (20*log10(env/percentile(env, 99) + 1e-10)) is taken
from the notebook the same way.  Inputs are float32 images (what the
beamformers return), passed as float64 so the outputs carry no float32
rounding of their own.

    python tests/golden/make_demod_golden.py /path/to/reference
"""
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NOTEBOOK = os.path.join("examples", "SyntheticPointBeamforming.ipynb")


def notebook_cells(ref):
    with open(os.path.join(ref, NOTEBOOK)) as f:
        nb = json.load(f)
    return ["".join(c["source"]) for c in nb["cells"]]


def reference_functions(ref):
    cells = notebook_cells(ref)
    src = next(c for c in cells if "def fft_tukey_demod" in c)
    stub = types.ModuleType("cupy")

    class _NotCupy:  # isinstance(x, cp.ndarray) is False for NumPy input
        pass

    stub.ndarray = _NotCupy
    sys.modules.setdefault("cupy", stub)
    ns = {}
    exec(compile(src, NOTEBOOK + ":cell-fft_tukey_demod", "exec"), ns)
    disp = next(c for c in cells if "np.percentile(env, 99)" in c)
    line = next(l.strip() for l in disp.splitlines() if l.strip().startswith("logged"))
    return ns["fft_tukey_demod"], ns["zout_fft_tukey_demod"], line


def rf_image(rng, nlines, n, dz, f0, c0=1540.0):
    """Echo-like lines: Gaussian-modulated pulses at random depths plus speckle."""
    z = np.arange(n) * dz
    k0 = 2 * f0 / c0
    img = 0.05 * rng.standard_normal((nlines, n))
    for ln in range(nlines):
        for _ in range(6):
            zc = rng.uniform(z[0], z[-1])
            sig = 1.5 / k0
            img[ln] += rng.uniform(0.2, 2.0) * np.exp(-0.5 * ((z - zc) / sig) ** 2) * np.cos(
                2 * np.pi * k0 * (z - zc) + rng.uniform(0, 2 * np.pi))
    return img.astype(np.float32)


def cases():
    rng = np.random.default_rng(20240613)
    c0 = 1540.0
    dz = 40e-3 / 511
    out = []
    # the examples' DAS band (1-9 MHz) on 512-sample lines
    out.append(dict(name="das_band", x=rf_image(rng, 24, 512, dz, 5e6), kmin=2 * 1e6 / c0,
                    kmax=2 * 9e6 / c0, ks=1 / dz, alpha=0.25, axis=-1, shiftit=True))
    # the DMAS band (5-12 MHz) on a finer grid, no shift
    dzf = 10e-3 / 511
    out.append(dict(name="noshift", x=rf_image(rng, 16, 512, dzf, 8e6), kmin=2 * 5e6 / c0,
                    kmax=2 * 12e6 / c0, ks=1 / dzf, alpha=0.25, axis=-1, shiftit=False))
    # a band above the Nyquist bin of the coarse grid: a single bin is kept
    out.append(dict(name="nyq", x=out[0]["x"][:5], kmin=2 * 5e6 / c0, kmax=2 * 12e6 / c0,
                    ks=1 / dz, alpha=0.25, axis=-1, shiftit=True))
    # odd line length, demodulated along axis 0, another window
    dz2 = 30e-3 / 300
    out.append(dict(name="axis0", x=np.ascontiguousarray(rf_image(rng, 7, 301, dz2, 4e6).T),
                    kmin=2 * 1.5e6 / c0, kmax=2 * 7e6 / c0, ks=1 / dz2, alpha=0.5, axis=0,
                    shiftit=True))
    # batch of frames (3, 10, 256), a narrow band
    dz3 = 20e-3 / 255
    out.append(dict(name="frames", x=rf_image(rng, 30, 256, dz3, 6e6).reshape(3, 10, 256),
                    kmin=2 * 4e6 / c0, kmax=2 * 8e6 / c0, ks=1 / dz3, alpha=0.25, axis=-1,
                    shiftit=True))
    return out, dz


def main(ref):
    demod, zdemod, logline = reference_functions(ref)
    cs, dz = cases()
    out = {}
    for c in cs:
        iq = demod(c["x"].astype(np.float64), kmin=c["kmin"], kmax=c["kmax"], ks=c["ks"],
                   alpha=c["alpha"], axis=c["axis"], shiftit=c["shiftit"])
        p = c["name"]
        out[f"{p}_x"] = c["x"]
        out[f"{p}_params"] = np.array([c["kmin"], c["kmax"], c["ks"], c["alpha"], c["axis"],
                                       float(c["shiftit"])])
        out[f"{p}_iq"] = np.asarray(iq, np.complex128)
    zout = 5e-3 + np.arange(512) * dz
    out["das_band_zout"] = zout
    out["das_band_zout_demod"] = zdemod(zout, 2 * 1e6 / 1540.0, 2 * 9e6 / 1540.0)
    ns = {"np": np, "env": np.abs(out["das_band_iq"])}
    exec(logline, ns)
    out["das_band_logged"] = ns["logged"]
    np.savez_compressed(os.path.join(HERE, "demod.npz"), **out)
    print("wrote demod.npz:", {k: v.shape for k, v in out.items()})


def oracle_ref_root() -> str:
    """The reference checkout: $PYCBF_REF, else the default of oracle/Makefile."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from oracle.oracle import ref_root
    return ref_root()


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else oracle_ref_root())

"""CPU oracle for the pycbf beamforming hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker (or as the timed CPU
baseline).  The product package ``pycbf_gb300`` never imports it.

Four layers:

* ``liboracle.so`` built from ``oracle/pycbf_oracle.c`` -- a float32
  restatement of the reference's C path (pycbf/cpu/pycbf.c) and of the
  formulas of its CUDA kernels and notebooks (see the C file's header).
* ``oracle/_ref/libpycbf_ref.so`` -- the reference's own ``pycbf.c`` compiled
  from its sources by ``oracle/Makefile`` (only where the reference checkout
  exists).  Used to pin the restatement and, when present, as the CPU baseline.
* ``oracle/_ref/libpycbf_refgpu.so`` -- the reference's CUDA delay-and-sum
  kernels (pycbf/gpu/__engines__.cu) compiled for the CPU where they lie,
  with oracle/refgpu_shim.h for the CUDA built-ins and oracle/refgpu_driver.cpp
  emulating their launches (only where the reference checkout exists).  Pins
  the restatement of the interpolators and the synthetic geometry that the
  reference has only on the GPU.
* float64 NumPy/SciPy restatements (``*_fp64``) -- the accuracy yardstick.

Pinning: tests/test_oracle.py checks the restatement against the golden
vectors in tests/golden/ (generated by importing the reference's own Python
package, tests/golden/make_golden.py) and against the compiled reference.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
import sys
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None
_REFGPU: dict = {}
_LOCK = threading.Lock()
_POLY_LOCK = threading.Lock()  # guards the C library's fusion switch
_NO_LOCK = __import__("contextlib").nullcontext()

INTERP_CODES = {"cubic": 0, "nearest": 1, "linear": 2, "linear_floor": 3}
SUMTYPE_CODES = {"none": 0, "tx_only": 1, "rx_only": 2, "tx_and_rx": 3}

_f = ct.c_float
_i = ct.c_int
_ll = ct.c_longlong
_p = ct.c_void_p


def build(force: bool = False) -> str:
    """Compile liboracle.so with oracle/Makefile; returns its path."""
    path = os.path.join(HERE, "_build", "liboracle.so")
    src = os.path.join(HERE, "pycbf_oracle.c")
    if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return path


def ref_root() -> str:
    """The reference checkout: $PYCBF_REF, else the default that oracle/Makefile
    names (its recipe is the one place that names this machine's checkout)."""
    env = os.environ.get("PYCBF_REF")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip()


def ref_src_copy() -> str:
    """The private copy of the reference's pycbf.c (oracle/_ref/src, never committed)."""
    return os.path.join(HERE, "_ref", "src", "pycbf.c")


def build_ref(ref_root_dir: str | None = None) -> str | None:
    """Compile the reference's own pycbf.c into oracle/_ref.

    Where the checkout exists, from its sources where they lie (and a private
    copy of the two C files is left in oracle/_ref/src, which is git-ignored);
    elsewhere -- the GPU host, which has no checkout -- from that copy.  None
    when neither exists."""
    root = ref_root_dir or ref_root()
    src = os.path.join(root, "pycbf", "cpu", "pycbf.c")
    env = dict(os.environ, PYCBF_REF=root)
    if os.path.exists(src):
        subprocess.run(["make", "-s", "-C", HERE, "ref-src"], check=True, env=env)
    elif not os.path.exists(ref_src_copy()):
        return None
    r = subprocess.run(["make", "-s", "-C", HERE, "ref"], capture_output=True, text=True, env=env)
    if r.returncode != 0:  # the baseline then falls back to the port
        print("oracle: the reference's pycbf.c did not build:\n" + r.stderr[-2000:],
              file=sys.stderr)
        return None
    return os.path.join(HERE, "_ref", "libpycbf_ref.so")


def lib() -> ct.CDLL:
    global _LIB
    with _LOCK:
        if _LIB is None:
            L = ct.CDLL(build())
            L.orc_spline_y2.argtypes = [_p, _i, _f, _p, _p]
            L.orc_cubic_point.argtypes = [_f, _p, _p, _i, _f, _f, _f]
            L.orc_cubic_point.restype = _f
            L.orc_xmax.argtypes = [_f, _f, _i]
            L.orc_xmax.restype = _f
            chan = [_f, _f, _i, _p, _i, _f, _p, _p, _p, _p, _p]
            L.orc_beamform_cubic.argtypes = chan
            L.orc_beamform_nearest.argtypes = chan + [_i]
            L.orc_beamform_linear.argtypes = chan + [_i]
            L.orc_das_tabbed.argtypes = [_i, _i, _f, _f, _i, _p, _i, _i, _ll, _f,
                                         _p, _p, _p, _p, _i, _p, _i, _i]
            L.orc_tap_census.argtypes = [_i, _i, _f, _f, _i, _i, _i, _ll, _f,
                                         _p, _p, _p, _p, _p, _p]
            L.orc_synth_tx.argtypes = [_i, _p, _p, _f, _f, _f, _f, _f, _f, _f, _p, _p, _p]
            L.orc_synth_rx.argtypes = [_i, _p, _p, _f, _f, _p, _p, _p]
            L.orc_synth_tables.argtypes = [_i, _ll, _p, _f, _i, _p, _p, _p, _p, _p, _p, _p, _p,
                                           _i, _p, _p, _p, _p, _p, _p, _p]
            L.orc_dmas.argtypes = [_p, _ll, _ll, _p, _i, _i, _i, _p]
            L.orc_slsc.argtypes = [_p, _p, _i, _i, _i, _i, _i, _p]
            L.orc_poly_index.argtypes = [_i, _f, _f, _f, _i]
            L.orc_poly_index.restype = _i
            L.orc_das_poly.argtypes = [_i, _i, _p, _f, _f, _i, _p, _i, _i, _ll, _f, _p, _p, _p, _p,
                                       _i, _p]
            L.orc_set_poly_fusion.argtypes = [_i]
            L.orc_set_poly_fusion.restype = None
            _LIB = L
        return _LIB


def ref_lib() -> ct.CDLL | None:
    """The reference's compiled pycbf.c, or None where it was not built."""
    global _REF
    with _LOCK:
        if _REF is None:
            path = os.path.join(HERE, "_ref", "libpycbf_ref.so")
            if not os.path.exists(path):
                return None
            try:
                R = ct.CDLL(path)
            except OSError:  # e.g. a binary built for another machine
                return None
            chan = [_f, _f, _i, _p, _i, _f, _p, _p, _p, _p, _p]
            R.beamform_cubic.argtypes = chan
            R.beamform_cubic.restype = None
            R.beamform_nearest.argtypes = chan + [_i]
            R.beamform_nearest.restype = None
            _REF = R
        return _REF


def build_refgpu(ref_root_dir: str | None = None, contracted: bool = False) -> str | None:
    """Compile the reference's CUDA kernels for the CPU into oracle/_ref when its
    checkout exists (oracle/refgpu_driver.cpp); contracted=True: the build with
    multiply-adds fused, as NVRTC's default does."""
    root = ref_root_dir or ref_root()
    src = os.path.join(root, "pycbf", "gpu", "__engines__.cu")
    if not os.path.exists(src):
        return None
    target = "refgpu-fused" if contracted else "refgpu"
    r = subprocess.run(["make", "-s", "-C", HERE, target], capture_output=True, text=True,
                       env=dict(os.environ, PYCBF_REF=root))
    if r.returncode != 0:  # the checker only: its tests skip without it
        print("oracle: the reference's kernels did not build:\n" + r.stderr[-2000:],
              file=sys.stderr)
        return None
    return os.path.join(HERE, "_ref", "libpycbf_refgpu_fused.so" if contracted
                        else "libpycbf_refgpu.so")


def refgpu_lib(contracted: bool = False) -> ct.CDLL | None:
    """The reference's CUDA delay-and-sum kernels compiled for the CPU, or None
    where they were not built.  contracted=True: the build with multiply-adds
    fused, as NVRTC's default does (make -C oracle refgpu-fused)."""
    name = "libpycbf_refgpu_fused.so" if contracted else "libpycbf_refgpu.so"
    with _LOCK:
        if name not in _REFGPU:
            path = os.path.join(HERE, "_ref", name)
            if not os.path.exists(path):
                return None
            try:
                R = ct.CDLL(path)
            except OSError:  # e.g. a binary built for another machine
                return None
            R.rgd_tabbed.argtypes = [_i, _i, _p, _f, _f, _i, _p, _ll, _ll, _ll, _ll, _p, _p, _p,
                                     _p, _i, _p]
            R.rgd_tabbed.restype = _i
            R.rgd_synthetic.argtypes = [_i, _i, _p, _f, _f, _i, _i, _p, _ll, _ll, _ll, _ll, _p, _p,
                                        _p, _p, _p, _p, _p, _p, _f, _p, _i, _p]
            R.rgd_synthetic.restype = _i
            R.rgd_dmas.argtypes = [_p, _ll, _ll, _p, _i, _i, _i, _p, _ll]
            R.rgd_dmas.restype = _i
            _REFGPU[name] = R
        return _REFGPU[name]


# the reference's interp flags (its jumpTable order) and -1 for its korder kernel
REFGPU_INTERP = {"nearest": 0, "linear": 1, "akima": 2, "makima": 3, "korder_cubic": -1}


def _refgpu_S(interp, k):
    if interp == "korder_cubic" and k > 0:
        return korder_S(k)
    return np.zeros((1, 1), np.float32)


def das_tabbed_refgpu(rf, tautx, apodtx, taurx, apodrx, t0, dt, nt, interp, k=4,
                      sumtype="tx_and_rx", contracted=False):
    """Tabbed image from the reference's own CUDA kernel
    (das_bmode_tabbed_multi_interp / _korder_cubic, pycbf/gpu/__engines__.cu:
    726-864) run on the CPU.  Its tap rule is |apodtx*apodrx| > 0.01."""
    R = refgpu_lib(contracted)
    if R is None:
        raise RuntimeError("the reference's kernels are not built (make -C oracle refgpu)")
    rf = _c32(rf)
    tautx, apodtx, taurx, apodrx = map(_c32, (tautx, apodtx, taurx, apodrx))
    nfr = rf.shape[0] if rf.ndim == 4 else 1
    ntx, nrx, np_ = tautx.shape[0], taurx.shape[0], tautx.shape[1]
    S = _refgpu_S(interp, k)
    out = np.zeros(nfr * out_size(sumtype, ntx, nrx, np_), dtype=np.float32)
    st = R.rgd_tabbed(REFGPU_INTERP[interp], int(k), _ptr(S), float(t0), float(dt), int(nt),
                      _ptr(rf), ntx, nrx, np_, nfr, _ptr(tautx), _ptr(apodtx), _ptr(taurx),
                      _ptr(apodrx), SUMTYPE_CODES[sumtype], _ptr(out))
    if st:
        raise ValueError("rgd_tabbed rejected its arguments")
    return out


def das_synthetic_refgpu(rf, geometry, t0, dt, nt, interp, k=4, sumtype="tx_and_rx",
                         contracted=False):
    """Synthetic-point image from the reference's own CUDA kernel
    (das_bmode_synthetic_multi_interp / _korder_cubic, pycbf/gpu/__engines__.cu:
    506-725, delays and masks of calc_tautx_apodtx / calc_taurx_apodrx :377-470)
    run on the CPU.  geometry: the constructor arrays (ovectx, nvectx, doftx,
    alatx, t0tx, ovecrx, nvecrx, alarx, c0, pnts).  korder receives k as the
    reference's launch passes it: an int32 in a float parameter."""
    R = refgpu_lib(contracted)
    if R is None:
        raise RuntimeError("the reference's kernels are not built (make -C oracle refgpu)")
    g = {name: _c32(geometry[name]) for name in ("ovectx", "nvectx", "doftx", "alatx", "t0tx",
                                                  "ovecrx", "nvecrx", "alarx", "pnts")}
    rf = _c32(rf)
    nfr = rf.shape[0] if rf.ndim == 4 else 1
    ntx, nrx = g["ovectx"].shape[0], g["ovecrx"].shape[0]
    np_, ndim = g["pnts"].shape
    S = _refgpu_S(interp, k)
    out = np.zeros(nfr * out_size(sumtype, ntx, nrx, np_), dtype=np.float32)
    st = R.rgd_synthetic(REFGPU_INTERP[interp], int(k), _ptr(S), float(t0), float(dt), int(nt),
                         int(ndim), _ptr(rf), ntx, nrx, np_, nfr, _ptr(g["ovectx"]),
                         _ptr(g["nvectx"]), _ptr(g["t0tx"]), _ptr(g["alatx"]), _ptr(g["doftx"]),
                         _ptr(g["ovecrx"]), _ptr(g["nvecrx"]), _ptr(g["alarx"]),
                         float(np.float32(geometry["c0"])), _ptr(g["pnts"]),
                         SUMTYPE_CODES[sumtype], _ptr(out))
    if st:
        raise ValueError("rgd_synthetic rejected its arguments")
    return out


def dmas_refgpu(im, nlag, power=False, sumlags=True, launched=None):
    """DMAS from the reference's own kernel (calc_dmas,
    pycbf/gpu/__advanced_engines__.cu:17-61) run on the CPU: im (nsep, np);
    the lags are the positions 0..nlag-1 (the kernel does not read the lag
    values).  launched: the number of threads the reference's class launches
    (ceil(ntx*nrx*nop/nthread)*nthread); default every (lag, image, pixel)."""
    R = refgpu_lib()
    if R is None:
        raise RuntimeError("the reference's kernels are not built (make -C oracle refgpu)")
    im = _c32(im)
    nsep, np_ = im.shape
    lags = np.arange(nlag, dtype=np.int32)
    out = np.zeros(np_ if sumlags else nlag * np_, dtype=np.float32)
    n = nlag * nsep * np_ if launched is None else int(launched)
    if R.rgd_dmas(_ptr(im), nsep, np_, _ptr(lags), int(nlag), int(bool(power)),
                  int(bool(sumlags)), _ptr(out), n):
        raise ValueError("rgd_dmas rejected its arguments")
    return out


def _c32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_p)


def out_size(sumtype: str, ntx: int, nrx: int, np_: int) -> int:
    return {"none": ntx * nrx * np_, "tx_only": nrx * np_, "rx_only": ntx * np_,
            "tx_and_rx": np_}[sumtype]


# ---------------------------------------------------------------------------
# Tabbed DAS, float32, the reference's loop order
# ---------------------------------------------------------------------------
def das_tabbed(rf, tautx, apodtx, taurx, apodrx, t0, dt, nt, interp="cubic", usf=1,
               thresh=1e-2, sumtype="tx_and_rx", threads=1, use_ref=False):
    """Float32 image of a Tabbed beamformer.

    With threads == 1 the accumulation order is the reference's
    (pycbf/cpu/__core_bf_classes__.py:240-245, tx-major, rx-minor, in place).
    With threads > 1 the transmits are split across threads, each with a
    private buffer, summed at the end (the same taps, another rounding order).
    use_ref=True calls the reference's own compiled beamform_cubic /
    beamform_nearest per channel instead of the restatement.
    """
    rf = _c32(rf)
    tautx, apodtx, taurx, apodrx = map(_c32, (tautx, apodtx, taurx, apodrx))
    ntx, nrx = tautx.shape[0], taurx.shape[0]
    np_ = tautx.shape[1]
    assert rf.shape == (ntx, nrx, nt)
    size = out_size(sumtype, ntx, nrx, np_)
    if use_ref:
        if threads > 1 and ntx > 1 and sumtype == "tx_and_rx":
            # the reference's beamform_* are reentrant: transmits on threads with
            # private images (ctypes releases the GIL), summed at the end
            with ThreadPoolExecutor(min(threads, ntx)) as ex:
                parts = list(ex.map(
                    lambda t: _das_tabbed_ref(rf[t:t + 1], tautx[t:t + 1], apodtx[t:t + 1], taurx,
                                              apodrx, t0, dt, nt, interp, usf, thresh, sumtype,
                                              size), range(ntx)))
            return np.sum(parts, axis=0, dtype=np.float32)
        return _das_tabbed_ref(rf, tautx, apodtx, taurx, apodrx, t0, dt, nt, interp, usf,
                               thresh, sumtype, size)
    L = lib()
    code = INTERP_CODES[interp]
    st = SUMTYPE_CODES[sumtype]

    def run(tx0, tx1):
        out = np.zeros(size, dtype=np.float32)
        L.orc_das_tabbed(code, int(usf), float(t0), float(dt), int(nt), _ptr(rf), ntx, nrx, np_,
                         float(thresh), _ptr(tautx), _ptr(apodtx), _ptr(taurx), _ptr(apodrx),
                         st, _ptr(out), tx0, tx1)
        return out

    if threads <= 1 or ntx == 1:
        return run(0, ntx)
    if sumtype in ("none", "rx_only"):
        # outputs are disjoint per transmit: one shared buffer, no reduction
        out = np.zeros(size, dtype=np.float32)

        def run_into(tx0, tx1):
            L.orc_das_tabbed(code, int(usf), float(t0), float(dt), int(nt), _ptr(rf), ntx, nrx,
                             np_, float(thresh), _ptr(tautx), _ptr(apodtx), _ptr(taurx),
                             _ptr(apodrx), st, _ptr(out), tx0, tx1)

        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda t: run_into(t, t + 1), range(ntx)))
        return out
    with ThreadPoolExecutor(min(threads, ntx)) as ex:
        parts = list(ex.map(lambda t: run(t, t + 1), range(ntx)))
    return np.sum(parts, axis=0, dtype=np.float32)


def _das_tabbed_ref(rf, tautx, apodtx, taurx, apodrx, t0, dt, nt, interp, usf, thresh,
                    sumtype, size):
    R = ref_lib()
    if R is None:
        raise RuntimeError("the reference C library was not built (oracle/Makefile ref)")
    ntx, nrx, np_ = tautx.shape[0], taurx.shape[0], tautx.shape[1]
    out = np.zeros(size, dtype=np.float32)
    for itx in range(ntx):
        for irx in range(nrx):
            if sumtype == "none":
                off = np_ * (irx + itx * nrx)
            elif sumtype == "tx_only":
                off = np_ * irx
            elif sumtype == "rx_only":
                off = np_ * itx
            else:
                off = 0
            args = [_f(t0), _f(dt), _i(nt), _ptr(rf[itx, irx]), _i(np_), _f(thresh),
                    _ptr(tautx[itx]), _ptr(apodtx[itx]), _ptr(taurx[irx]), _ptr(apodrx[irx]),
                    ct.c_void_p(out.ctypes.data + 4 * off)]
            if interp == "cubic":
                R.beamform_cubic(*args)
            elif interp == "nearest":
                R.beamform_nearest(*args, _i(usf))
            else:
                raise ValueError("the reference C path has cubic and nearest only")
    return out


def tap_census(tautx, apodtx, taurx, apodrx, t0, dt, nt, interp="cubic", usf=1, thresh=1e-2):
    """Per pixel: (number of contributing taps, sum of their sample indices)."""
    tautx, apodtx, taurx, apodrx = map(_c32, (tautx, apodtx, taurx, apodrx))
    ntx, nrx, np_ = tautx.shape[0], taurx.shape[0], tautx.shape[1]
    count = np.zeros(np_, dtype=np.int32)
    isum = np.zeros(np_, dtype=np.int64)
    code = {"nearest": 1, "korder_cubic": 4, "akima": 5, "makima": 6}.get(interp, 0)
    # the poly kinds' range test reads the C library's fusion switch
    lock = _POLY_LOCK if code >= 4 else _NO_LOCK
    with lock:
        lib().orc_tap_census(code, int(usf), float(t0), float(dt), int(nt), ntx, nrx, np_,
                             float(thresh), _ptr(tautx), _ptr(apodtx), _ptr(taurx),
                             _ptr(apodrx), _ptr(count), _ptr(isum))
    return count, isum


def _pixel_chunks(np_, threads, min_chunk=2048):
    n = max(1, min(4 * max(1, threads), -(-np_ // min_chunk)))
    edges = np.linspace(0, np_, n + 1).astype(np.int64)
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]


def das_tabbed_by_pixels(rf, tautx, apodtx, taurx, apodrx, t0, dt, nt, interp="cubic",
                         thresh=1e-2, sumtype="tx_and_rx", threads=1, min_chunk=2048):
    """das_tabbed over column ranges of the tables on a thread pool.

    Pixels are independent, so each pixel's taps are still added in the
    reference's own order (transmit-major, receive-minor, in place:
    pycbf/cpu/__core_bf_classes__.py:240-245) whatever the split; only the
    work is divided.  Sized for the large workloads (hundreds of millions of
    table entries): no per-thread copy of a whole output.
    """
    rf = _c32(rf)
    tautx, apodtx, taurx, apodrx = (np.asarray(a, np.float32) for a in (tautx, apodtx, taurx, apodrx))
    ntx, nrx, np_ = tautx.shape[0], taurx.shape[0], tautx.shape[1]
    rows = {"none": ntx * nrx, "tx_only": nrx, "rx_only": ntx, "tx_and_rx": 1}[sumtype]
    out = np.zeros((rows, np_), np.float32)

    def run(span):
        p0, p1 = span
        cols = [np.ascontiguousarray(a[:, p0:p1]) for a in (tautx, apodtx, taurx, apodrx)]
        part = das_tabbed(rf, *cols, t0, dt, nt, interp=interp, thresh=thresh, sumtype=sumtype,
                          threads=1)
        out[:, p0:p1] = part.reshape(rows, p1 - p0)

    with ThreadPoolExecutor(max(1, threads)) as ex:
        list(ex.map(run, _pixel_chunks(np_, threads, min_chunk)))
    return out.ravel()


def tap_census_by_pixels(tautx, apodtx, taurx, apodrx, t0, dt, nt, interp="cubic", thresh=1e-2,
                         threads=1, min_chunk=2048):
    """tap_census over column ranges of the tables on a thread pool (cubic and
    nearest; the per-pixel counts do not depend on the split)."""
    if interp not in ("cubic", "nearest", "linear"):
        raise ValueError("tap_census_by_pixels: cubic, linear or nearest")
    np_ = tautx.shape[1]
    count = np.zeros(np_, np.int32)
    isum = np.zeros(np_, np.int64)

    def run(span):
        p0, p1 = span
        cols = [np.ascontiguousarray(a[:, p0:p1]) for a in (tautx, apodtx, taurx, apodrx)]
        c, s = tap_census(*cols, t0, dt, nt, interp=interp, thresh=thresh)
        count[p0:p1] = c
        isum[p0:p1] = s

    with ThreadPoolExecutor(max(1, threads)) as ex:
        list(ex.map(run, _pixel_chunks(np_, threads, min_chunk)))
    return count, isum


def dmas_by_pixels(im, lags, power=False, threads=1, min_chunk=2048):
    """dmas (summed over lags) over column ranges of the per-element image."""
    im = np.asarray(im, np.float32)
    out = np.zeros(im.shape[1], np.float32)

    def run(span):
        p0, p1 = span
        out[p0:p1] = dmas(np.ascontiguousarray(im[:, p0:p1]), lags, power=power)

    with ThreadPoolExecutor(max(1, threads)) as ex:
        list(ex.map(run, _pixel_chunks(im.shape[1], threads, min_chunk)))
    return out


def slsc_by_lines(im, mask, nlag, nkern, threads=1, min_chunk=4):
    """slsc over ranges of lateral lines (the kernel is axial, so lines are
    independent).  im, mask: (nrx, nx, nz)."""
    im = np.asarray(im, np.float32)
    nrx, nx, nz = im.shape
    out = np.zeros((nx, nz), np.float64)

    def run(span):
        x0, x1 = span
        out[x0:x1] = slsc(np.ascontiguousarray(im[:, x0:x1]), np.asarray(mask)[:, x0:x1], nlag,
                          nkern)

    with ThreadPoolExecutor(max(1, threads)) as ex:
        list(ex.map(run, _pixel_chunks(nx, threads, min_chunk)))
    return out


def spline_y2(y, dt):
    y = _c32(y)
    n = y.shape[-1]
    y2 = np.empty(n, np.float32)
    u = np.empty(n, np.float32)
    lib().orc_spline_y2(_ptr(y), n, float(dt), _ptr(y2), _ptr(u))
    return y2


# ---------------------------------------------------------------------------
# synthetic-point geometry -> float32 tables (restated delay/mask formulas)
# ---------------------------------------------------------------------------
def synth_constants(alatx, doftx, alarx):
    """Per-element constants shared by the product and the oracle (float32)."""
    alatx = np.asarray(alatx, np.float32).astype(np.float64)
    doftx = np.asarray(doftx, np.float32).astype(np.float64)
    alarx = np.asarray(alarx, np.float32).astype(np.float64)
    cos_tx = np.cos(alatx).astype(np.float32)
    sec_tx = np.sqrt(1.0 + np.tan(alatx) ** 2).astype(np.float32)
    hds_tx = (doftx * np.sin(alatx) / 2.0).astype(np.float32)
    cos_rx = np.cos(alarx).astype(np.float32)
    return cos_tx, sec_tx, hds_tx, cos_rx


def synth_tables(ovectx, nvectx, doftx, alatx, t0tx, ovecrx, nvecrx, alarx, c0, pnts):
    pnts = _c32(pnts)
    ndim = pnts.shape[1]
    np_ = pnts.shape[0]
    ovectx, nvectx, ovecrx, nvecrx = map(_c32, (ovectx, nvectx, ovecrx, nvecrx))
    t0tx, alatx, doftx = map(_c32, (t0tx, alatx, doftx))
    cos_tx, sec_tx, hds_tx, cos_rx = synth_constants(alatx, doftx, alarx)
    ntx, nrx = ovectx.shape[0], ovecrx.shape[0]
    tautx = np.empty((ntx, np_), np.float32)
    apodtx = np.empty((ntx, np_), np.float32)
    taurx = np.empty((nrx, np_), np.float32)
    apodrx = np.empty((nrx, np_), np.float32)
    lib().orc_synth_tables(ndim, np_, _ptr(pnts), float(np.float32(c0)), ntx, _ptr(ovectx),
                           _ptr(nvectx), _ptr(t0tx), _ptr(alatx), _ptr(cos_tx), _ptr(sec_tx),
                           _ptr(hds_tx), _ptr(doftx), nrx, _ptr(ovecrx), _ptr(nvecrx),
                           _ptr(cos_rx), _ptr(tautx), _ptr(apodtx), _ptr(taurx), _ptr(apodrx))
    return tautx, apodtx, taurx, apodrx


# ---------------------------------------------------------------------------
# DMAS and SLSC
# ---------------------------------------------------------------------------
def dmas(im, lags, power=False, sumlags=True):
    im = _c32(im)
    nsep, np_ = im.shape
    lags = np.ascontiguousarray(lags, dtype=np.int32)
    out = np.zeros(np_ if sumlags else len(lags) * np_, np.float32)
    lib().orc_dmas(_ptr(im), nsep, np_, _ptr(lags), len(lags), int(power), int(sumlags),
                   _ptr(out))
    return out if sumlags else out.reshape(len(lags), np_)


def slsc(im, mask, nlag, nkern):
    """im, mask: (nrx, nx, nz).  Returns (nx, nz) float64."""
    im = _c32(im)
    nrx, nx, nz = im.shape
    m = np.ascontiguousarray(np.asarray(mask) != 0, dtype=np.uint8)
    out = np.zeros((nx, nz), np.float64)
    lib().orc_slsc(_ptr(im), _ptr(m), nrx, nx, nz, int(nlag), int(nkern), _ptr(out))
    return out


# ---------------------------------------------------------------------------
# float64 yardsticks
# ---------------------------------------------------------------------------
def das_tabbed_fp64(rf, tautx, apodtx, taurx, apodrx, t0, dt, nt, interp="cubic",
                    thresh=1e-2, sumtype="tx_and_rx", mask32=True):
    """Float64 DAS: SciPy natural cubic spline (or nearest) evaluated in double.

    The set of contributing taps is decided exactly as in float32 (mask32=True)
    so that the float64 image differs from the float32 one by arithmetic only.
    """
    from scipy.interpolate import CubicSpline

    rf = np.asarray(rf, np.float64)
    ntx, nrx, np_ = tautx.shape[0], taurx.shape[0], tautx.shape[1]
    t = t0 + dt * np.arange(nt, dtype=np.float64)
    t32 = np.float32(t0)
    xmax32 = lib().orc_xmax(float(t0), float(dt), int(nt))
    out = np.zeros(out_size(sumtype, ntx, nrx, np_), np.float64)
    ttx32, atx32, trx32, arx32 = map(_c32, (tautx, apodtx, taurx, apodrx))
    for itx in range(ntx):
        for irx in range(nrx):
            apod32 = atx32[itx] * arx32[irx]
            x32 = ttx32[itx] + trx32[irx]
            if interp == "cubic":
                ok = (np.abs(apod32) >= np.float32(thresh)) & (x32 >= t32) & (x32 <= xmax32)
                cs = CubicSpline(t, rf[itx, irx], bc_type="natural")
                x = np.asarray(tautx[itx], np.float64) + np.asarray(taurx[irx], np.float64)
                v = np.where(ok, cs(np.clip(x, t[0], t[-1])), 0.0)
            elif interp == "nearest":
                q = ((x32 - t32) / np.float32(dt)).astype(np.float64) + 0.5
                it = np.where((q > -2**31) & (q < 2**31 - 1), q, -1).astype(np.int64)
                ok = (np.abs(apod32) >= np.float32(thresh)) & (it >= 0) & (it < nt)
                v = np.where(ok, rf[itx, irx][np.clip(it, 0, nt - 1)], 0.0)
            else:
                raise ValueError(interp)
            apod = np.asarray(apodtx[itx], np.float64) * np.asarray(apodrx[irx], np.float64)
            contrib = np.where(ok, apod * v, 0.0)
            if sumtype == "none":
                out[np_ * (irx + itx * nrx):np_ * (irx + itx * nrx + 1)] += contrib
            elif sumtype == "tx_only":
                out[np_ * irx:np_ * (irx + 1)] += contrib
            elif sumtype == "rx_only":
                out[np_ * itx:np_ * (itx + 1)] += contrib
            else:
                out += contrib
    return out


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def max_abs_rel_peak(a, b) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    peak = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / peak) if peak > 0 else float(np.max(np.abs(a - b)))


def spline_z64(rf):
    """Float64 natural-spline records z = y'' dt^2 / 6 of every channel (last axis),
    the same system as pycbf.c:114-166 (0.5 z_i-1 + 2 z_i + 0.5 z_i+1 =
    (y_i+1 - 2 y_i + y_i-1) / 2, z_0 = z_n-1 = 0), by a banded solve."""
    from scipy.linalg import solve_banded

    rf = np.asarray(rf, np.float64)
    n = rf.shape[-1]
    flat = rf.reshape(-1, n).T
    z = np.zeros_like(flat)
    if n >= 3:
        d = flat[2:] - 2.0 * flat[1:-1] + flat[:-2]
        ab = np.zeros((3, n - 2))
        ab[0, 1:] = 0.5
        ab[1, :] = 2.0
        ab[2, :-1] = 0.5
        z[1:-1] = solve_banded((1, 1), ab, 0.5 * d)
    return z.T.reshape(rf.shape)


def das_fp64_columns(rf, tautx, apodtx, taurx, apodrx, t0, dt, thresh=1e-2, z=None):
    """Float64 'tx_and_rx' image of the given table columns (any subset of the
    pixels): natural cubic spline in double, taps decided as in float32
    (|fl(apodtx apodrx)| >= thresh, t0 <= fl(tautx + taurx) <= xmax,
    pycbf.c:68-105, 179-207), values at the float64 delay sum."""
    rf64 = np.asarray(rf, np.float64)
    ntx, nrx, nt = rf64.shape
    z = spline_z64(rf64) if z is None else z
    ttx32, atx32, trx32, arx32 = map(_c32, (tautx, apodtx, taurx, apodrx))
    x32 = ttx32[:, None, :] + trx32[None, :, :]
    apod32 = atx32[:, None, :] * arx32[None, :, :]
    xmax32 = lib().orc_xmax(float(t0), float(dt), int(nt))
    with np.errstate(invalid="ignore"):
        ok = (np.abs(apod32) >= np.float32(thresh)) & (x32 >= np.float32(t0)) & (x32 <= xmax32)
    x = ttx32.astype(np.float64)[:, None, :] + trx32.astype(np.float64)[None, :, :]
    q = np.where(ok, (x - float(np.float32(t0))) / float(np.float32(dt)), 0.0)
    j = np.clip(np.floor(q), 0, max(nt - 2, 0)).astype(np.int64)
    a = (j + 1) - q
    b = q - j
    t_i = np.arange(ntx)[:, None, None]
    r_i = np.arange(nrx)[None, :, None]
    j1 = np.minimum(j + 1, nt - 1)
    s = (a * rf64[t_i, r_i, j] + b * rf64[t_i, r_i, j1] + (a ** 3 - a) * z[t_i, r_i, j]
         + (b ** 3 - b) * z[t_i, r_i, j1])
    apod = atx32.astype(np.float64)[:, None, :] * arx32.astype(np.float64)[None, :, :]
    return np.where(ok, apod * s, 0.0).sum(axis=(0, 1))


POLY_CODES = {"korder_cubic": 4, "akima": 5, "makima": 6}


def korder_S(k):
    """The k x k derivative matrix of korder cubic interpolation, C^-1 P
    (pycbf/gpu/__core_bf_classes__.py:366-395, from the published k-point
    method of Praesius and Jensen), float64 then rounded to float32."""
    c00 = np.ones(k)
    c00[1:-1] = 4
    cp1 = np.ones(k - 1)
    cp1[0] = 2
    C = np.diag(c00) + np.diag(cp1, 1) + np.diag(cp1[::-1], -1)
    pp1 = 3 * np.ones(k - 1)
    pp1[0] = 2
    P = np.diag(pp1, 1) + np.diag(-pp1[::-1], -1)
    P[0, 0] = -2.5
    P[-1, -1] = 2.5
    P[0, 2] = 0.5
    P[-1, -3] = -0.5
    return (np.linalg.inv(C) @ P).astype(np.float32)


def das_poly(rf, tautx, apodtx, taurx, apodrx, t0, dt, nt, interp, k=8, S=None, thresh=1e-2,
             sumtype="tx_and_rx", fused=True):
    """Float32 Tabbed image with korder_cubic (k, S), akima or makima (restated
    from pycbf/gpu/__engines__.cu:58-355).  fused=False rounds the multiply-adds
    that the device contracts in two steps, as a host build of the reference's
    kernels does."""
    rf = _c32(rf)
    tautx, apodtx, taurx, apodrx = map(_c32, (tautx, apodtx, taurx, apodrx))
    ntx, nrx, np_ = tautx.shape[0], taurx.shape[0], tautx.shape[1]
    code = POLY_CODES[interp]
    if code == 4 and k > 0:
        S = korder_S(k) if S is None else _c32(S)
    else:  # akima / makima, or korder with k = 0 (zero derivative estimates)
        S, k = np.zeros((1, 1), np.float32), 0
    out = np.zeros(out_size(sumtype, ntx, nrx, np_), dtype=np.float32)
    L = lib()
    with _POLY_LOCK:
        L.orc_set_poly_fusion(int(bool(fused)))
        try:
            L.orc_das_poly(code, int(k), _ptr(S), float(t0), float(dt), int(nt), _ptr(rf), ntx,
                           nrx, np_, float(thresh), _ptr(tautx), _ptr(apodtx), _ptr(taurx),
                           _ptr(apodrx), SUMTYPE_CODES[sumtype], _ptr(out))
        finally:
            L.orc_set_poly_fusion(1)
    return out

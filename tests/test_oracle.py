"""The oracle is pinned before it is trusted (CPU only).

* Tabbed cubic / nearest outputs of the reference's own CPU class, every
  sumtype, on seeded and edge cases (tests/golden/tabbed_*.npz) -- bit-exact.
* The reference's own pycbf.c compiled here (oracle/_ref), where present --
  bit-exact on the same inputs.
* The interpolation known answer of the reference notebook (35.48316740429086),
  and the notebook's RMSEs of the reference's GPU nearest / linear / akima /
  makima, reproduced by its CUDA kernels compiled for the CPU.
* SLSC and DMAS outputs of the reference notebook's own code.
* The float64 yardstick agrees with the float32 oracle to float32 accuracy.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle

CASES = ["pw_small", "edge", "short2", "short3"]
HERE = os.path.dirname(os.path.abspath(__file__))


def _run(case, kind, sumtype="tx_and_rx", usf=1, **kw):
    return oracle.das_tabbed(case["rf"], case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
                             float(case["t0"]), float(case["dt"]), int(case["nt"]), interp=kind,
                             usf=usf, sumtype=sumtype, **kw)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only", "rx_only", "none"])
def test_cubic_matches_reference_golden(golden, name, sumtype):
    case = golden(f"tabbed_{name}.npz")
    out = _run(case, "cubic", sumtype)
    ref = case[f"ref_cubic_{sumtype}"]
    np.testing.assert_array_equal(out.astype(np.float64), ref)


@pytest.mark.parametrize("name", CASES)
def test_nearest_matches_reference_golden(golden, name):
    case = golden(f"tabbed_{name}.npz")
    np.testing.assert_array_equal(_run(case, "nearest").astype(np.float64),
                                  case["ref_nearest_tx_and_rx"])
    np.testing.assert_array_equal(_run(case, "nearest", "rx_only").astype(np.float64),
                                  case["ref_nearest_rx_only"])
    np.testing.assert_array_equal(_run(case, "nearest", usf=4).astype(np.float64),
                                  case["ref_nearest_usf4_tx_and_rx"])


@pytest.mark.parametrize("name", CASES)
def test_restatement_matches_compiled_reference(golden, name):
    if oracle.ref_lib() is None:
        pytest.skip("the reference C library is not built here")
    case = golden(f"tabbed_{name}.npz")
    # At x == xmax the reference reads y[N], y2[N] one past its channel buffers
    # (pycbf.c:103) with zero weights; a non-finite heap value there poisons its
    # output, so those pixels are compared only through the golden fixtures.
    x = case["tautx"][:, None, :] + case["taurx"][None, :, :]
    xmax = np.float32(oracle.lib().orc_xmax(float(case["t0"]), float(case["dt"]), int(case["nt"])))
    clean = ~np.any(x == xmax, axis=(0, 1))
    np.testing.assert_array_equal(_run(case, "cubic")[clean], _run(case, "cubic", use_ref=True)[clean])
    np.testing.assert_array_equal(_run(case, "nearest"), _run(case, "nearest", use_ref=True))


def test_threaded_reference_matches_serial(golden):
    """The reference arm runs the compiled reference on threads over transmits
    (private images, summed at the end): the same taps, another rounding order."""
    if oracle.ref_lib() is None:
        pytest.skip("the reference C library is not built here")
    case = golden("tabbed_pw_small.npz")
    args = (case["rf"], case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
            float(case["t0"]), float(case["dt"]), int(case["nt"]))
    serial = oracle.das_tabbed(*args, use_ref=True)
    threaded = oracle.das_tabbed(*args, use_ref=True, threads=4)
    ok = np.isfinite(serial)
    assert oracle.rel_l2(threaded[ok], serial[ok]) <= 1e-6


def test_threaded_oracle_same_taps(golden):
    case = golden("tabbed_pw_small.npz")
    one = _run(case, "cubic")
    many = _run(case, "cubic", threads=3)
    assert oracle.rel_l2(many, one) < 1e-6


def test_census_counts_match_image_support(golden):
    case = golden("tabbed_edge.npz")
    cnt, isum = oracle.tap_census(case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
                                  float(case["t0"]), float(case["dt"]), int(case["nt"]))
    # pixels 0..11 of the first block: every (tx, rx) tap has weight 1
    ntx, nrx = case["tautx"].shape[0], case["taurx"].shape[0]
    assert cnt.max() <= ntx * nrx
    # t0 exactly and xmax exactly are in range; one ulp past xmax and one before t0 are not
    assert cnt[0] == ntx * nrx and cnt[1] == ntx * nrx
    assert cnt[2] == 0 and cnt[3] == 0
    # apodization exactly at the threshold counts, one ulp below does not
    blk = slice(12, 24)
    assert np.all(cnt[blk][:2] == (ntx * nrx - ntx))  # receive 1 below the threshold
    assert isum[0] == 0 and isum[1] == ntx * nrx * (int(case["nt"]) - 1)


def test_spline_y2_natural_boundary():
    y = np.sin(np.linspace(0, 6, 200)).astype(np.float32)
    y2 = oracle.spline_y2(y, 0.03)
    assert y2[0] == 0 and y2[-1] == 0
    from scipy.interpolate import CubicSpline
    cs = CubicSpline(np.arange(200) * 0.03, y.astype(np.float64), bc_type="natural")
    np.testing.assert_allclose(y2, cs(np.arange(200) * 0.03, 2), atol=2e-3)


def test_fp64_yardstick_close(golden):
    case = golden("tabbed_pw_small.npz")
    out32 = _run(case, "cubic")
    out64 = oracle.das_tabbed_fp64(case["rf"], case["tautx"], case["apodtx"], case["taurx"],
                                   case["apodrx"], float(case["t0"]), float(case["dt"]),
                                   int(case["nt"]))
    assert oracle.rel_l2(out32, out64) < 1e-5


def test_slsc_matches_notebook_code(golden):
    g = golden("coherence_small.npz")
    out = oracle.slsc(g["im"], g["mask"], int(g["nlag"]), int(g["nkern"]))
    ref = g["ref_slsc"]
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    ok = ~np.isnan(ref)
    np.testing.assert_allclose(out[ok], ref[ok], rtol=1e-9, atol=1e-12)
    assert np.count_nonzero(ref[ok]) > 10  # the case is not trivial


def test_dmas_matches_notebook_code(golden):
    g = golden("coherence_small.npz")
    nrx, nx, nz = g["im"].shape
    lags = np.arange(1, int(g["dmas_nlag"]) + 1)
    out = oracle.dmas(g["im"].reshape(nrx, nx * nz), lags).reshape(nx, nz)
    np.testing.assert_allclose(out, g["ref_dmas"], rtol=2e-6, atol=1e-5)


def test_dmas_reference_kernel_lag_positions():
    # the reference kernel uses the lag's position as the lag: with lags = arange(nlag)
    # the two conventions coincide (lag 0 adds |x|)
    rng = np.random.default_rng(3)
    im = rng.normal(size=(7, 50)).astype(np.float32)
    out = oracle.dmas(im, np.arange(4), sumlags=False)
    np.testing.assert_allclose(out[0], np.abs(im).sum(0), rtol=1e-6)


@pytest.fixture(scope="module")
def kat():
    """The notebook's seeded data (tests/kat_interp.py), its argument tuple and
    the CPU cubic image every RMSE is taken against."""
    import kat_interp
    d = kat_interp.make_data()
    args = (d["rf"], d["tautxrx"], d["apod"], d["tautxrx"], d["apod"], d["t"][0],
            d["t"][1] - d["t"][0], len(d["t"]))
    return d, args, oracle.das_tabbed(*args, interp="cubic")


@pytest.mark.slow
def test_interp_known_answer(kat):
    import kat_interp
    d, args, cubic = kat
    near = oracle.das_tabbed(*args, interp="nearest")
    rmse = kat_interp.rmse_roi(near, cubic, d)
    assert abs(rmse - kat_interp.NOTEBOOK_RMSE) <= 1e-9 * kat_interp.NOTEBOOK_RMSE
    with open(os.path.join(HERE, "golden", "kat_interp.json")) as fp:
        recorded = json.load(fp)
    assert abs(float(np.sum(cubic.astype(np.float64))) - recorded["checksum_cubic"]) < 1e-6 * abs(
        recorded["checksum_cubic"])


# RMSEs against the CPU cubic image that the notebook printed for the
# reference's GPU classes (compare_interpolation_methods.ipynb, cell 10 output)
GPU_KAT = {"nearest": (35.48316740429086, 1e-6), "linear": (246.199658213788, 1e-7),
           "akima": (246.1996543436526, 1e-7), "makima": (246.19965454650733, 1e-7)}


@pytest.mark.slow
@pytest.mark.parametrize("kind", list(GPU_KAT))
def test_reference_gpu_known_answers(kat, kind):
    """The reference's CUDA kernels compiled for the CPU (oracle/_ref) reproduce
    the notebook's device-run RMSEs (float summation order aside: nearest
    2e-7, the others 5e-9 relative); the oracle equals that build bit for bit
    on the golden cases (tests/test_reference_kernels.py).  linear returns the
    floor sample, and akima / makima multiply per-sample slopes by a delta in
    seconds, so all three sit at ~246.2, about half the image RMS."""
    import kat_interp
    if oracle.refgpu_lib() is None:
        pytest.skip("the reference's kernels are not built here")
    d, args, cubic = kat
    want, tol = GPU_KAT[kind]
    got = kat_interp.rmse_roi(oracle.das_tabbed_refgpu(*args, interp=kind), cubic, d)
    assert abs(got - want) <= tol * want


def test_fp64_columns_agree_with_the_scipy_spline():
    """das_fp64_columns (banded float64 spline on the float32 time axis) and
    das_tabbed_fp64 (SciPy CubicSpline on the float64 axis) agree to the
    axis difference (~1e-6)."""
    from pycbf_gb300 import phantom
    w = phantom.linear_pw_tabbed(nele=16, nsteer=3, nt=512, nx=24, nz=40, xlim=(-2.4e-3, 2.4e-3),
                                 zlim=(4e-3, 12e-3), n_speckle=200, n_points=3, device="cpu")
    a = oracle.das_tabbed_fp64(w.rf, w.tautx, w.apodtx, w.taurx, w.apodrx, w.t0, w.dt, w.nt)
    sub = np.arange(0, w.tautx.shape[1], 7)
    c = oracle.das_fp64_columns(w.rf, w.tautx[:, sub], w.apodtx[:, sub], w.taurx[:, sub],
                                w.apodrx[:, sub], w.t0, w.dt)
    assert oracle.rel_l2(c, a[sub]) <= 1e-5


def test_pixel_split_oracle_equals_whole(golden):
    """The pixel-range thread split keeps every pixel's summation order: the
    image, the per-element image, the census, DMAS and SLSC equal the whole-range
    calls bit for bit."""
    case = golden("tabbed_pw_small.npz")
    args = (case["rf"], case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
            float(case["t0"]), float(case["dt"]), int(case["nt"]))
    for sumtype in ("tx_and_rx", "tx_only", "none"):
        whole = oracle.das_tabbed(*args, sumtype=sumtype, threads=1)
        split = oracle.das_tabbed_by_pixels(*args, sumtype=sumtype, threads=3, min_chunk=50)
        np.testing.assert_array_equal(whole, split)
    np.testing.assert_array_equal(np.stack(oracle.tap_census(*args[1:])),
                                  np.stack(oracle.tap_census_by_pixels(*args[1:], threads=3, min_chunk=50)))
    nrx = case["taurx"].shape[0]
    sep = oracle.das_tabbed(*args, sumtype="tx_only").reshape(nrx, -1)
    lags = np.arange(1, nrx)
    np.testing.assert_array_equal(oracle.dmas(sep, lags), oracle.dmas_by_pixels(sep, lags, threads=3, min_chunk=50))
    nx, nz = 24, 32
    mask = np.abs(case["apodrx"]).reshape(nrx, nx, nz) >= np.float32(0.01)
    a = oracle.slsc(sep.reshape(nrx, nx, nz), mask, 4, 2)
    b = oracle.slsc_by_lines(sep.reshape(nrx, nx, nz), mask, 4, 2, threads=3, min_chunk=2)
    np.testing.assert_array_equal(a, b)

"""IQ demodulation, percentile and log compression.

CPU: the oracle and the host-side matrix builder against the golden vectors
the reference's own notebook code produced (tests/golden/make_demod_golden.py),
the Tukey window against SciPy's, and the ABI's argument checks.
GPU: pycbf_gb_demod against the golden IQ (float32 product, rel-L2 <= 1e-5),
the percentile selection exactly against NumPy on the same float32 data, and
the log-compressed image against the golden display values.
"""
import ctypes as ct

import numpy as np
import pytest

from oracle import demod_ref
from pycbf_gb300 import _lib
from pycbf_gb300 import demod as dm

CASES = ("das_band", "noshift", "nyq", "axis0", "frames")


def _params(g, p):
    kmin, kmax, ks, alpha, axis, sh = g[p + "_params"]
    return dict(kmin=kmin, kmax=kmax, ks=ks, alpha=alpha, axis=int(axis), shiftit=bool(sh))


@pytest.fixture(scope="module")
def g(golden):
    return golden("demod.npz")


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_golden(g, case):
    iq = demod_ref.fft_tukey_demod(g[case + "_x"], **_params(g, case))
    ref = g[case + "_iq"]
    assert iq.shape == ref.shape
    assert np.abs(iq - ref).max() <= 1e-12 * np.abs(ref).max()


def test_oracle_zout_and_display_line(g):
    z = demod_ref.zout_fft_tukey_demod(g["das_band_zout"], 2 * 1e6 / 1540.0, 2 * 9e6 / 1540.0)
    assert np.array_equal(z, g["das_band_zout_demod"])
    assert np.array_equal(dm.zout_fft_tukey_demod(g["das_band_zout"], 2 * 1e6 / 1540.0,
                                                  2 * 9e6 / 1540.0), g["das_band_zout_demod"])
    logged = demod_ref.log_compress(np.abs(g["das_band_iq"]))
    assert np.abs(logged - g["das_band_logged"]).max() <= 1e-9


@pytest.mark.parametrize("case", CASES)
def test_demod_matrix_reproduces_golden(g, case):
    p = _params(g, case)
    x = g[case + "_x"].astype(np.float64)
    W = dm.demod_matrix(x.shape[p["axis"]], p["kmin"], p["kmax"], p["ks"], p["alpha"], p["shiftit"])
    iq = np.moveaxis(np.moveaxis(x, p["axis"], -1) @ W, -1, p["axis"])
    ref = g[case + "_iq"]
    assert np.abs(iq - ref).max() <= 1e-12 * np.abs(ref).max()


def test_tukey_window_matches_scipy():
    signal = pytest.importorskip("scipy.signal")
    for M in (1, 2, 3, 7, 92, 205, 1000):
        for a in (0.0, 0.1, 0.25, 0.5, 1.0, 2.0):
            w = signal.windows.tukey(M, alpha=a)
            assert np.abs(dm.tukey(M, a) - w).max() <= 1e-15
            assert np.abs(demod_ref.tukey(M, a) - w).max() <= 1e-15


def test_empty_band_is_rejected():
    with pytest.raises(ValueError):
        dm.demod_matrix(64, 5.0, 1.0, 100.0)


def test_abi_validates_first():
    L = _lib.load()
    p = ct.c_void_p(16)
    assert L.pycbf_gb_demod(None, 4, 8, p, 3, p, None, None) == _lib.EINVAL
    assert L.pycbf_gb_demod(p, 4, 8, p, 3, None, None, None) == _lib.EINVAL
    assert L.pycbf_gb_demod(p, 4, 0, p, 3, p, None, None) == _lib.EINVAL
    assert L.pycbf_gb_demod(p, 4, 8, p, 70000 * 32, p, None, None) == _lib.ERANGE
    assert L.pycbf_gb_percentile_workspace_bytes(0) == 0
    assert L.pycbf_gb_percentile_workspace_bytes(3) == 3 * (4 * 2 * 256 + 32) * 4
    assert L.pycbf_gb_percentile(p, 1, 10, 101.0, p, p, 1 << 20, None) == _lib.EINVAL
    assert L.pycbf_gb_percentile(p, 1, 10, float("nan"), p, p, 1 << 20, None) == _lib.EINVAL
    assert L.pycbf_gb_percentile(p, 1, 0, 50.0, p, p, 1 << 20, None) == _lib.EINVAL
    assert L.pycbf_gb_percentile(p, 1, 1 << 31, 50.0, p, p, 1 << 20, None) == _lib.ERANGE
    assert L.pycbf_gb_percentile(p, 2, 10, 50.0, p, p, 16, None) == _lib.EWORKSPACE
    assert L.pycbf_gb_percentile(p, 0, 10, 50.0, p, None, 0, None) == _lib.OK
    assert L.pycbf_gb_log_compress(p, 1, 10, None, 1e-10, p, None) == _lib.EINVAL
    assert L.pycbf_gb_log_compress(p, 1, 10, p, float("inf"), p, None) == _lib.EINVAL


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_demod_matches_golden(g, case):
    import torch
    p = _params(g, case)
    x = g[case + "_x"]
    iq = dm.fft_tukey_demod(x, **p)                       # NumPy in, NumPy out
    ref = g[case + "_iq"]
    assert iq.dtype == np.complex64 and iq.shape == ref.shape
    assert _rel_l2(iq, ref) <= 1e-5
    xt = torch.as_tensor(x, device="cuda")
    iqt = dm.fft_tukey_demod(xt, **p)                     # CUDA in, CUDA out
    assert iqt.is_cuda and torch.equal(iqt.cpu(), torch.as_tensor(iq))
    d = dm.Demodulator(x.shape[p["axis"]], p["kmin"], p["kmax"], p["ks"], p["alpha"], p["shiftit"])
    env = d.envelope(xt, p["axis"]).cpu().numpy()
    assert np.abs(env - np.abs(iq)).max() <= 2e-6 * np.abs(iq).max()


@pytest.mark.gpu
@pytest.mark.parametrize("n,nseg", [(1, 1), (2, 3), (1000, 1), (4097, 2), (100003, 3),
                                    (300007, 2), (500001, 1)])
def test_gpu_percentile_is_numpys(n, nseg):
    import torch
    rng = np.random.default_rng(n + nseg)
    v = rng.standard_normal(n * nseg).astype(np.float32)
    v[::7] = np.round(v[::7])                  # ties
    if n > 2:
        v[: n // 3] = np.abs(v[: n // 3])
    vt = torch.as_tensor(v, device="cuda")
    for q in (0.0, 1.0, 37.5, 50.0, 99.0, 100.0):
        got = dm.percentile(vt, q, nseg).cpu().numpy()
        want = np.percentile(v.reshape(nseg, n).astype(np.float64), q, axis=1)
        assert np.array_equal(got, want.astype(np.float32)), (q, got, want)


@pytest.mark.gpu
def test_gpu_percentile_nan_and_signed_zero():
    import torch
    v = np.array([3.0, np.nan, 1.0, 2.0], np.float32)
    assert np.isnan(dm.percentile(torch.as_tensor(v, device="cuda"), 50.0).item())
    z = np.array([-0.0, 0.0, -1.0, 1.0, -0.0], np.float32)
    got = dm.percentile(torch.as_tensor(z, device="cuda"), 50.0).item()
    assert got == 0.0


@pytest.mark.gpu
def test_gpu_bmode_matches_display_line(g):
    p = _params(g, "das_band")
    d = dm.Demodulator(g["das_band_x"].shape[-1], p["kmin"], p["kmax"], p["ks"], p["alpha"], p["shiftit"])
    db = d.bmode(g["das_band_x"]).cpu().numpy()
    ref = g["das_band_logged"]
    shown = ref > -60.0                        # the displayed range (examples: -45..5 dB)
    assert np.abs(db - ref)[shown].max() <= 2e-3
    # frames: one percentile per image
    pf = _params(g, "frames")
    x = g["frames_x"]
    d2 = dm.Demodulator(x.shape[-1], pf["kmin"], pf["kmax"], pf["ks"], pf["alpha"], pf["shiftit"])
    db2 = d2.bmode(x, image_ndim=2).cpu().numpy()
    for f in range(x.shape[0]):
        want = demod_ref.log_compress(np.abs(g["frames_iq"][f]))
        m = want > -60.0
        assert np.abs(db2[f] - want)[m].max() <= 2e-3


@pytest.mark.gpu
@pytest.mark.parametrize("n,nseg", [(5000, 3), (8, 5), (70001, 2), (425984, 1), (500001, 2)])
def test_gpu_fused_percentile_and_compression(n, nseg):
    """The one-CTA (small), cluster (up to 8 x 52K values) and multi-CTA
    paths give the percentile of pycbf_gb_percentile and the compression of
    pycbf_gb_log_compress, bit for bit."""
    import torch
    rng = np.random.default_rng(n)
    env = torch.as_tensor(np.abs(rng.standard_normal(n * nseg)).astype(np.float32), device="cuda")
    out, ref = dm.bmode_compress(env, 99.0, 1e-10, nseg)
    assert torch.equal(ref, dm.percentile(env, 99.0, nseg))
    assert torch.equal(out, dm.log_compress(env, ref, 1e-10))
    want = np.percentile(env.cpu().numpy().reshape(nseg, n).astype(np.float64), 99.0, axis=1)
    assert np.array_equal(ref.cpu().numpy(), want.astype(np.float32))

"""The float64 autograd reference of the differentiable delay-and-sum agrees
with the float32 oracle's forward (same spline, same tap decisions) and with
central differences (CPU only)."""
import numpy as np
import pytest
import torch

from oracle import adjoint_ref, oracle


def _bandlimited(rng, shape, frac=0.4):
    """White noise low-passed to frac of the Nyquist band (echo-like spectra)."""
    spec = np.fft.rfft(rng.standard_normal(shape), axis=-1)
    spec[..., int(frac * spec.shape[-1]):] = 0
    return np.fft.irfft(spec, n=shape[-1], axis=-1)


def _case(seed=3, ntx=3, nrx=5, nt=96, np_=400, nf=2, inside=False):
    rng = np.random.default_rng(seed)
    dt, t0 = 1.0 / 25e6, 2e-7
    rf = _bandlimited(rng, (nf, ntx, nrx, nt)).astype(np.float32)
    span = dt * (nt - 1)
    lo = 0.05 if inside else -0.05
    tautx = (t0 + rng.uniform(lo, 0.45, (ntx, np_)) * span).astype(np.float32)
    taurx = rng.uniform(0.0, 0.45, (nrx, np_)).astype(np.float32) * np.float32(span)
    apodtx = rng.uniform(0.5, 1.0, (ntx, np_)).astype(np.float32)
    apodrx = np.where(rng.uniform(size=(nrx, np_)) < 0.8, rng.uniform(0, 1, (nrx, np_)), 0)
    return rf, tautx, taurx, apodtx, apodrx.astype(np.float32), t0, dt


def test_spline_z_matches_the_float32_prefilter():
    rng = np.random.default_rng(0)
    y = rng.standard_normal(200).astype(np.float32)
    dt = 0.04
    y2 = oracle.spline_y2(y, dt)
    z32 = y2.astype(np.float64) * (np.float64(np.float32(dt)) ** 2 / 6.0)
    z64 = adjoint_ref.spline_z(torch.from_numpy(y.astype(np.float64))).numpy()
    assert np.max(np.abs(z64 - z32)) <= 1e-5 * np.max(np.abs(z64))


@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only"])
def test_reference_forward_matches_the_oracle(sumtype):
    rf, tautx, taurx, apodtx, apodrx, t0, dt = _case()
    T = lambda a: torch.from_numpy(a.astype(np.float64))
    ref = adjoint_ref.das_tabbed_ref(T(rf), T(tautx), T(taurx), T(apodtx), T(apodrx), t0, dt,
                                     0.01, sumtype).numpy()
    for f in range(rf.shape[0]):
        orc = oracle.das_tabbed(rf[f], tautx, apodtx, taurx, apodrx, t0, dt, rf.shape[-1],
                                thresh=0.01, sumtype=sumtype).reshape(ref[f].shape)
        assert oracle.rel_l2(orc, ref[f]) <= 1e-5


def test_reference_gradients_match_central_differences():
    rf, tautx, taurx, apodtx, apodrx, t0, dt = _case(seed=5, np_=120, inside=True)
    rng = np.random.default_rng(9)
    w = torch.from_numpy(rng.standard_normal((rf.shape[0], tautx.shape[1])))
    T = lambda a: torch.from_numpy(a.astype(np.float64)).requires_grad_(True)
    rf64, ttx, trx = T(rf), T(tautx), T(taurx)

    def loss(rf_, ttx_, trx_):
        return (w * adjoint_ref.das_tabbed_ref(rf_, ttx_, trx_, torch.from_numpy(apodtx.astype(np.float64)),
                                               torch.from_numpy(apodrx.astype(np.float64)), t0, dt)).sum()

    loss(rf64, ttx, trx).backward()
    v = torch.from_numpy(rng.standard_normal(rf.shape))
    h = 1e-3
    with torch.no_grad():
        fd = (loss(rf64 + h * v, ttx, trx) - loss(rf64 - h * v, ttx, trx)) / (2 * h)
    assert abs(fd - (rf64.grad * v).sum()) <= 1e-9 * max(1.0, abs(fd))
    # delays: a step of 1e-2 of the sample interval (far above the float32
    # rounding of the delays, far below the signal period)
    vt = torch.from_numpy(rng.standard_normal(tautx.shape))
    ht = 1e-2 * dt
    with torch.no_grad():
        fd = (loss(rf64, ttx + ht * vt, trx) - loss(rf64, ttx - ht * vt, trx)) / (2 * ht)
    an = (ttx.grad * vt).sum()
    assert abs(fd - an) <= 1e-2 * abs(an)

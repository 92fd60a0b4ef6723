"""The speed-of-sound objective's torch ops on the CPU: slsc_lag1 against a
direct NumPy evaluation of its definition, float64 gradients against central
differences, and the slowness model's shape and uniform start."""
import numpy as np
import torch

from pycbf_gb300 import sos


def _lag1_numpy(u, m, nkern, eps=1e-20):
    nrx, nx, nz = u.shape
    out = np.zeros((nx, nz))
    for ix in range(nx):
        for iz in range(nz):
            lo, hi = max(0, iz - nkern), min(nz, iz + nkern + 1)
            acc, npair = 0.0, 0
            for e in range(nrx - 1):
                if m[e, ix, iz] and m[e + 1, ix, iz]:
                    a, b = u[e, ix, lo:hi], u[e + 1, ix, lo:hi]
                    acc += (a * b).sum() / np.sqrt((a * a).sum() * (b * b).sum() + eps)
                    npair += 1
            out[ix, iz] = acc / max(npair, 1)
    return out


def test_slsc_lag1_matches_its_definition():
    rng = np.random.default_rng(3)
    nrx, nx, nz = 6, 5, 9
    u = rng.normal(size=(nrx, nx, nz))
    m = rng.random((nrx, nx, nz)) > 0.3
    for nkern in (0, 2):
        got = sos.slsc_lag1(torch.as_tensor(u.reshape(nrx, -1)), torch.as_tensor(m.reshape(nrx, -1)),
                            (nx, nz), nkern).numpy()
        np.testing.assert_allclose(got, _lag1_numpy(u, m, nkern), rtol=1e-12, atol=1e-12)


def test_sos_loss_gradient_float64():
    rng = np.random.default_rng(4)
    nrx, nx, nz = 4, 3, 7
    u = torch.tensor(rng.normal(size=(nrx, nx * nz)), dtype=torch.float64, requires_grad=True)
    m = torch.as_tensor(rng.random((nrx, nx * nz)) > 0.2)
    f = lambda v: sos.sos_loss(v, m, (nx, nz), nkern=1, weight=1e-2)
    assert torch.autograd.gradcheck(f, (u,), eps=1e-6, atol=1e-7)


def test_slowness_model_starts_uniform():
    model = sos.SlownessModel((8, 12), map_shape=(2, 3), c_init=1500.0, device="cpu")
    s = model()
    assert s.shape == (96,)
    assert torch.allclose(s, torch.full((96,), 1 / 1500.0))
    s.sum().backward()
    assert model.c.grad is not None and model.dmap.grad.shape == (2, 3)

"""Constructor validation of the drop-in classes (CPU only): the same checks and
exceptions as the reference's dataclasses, raised before any device work."""
import numpy as np
import pytest
import torch

import pycbf_gb300 as pg
from pycbf_gb300.beamformers import _morton


def tabs(ntx=2, nrx=3, np_=10):
    z = lambda n: np.zeros((n, np_), np.float32)
    return dict(tautx=z(ntx), taurx=z(nrx), apodtx=z(ntx) + 1, apodrx=z(nrx) + 1)


def synth(ntx=2, nrx=3, np_=10, nd=2):
    return dict(ovectx=np.zeros((ntx, nd)), nvectx=np.zeros((ntx, nd)), doftx=np.zeros(ntx),
                alatx=np.zeros(ntx), t0tx=np.zeros(ntx), ovecrx=np.zeros((nrx, nd)),
                nvecrx=np.zeros((nrx, nd)), alarx=np.zeros(nrx), c0=1540.0,
                pnts=np.zeros((np_, nd)))


T = dict(t0=0.0, dt=1e-8, nt=64)


def test_bad_sumtype_and_interp():
    with pytest.raises(pg.BeamformerException):
        pg.TabbedBeamformer(**tabs(), **T, sumtype="both")
    with pytest.raises(pg.BeamformerException):
        pg.TabbedBeamformer(**tabs(), **T, interp={"kind": "spline"})
    with pytest.raises(pg.BeamformerException):
        pg.TabbedBeamformer(**tabs(), **T, interp={"kind": "korder_cubic", "k": 5})
    with pytest.raises(pg.BeamformerException):
        pg.TabbedBeamformer(**tabs(), **T, interp={"kind": "nearest", "usf": 0})


def test_korder_matrix_matches_the_oracle_restatement():
    from oracle import oracle
    from pycbf_gb300 import helpers
    for k in (4, 8, 16, 126):
        np.testing.assert_array_equal(helpers.korder_matrix(k), oracle.korder_S(k))


def test_korder_matrix_matches_reference_golden(golden):
    """The reference's own __make_S_by_k__ (tests/golden/make_korder_golden.py),
    rounded to float32 as its classes round it: equal bit for bit."""
    from oracle import oracle
    from pycbf_gb300 import helpers
    g = golden("korder_S.npz")
    for k in (4, 6, 8, 16, 32):
        np.testing.assert_array_equal(helpers.korder_matrix(k), g[f"S{k}"])
        np.testing.assert_array_equal(oracle.korder_S(k), g[f"S{k}"])


def test_poly_kind_limits():
    with pytest.raises(pg.BeamformerException):
        pg.TabbedBeamformer(**tabs(), **T, interp={"kind": "korder_cubic", "k": 130})
    with pytest.raises(pg.BeamformerException):
        pg.TabbedBeamformer(**tabs(), t0=0.0, dt=1e-8, nt=4, interp={"kind": "akima"})


def test_tabbed_shape_checks():
    t = tabs()
    t["apodtx"] = np.zeros((3, 10), np.float32)
    with pytest.raises(pg.BeamformerException, match="dim 0"):
        pg.TabbedBeamformer(**t, **T)
    t = tabs()
    t["apodrx"] = np.zeros((3, 9), np.float32)       # the reference checks apodtx twice here
    with pytest.raises(pg.BeamformerException, match="dim 1"):
        pg.TabbedBeamformer(**t, **T)
    t = tabs()
    t["tautx"] = np.zeros(10, np.float32)
    with pytest.raises(pg.BeamformerException, match="2D"):
        pg.TabbedBeamformer(**t, **T)


def test_synthetic_shape_checks():
    s = synth()
    s["alarx"] = np.zeros(4)
    with pytest.raises(pg.BeamformerException, match="rx"):
        pg.SyntheticBeamformer(**s, **T)
    s = synth()
    s["nvecrx"] = np.zeros((3, 3))
    with pytest.raises(pg.BeamformerException, match="dimensions"):
        pg.SyntheticBeamformer(**s, **T)
    s = synth()
    s["doftx"] = np.zeros((2, 1))
    with pytest.raises(pg.BeamformerException, match="1D"):
        pg.SyntheticBeamformer(**s, **T)


def test_dmas_settings():
    with pytest.raises(pg.BeamformerException, match="lagaxis"):
        pg.TabbedDMASBeamformer(**tabs(), **T, lags=[1], lagaxis="z")
    with pytest.raises(pg.BeamformerException, match="dmastype"):
        pg.TabbedDMASBeamformer(**tabs(), **T, lags=[1], dmastype="abs")


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU error path")
def test_valid_construction_needs_cuda():
    with pytest.raises(pg.BeamformerException, match="CUDA"):
        pg.TabbedBeamformer(**tabs(), **T)


def test_morton_keeps_neighbours_close():
    x, z = np.meshgrid(np.arange(64), np.arange(64), indexing="ij")
    pts = torch.tensor(np.stack([x.ravel(), z.ravel()], 1), dtype=torch.float64)
    order = torch.argsort(_morton(pts)).numpy()
    blocks = pts.numpy()[order].reshape(-1, 32, 2)
    spans = blocks.max(1) - blocks.min(1)
    assert np.all(spans <= 8)       # 32 consecutive keys form an 8x4 or 4x8 block


def test_batch_branch_assignment():
    """Graph branches of the batch's frame-launch form: largest group first onto
    the least loaded branch."""
    from pycbf_gb300.batch import assign_branches
    assert assign_branches([5, 3, 3, 2, 1], 2) == [0, 1, 1, 0, 1]  # loads 7, 7
    assert assign_branches([1, 1, 1], 4) == [0, 1, 2]
    costs = [9, 7, 6, 5, 4, 3, 2, 1]
    b = assign_branches(costs, 3)
    loads = [sum(c for c, x in zip(costs, b) if x == k) for k in range(3)]
    assert max(loads) - min(loads) <= max(costs) and sum(loads) == sum(costs)
    assert assign_branches([], 3) == []

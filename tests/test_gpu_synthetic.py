"""GPU parity of the Synthetic path, DMAS and SLSC against the oracle.

The oracle builds float32 delay/mask tables from the same restated geometry
formulas and runs the reference's interpolation and sum on them, so the tap
set must match bit-exactly and the images to float32 accuracy."""
import os

import numpy as np
import pytest
import torch

import pycbf_gb300 as pg
from gpu_util import assert_image_close, report
from oracle import oracle
from pycbf_gb300 import _lib, helpers, phantom

pytestmark = pytest.mark.gpu
NCPU = max(1, len(os.sched_getaffinity(0)))
GEO_KEYS = ("ovectx", "nvectx", "doftx", "alatx", "t0tx", "ovecrx", "nvecrx", "alarx", "c0", "pnts")


@pytest.fixture(scope="module")
def synthetic_small():
    w = phantom.linear_pw_synthetic(nele=48, nsteer=9, nt=1536, nx=48, nz=96, n_speckle=2000,
                                    xlim=(-4.8e-3, 4.8e-3), zlim=(5e-3, 20e-3), device="cuda")
    return w


def synth_bf(w, cls=pg.SyntheticBeamformer, geo=None, **kw):
    g = geo or w.geometry
    return cls(**{k: g[k] for k in GEO_KEYS}, t0=w.t0, dt=w.dt, nt=w.nt, **kw)


def oracle_tables(w, geo=None):
    g = geo or w.geometry
    return oracle.synth_tables(g["ovectx"], g["nvectx"], g["doftx"], g["alatx"], g["t0tx"],
                               g["ovecrx"], g["nvecrx"], g["alarx"], g["c0"], g["pnts"])


def oracle_image(w, tables, kind="cubic", sumtype="tx_and_rx", rf=None):
    tt, at, tr, ar = tables
    return oracle.das_tabbed(w.rf if rf is None else rf, tt, at, tr, ar, w.t0, w.dt, w.nt,
                             interp=kind, sumtype=sumtype, thresh=0.01, threads=NCPU)


@pytest.mark.parametrize("kind", ["cubic", "nearest", "linear"])
def test_synthetic_das_vs_oracle(synthetic_small, kind):
    w = synthetic_small
    tables = oracle_tables(w)
    bf = synth_bf(w, interp={"kind": kind})
    out = bf(w.rf)
    r, m = assert_image_close(out, oracle_image(w, tables, kind), what=kind)
    report(f"synthetic_small_{kind}", rel_l2=r, max_abs_peak=m)
    cnt, isum = bf.tap_census()
    ok_cnt, ok_isum = oracle.tap_census(*tables, w.t0, w.dt, w.nt,
                                        interp="nearest" if kind == "nearest" else "cubic",
                                        thresh=0.01)
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


def test_synthetic_nearest_upsampled_vs_oracle(synthetic_small):
    w = synthetic_small
    tables = oracle_tables(w)
    bf = synth_bf(w, interp={"kind": "nearest", "usf": 3})
    out = bf(w.rf)
    tt, at, tr, ar = tables
    ref = oracle.das_tabbed(w.rf, tt, at, tr, ar, w.t0, w.dt, w.nt, interp="nearest", usf=3,
                            thresh=0.01, threads=NCPU)
    r, m = assert_image_close(out, ref, what="usf 3")
    report("synthetic_small_nearest_usf3", rel_l2=r, max_abs_peak=m)
    cnt, isum = bf.tap_census()
    ok_cnt, ok_isum = oracle.tap_census(*tables, w.t0, w.dt, w.nt, interp="nearest", usf=3,
                                        thresh=0.01)
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


@pytest.mark.parametrize("interp", [dict(kind="korder_cubic", k=8), dict(kind="makima")])
def test_synthetic_gpu_only_interpolators_vs_oracle(synthetic_small, interp):
    w = synthetic_small
    tt, at, tr, ar = oracle_tables(w)
    out = synth_bf(w, interp=interp)(w.rf)
    ref = oracle.das_poly(w.rf, tt, at, tr, ar, w.t0, w.dt, w.nt, interp["kind"],
                          k=interp.get("k", 8), thresh=0.01)
    r, m = assert_image_close(out, ref, what=str(interp))
    report(f"synthetic_small_{interp['kind']}", rel_l2=r, max_abs_peak=m)


@pytest.mark.parametrize("sumtype", ["tx_only", "rx_only", "none"])
def test_synthetic_sumtypes(synthetic_small, sumtype):
    w = synthetic_small
    out = synth_bf(w, sumtype=sumtype)(w.rf)
    assert_image_close(out, oracle_image(w, oracle_tables(w), "cubic", sumtype), what=sumtype)


def test_synthetic_receive_mask(synthetic_small):
    w = synthetic_small
    _, _, _, ar = oracle_tables(w)
    m = synth_bf(w).rx_mask().cpu().numpy()
    np.testing.assert_array_equal(m, (ar != 0).astype(np.uint8))


def _focused_geometry(ndim=2, dof=0.0, behind=False):
    rng = np.random.default_rng(9)
    nele = 40
    xele = helpers.element_positions(nele, 0.25e-3)
    ntx = 7
    steer = np.radians(np.linspace(-12, 12, ntx))
    r = -8e-3 if behind else 12e-3
    ovectx = np.stack([r * np.sin(steer), r * np.cos(steer)], 1)
    nvectx = np.stack([np.sin(steer), np.cos(steer)], 1)
    alatx = np.full(ntx, 0.3)
    t0tx = np.abs(r) / 1540 * (1 if not behind else -1) + rng.uniform(0, 1e-7, ntx)
    ovecrx = np.stack([xele, np.zeros(nele)], 1)
    nvecrx = np.stack([np.zeros(nele), np.ones(nele)], 1)
    alarx = np.full(nele, np.arctan2(0.5, 1.2))
    xs, zs = np.linspace(-5e-3, 5e-3, 40), np.linspace(2e-3, 22e-3, 64)
    pnts = helpers.pixel_grid(xs, zs)
    if ndim == 3:
        ovectx = np.insert(ovectx, 1, 0.0, axis=1)
        nvectx = np.insert(nvectx, 1, 0.0, axis=1)
        ovecrx = np.insert(ovecrx, 1, rng.uniform(-1e-3, 1e-3, nele), axis=1)
        nvecrx = np.insert(nvecrx, 1, 0.0, axis=1)
        pnts = np.insert(pnts, 1, rng.uniform(-1e-3, 1e-3, len(pnts)), axis=1)
    return dict(ovectx=ovectx, nvectx=nvectx, doftx=np.full(ntx, dof), alatx=alatx, t0tx=t0tx,
                ovecrx=ovecrx, nvecrx=nvecrx, alarx=alarx, c0=1540.0, pnts=pnts)


@pytest.mark.parametrize("ndim,dof,behind", [(2, 0.0, False), (2, 4e-3, False), (2, 0.0, True),
                                             (3, 0.0, False), (3, 6e-3, False)])
def test_synthetic_delay_branches(ndim, dof, behind):
    geo = _focused_geometry(ndim, dof, behind)
    nt = 1200
    rng = np.random.default_rng(3)

    class W:  # a minimal workload record
        pass
    w = W()
    w.t0, w.dt, w.nt = 1e-7, 1 / 30e6, nt
    ntx, nrx = geo["ovectx"].shape[0], geo["ovecrx"].shape[0]
    w.rf = rng.normal(size=(ntx, nrx, nt)).astype(np.float32)
    tables = oracle_tables(w, geo)
    assert np.count_nonzero(tables[1]) > 0 and np.count_nonzero(tables[1] == 0) > 0
    bf = synth_bf(w, geo=geo)
    assert_image_close(bf(w.rf), oracle_image(w, tables), what=f"{ndim}d dof={dof}")
    cnt, isum = bf.tap_census()
    ok_cnt, ok_isum = oracle.tap_census(*tables, w.t0, w.dt, w.nt, thresh=0.01)
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


@pytest.fixture(scope="module")
def synthetic_wide():
    """21 plane waves (> 12: the shared-memory column form) over a field
    wider than the aperture, so that most warps of pixels see only part of
    the transmits, some none, and the last warp is partial (37 x 45
    pixels)."""
    return phantom.linear_pw_synthetic(nele=32, nsteer=21, nt=1024, nx=37, nz=45, n_speckle=800,
                                       xlim=(-14e-3, 14e-3), zlim=(4e-3, 24e-3), device="cuda")


@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only"])
def test_synthetic_column_form_masked_field(synthetic_wide, sumtype):
    """The column form on transmit masks that differ between and within
    warps: images against the oracle, and (tx_and_rx) bit for bit the image
    of the batched queue kernel, which runs the same pixel body."""
    from pycbf_gb300.batch import BatchBeamformer, BatchConfig
    w = synthetic_wide
    tables = oracle_tables(w)
    live = (tables[1] != 0).reshape(21, -1)  # transmit masks, pixels in table order
    nwarp = -(-live.shape[1] // 32)
    pad = np.zeros((21, nwarp * 32 - live.shape[1]), bool)
    anyl = np.concatenate([live, pad], 1).reshape(21, nwarp, 32).any(-1)
    runs = anyl.sum(0)
    assert (runs < 21).sum() >= nwarp // 4 and (runs == 0).any() and (runs == 21).any()
    bf = synth_bf(w, interp={"kind": "cubic"}, sumtype=sumtype)
    out = bf(w.rf, out_as_numpy=False)
    ref = oracle_image(w, tables, "cubic", sumtype)
    r, m = assert_image_close(out.cpu().numpy(), ref, what=sumtype)
    report(f"synthetic_wide_column_{sumtype}", rel_l2=r, max_abs_peak=m)
    if sumtype == "tx_and_rx":
        rf = torch.as_tensor(w.rf, device="cuda")
        (b,) = BatchBeamformer([bf], config=BatchConfig(1, 1, 0, 4))([rf])
        assert torch.equal(b, bf(rf, out_as_numpy=False))


@pytest.mark.parametrize("dmastype", ["ssr", "power"])
def test_fused_dmas_all_pairs(synthetic_small, dmastype):
    w = synthetic_small
    nrx = w.geometry["ovecrx"].shape[0]
    bf = synth_bf(w, cls=pg.SyntheticDMASBeamformer, lags=np.arange(1, nrx), dmastype=dmastype)
    assert bf._fused
    out = bf(w.rf)
    sep = oracle_image(w, oracle_tables(w), "cubic", "tx_only").reshape(nrx, -1)
    ref = oracle.dmas(sep, np.arange(1, nrx), power=(dmastype == "power"))
    r, m = assert_image_close(out, ref, rel=1e-4, peak=1e-4, what=dmastype)
    report(f"synthetic_small_dmas_{dmastype}", rel_l2=r, max_abs_peak=m)


def test_dmas_lag_list_unfused(synthetic_small):
    w = synthetic_small
    nrx = w.geometry["ovecrx"].shape[0]
    lags = np.array([1, 2, 5])
    bf = synth_bf(w, cls=pg.SyntheticDMASBeamformer, lags=lags, sumlags=False)
    assert not bf._fused
    out = bf(w.rf)
    sep = oracle_image(w, oracle_tables(w), "cubic", "tx_only").reshape(nrx, -1)
    ref = oracle.dmas(sep, lags, sumlags=False)
    assert out.shape == (3, bf.nop)
    assert_image_close(out, ref, rel=1e-4, peak=1e-4, what="lag list")


def test_slsc_vs_oracle(synthetic_small):
    w = synthetic_small
    nx, nz = w.grid
    tables = oracle_tables(w)
    nrx = tables[2].shape[0]
    bf = synth_bf(w, cls=pg.SyntheticSLSCBeamformer, grid_shape=(nx, nz), nlag=8, nkern=2)
    out = bf(w.rf)
    sep = oracle_image(w, tables, "cubic", "tx_only").reshape(nrx, nx, nz)
    ref = oracle.slsc(sep, (tables[3] != 0).reshape(nrx, nx, nz), 8, 2)
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    ok = ~np.isnan(ref)
    err = np.max(np.abs(out[ok] - ref[ok]))
    report("synthetic_small_slsc", max_abs=err)
    assert err < 2e-4


@pytest.mark.parametrize("nlag,nkern", [(16, 3), (20, 2), (6, 5)])
def test_slsc_both_kernels_vs_oracle(synthetic_small, nlag, nkern):
    """nlag <= 16 with nkern <= 3 runs the register-blocked kernel, larger
    values the shared-memory ring kernel: both against the oracle, on a mask
    with holes (every fifth element off in part of the image) so that the
    kept elements are not contiguous."""
    w = synthetic_small
    nx, nz = w.grid
    tables = oracle_tables(w)
    nrx = tables[2].shape[0]
    sep = oracle_image(w, tables, "cubic", "tx_only").reshape(nrx, nx, nz)
    mask = (tables[3] != 0).reshape(nrx, nx, nz).copy()
    mask[::5, : nx // 2, :] = False
    L = _lib.load()
    im = torch.as_tensor(sep, device="cuda")
    m = torch.as_tensor(mask.astype(np.uint8), device="cuda")
    out = torch.empty((nx, nz), device="cuda")
    assert L.pycbf_gb_slsc(im.data_ptr(), m.data_ptr(), 1, nrx, nx, nz, nlag, nkern,
                           out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    out = out.cpu().numpy()
    ref = oracle.slsc(sep, mask, nlag, nkern)
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.max(np.abs(out[ok] - ref[ok])) < 2e-4


@pytest.mark.parametrize("nrx,nlag,nkern,nframes", [(40, 16, 3, 2), (256, 5, 0, 1),
                                                    (33, 1, 2, 1), (192, 16, 1, 3)])
def test_slsc_kept_sets_equal_the_mask_path(nrx, nlag, nkern, nframes):
    """The coherence from kept-element sets computed once per mask equals the
    mask-byte path bit for bit (NaNs included), on ragged masks: random holes,
    whole elements off, a grid whose z extent is not a multiple of the kernel."""
    nx, nz = 9, 37
    rng = np.random.default_rng(nrx + 7 * nkern)
    im = rng.normal(size=(nframes, nrx, nx, nz)).astype(np.float32)
    im[:, 3, 2, :] = 0.0  # a flat kernel: deviation below 1e-10
    mask = (rng.random((nrx, nx, nz)) > 0.15).astype(np.uint8)
    mask[::7] = 0
    mask[:, 4, :] = 1
    L = _lib.load()
    dim = torch.as_tensor(im, device="cuda")
    dm = torch.as_tensor(mask, device="cuda")
    nbytes = L.pycbf_gb_slsc_kept_bytes(nrx, nx, nz)
    assert nbytes == 4 * ((nrx + 31) // 32) * nx * nz
    kept = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    assert L.pycbf_gb_slsc_kept(dm.data_ptr(), nrx, nx, nz, nlag, nkern, kept.data_ptr(),
                                nbytes - 1, None) == _lib.ERANGE
    assert L.pycbf_gb_slsc_kept(dm.data_ptr(), nrx, nx, nz, nlag, nkern, kept.data_ptr(),
                                nbytes, None) == _lib.OK
    a = torch.full((nframes, nx, nz), 7.0, device="cuda")
    b = torch.full((nframes, nx, nz), 9.0, device="cuda")
    assert L.pycbf_gb_slsc(dim.data_ptr(), dm.data_ptr(), nframes, nrx, nx, nz, nlag, nkern,
                           a.data_ptr(), None) == _lib.OK
    assert L.pycbf_gb_slsc_with_kept(dim.data_ptr(), kept.data_ptr(), nframes, nrx, nx, nz, nlag,
                                     nkern, b.data_ptr(), None) == _lib.OK
    torch.cuda.synchronize()
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    ref = oracle.slsc(im[0], mask.astype(bool), nlag, nkern)
    assert np.array_equal(np.isnan(b[0]), np.isnan(ref))
    ok = ~np.isnan(ref)
    if nkern == 0:  # one-sample kernels have no deviation: every lag is NaN
        assert not ok[ref != 0].any()
    else:
        assert ok.any() and np.max(np.abs(b[0][ok] - ref[ok])) < 2e-4


def test_slsc_kernel_vs_notebook_golden(golden):
    g = golden("coherence_small.npz")
    L = _lib.load()
    im = torch.as_tensor(g["im"], device="cuda")
    mask = torch.as_tensor(g["mask"], device="cuda")
    nrx, nx, nz = g["im"].shape
    out = torch.empty((nx, nz), device="cuda")
    st = L.pycbf_gb_slsc(im.data_ptr(), mask.data_ptr(), 1, nrx, nx, nz, int(g["nlag"]),
                         int(g["nkern"]), out.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    out = out.cpu().numpy()
    ref = g["ref_slsc"]
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    ok = ~np.isnan(ref)
    np.testing.assert_allclose(out[ok], ref[ok], atol=1e-5)


def test_dmas_kernel_vs_notebook_golden(golden):
    g = golden("coherence_small.npz")
    L = _lib.load()
    nrx, nx, nz = g["im"].shape
    im = torch.as_tensor(g["im"].reshape(nrx, nx * nz), device="cuda")
    lags = torch.arange(1, int(g["dmas_nlag"]) + 1, dtype=torch.int32, device="cuda")
    out = torch.empty(nx * nz, device="cuda")
    st = L.pycbf_gb_dmas(im.data_ptr(), 1, nrx, nx * nz, lags.data_ptr(), lags.numel(), 0, 1,
                         out.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(out.cpu().numpy().reshape(nx, nz), g["ref_dmas"], rtol=1e-5,
                               atol=1e-4)


def test_tabbed_slsc_and_dmas_classes(golden):
    case = golden("tabbed_pw_small.npz")
    kw = dict(tautx=case["tautx"], taurx=case["taurx"], apodtx=case["apodtx"], apodrx=case["apodrx"],
              t0=float(case["t0"]), dt=float(case["dt"]), nt=int(case["nt"]))
    nrx = case["taurx"].shape[0]
    sep = oracle.das_tabbed(case["rf"], case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
                            kw["t0"], kw["dt"], kw["nt"], sumtype="tx_only").reshape(nrx, -1)
    out = pg.TabbedDMASBeamformer(**kw, lags=np.arange(1, nrx))(case["rf"])
    assert_image_close(out, oracle.dmas(sep, np.arange(1, nrx)), rel=1e-4, peak=1e-4)
    nx, nz = 24, 32
    slsc = pg.TabbedSLSCBeamformer(**kw, grid_shape=(nx, nz), nlag=4, nkern=2)(case["rf"])
    ref = oracle.slsc(sep.reshape(nrx, nx, nz), (np.abs(case["apodrx"]) >= np.float32(0.01)).reshape(
        nrx, nx, nz), 4, 2)
    ok = ~np.isnan(ref)
    assert np.array_equal(np.isnan(slsc), np.isnan(ref))
    assert np.max(np.abs(slsc[ok] - ref[ok])) < 2e-4

"""The oracle against the reference's own CUDA kernels (pycbf/gpu/__engines__.cu,
__advanced_engines__.cu) compiled for the CPU from where they lie
(oracle/refgpu_driver.cpp; CPU only,
skipped where the reference checkout was not built into oracle/_ref).

The host build rounds every operation alone, so the oracle's interpolators
run with fused=False here (the device contracts a few multiply-adds; the
oracle's default mode fuses those).  The reference's tap rule is
|apodtx*apodrx| > 0.01 against a double 0.01, which for float32 weights is
>= the float after 0.01f.
"""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.skipif(oracle.refgpu_lib() is None,
                                reason="the reference's kernels are not built here")

GPU_RULE = float(np.nextafter(np.float32(0.01), np.float32(1)))
POLY = [("korder_cubic", 4), ("korder_cubic", 8), ("korder_cubic", 16), ("akima", 0),
        ("makima", 0)]


def _tabbed_args(case):
    return (case["rf"], case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
            float(case["t0"]), float(case["dt"]), int(case["nt"]))


@pytest.mark.parametrize("name", ["pw_small", "edge"])
@pytest.mark.parametrize("interp,k", POLY)
def test_tabbed_poly_kinds_equal_reference_kernels(golden, name, interp, k):
    args = _tabbed_args(golden(f"tabbed_{name}.npz"))
    for sumtype in ("tx_and_rx", "none"):
        ref = oracle.das_tabbed_refgpu(*args, interp=interp, k=k, sumtype=sumtype)
        orc = oracle.das_poly(*args, interp=interp, k=k, thresh=GPU_RULE, sumtype=sumtype,
                              fused=False)
        np.testing.assert_array_equal(orc, ref)


@pytest.mark.parametrize("name", ["pw_small", "edge", "short2", "short3"])
def test_tabbed_nearest_and_linear_equal_reference_kernels(golden, name):
    """The reference's CUDA nearest (round half up) and linear (which returns
    the floor sample: the oracle's linear_floor)."""
    args = _tabbed_args(golden(f"tabbed_{name}.npz"))
    for ref_kind, orc_kind in (("nearest", "nearest"), ("linear", "linear_floor")):
        for sumtype in ("tx_and_rx", "none"):
            ref = oracle.das_tabbed_refgpu(*args, interp=ref_kind, sumtype=sumtype)
            orc = oracle.das_tabbed(*args, interp=orc_kind, thresh=GPU_RULE, sumtype=sumtype)
            np.testing.assert_array_equal(orc, ref)


def _focused_2d():
    """Focused transmits with a depth of field (the reference's hourglass and
    planar branches, __engines__.cu:409-423) and an F-number receive."""
    rng = np.random.default_rng(5)
    nele, ntx, nt = 32, 5, 512
    xele = (np.arange(nele) - (nele - 1) / 2) * 0.3e-3
    xf = np.linspace(-3e-3, 3e-3, ntx)
    xs, zs = np.meshgrid(np.linspace(-5e-3, 5e-3, 40), np.linspace(5e-3, 25e-3, 60), indexing="ij")
    f32 = lambda a: np.asarray(a, np.float32)
    geo = dict(ovectx=f32(np.stack([xf, np.full(ntx, 15e-3)], 1)),
               nvectx=f32(np.tile([0.0, 1.0], (ntx, 1))), doftx=f32(np.full(ntx, 6e-3)),
               alatx=f32(np.full(ntx, 0.3)), t0tx=f32(np.full(ntx, 15e-3 / 1540.0)),
               ovecrx=f32(np.stack([xele, np.zeros(nele)], 1)),
               nvecrx=f32(np.tile([0.0, 1.0], (nele, 1))), alarx=f32(np.full(nele, 0.4)),
               c0=np.float32(1540.0), pnts=f32(np.stack([xs.ravel(), zs.ravel()], 1)))
    rf = rng.normal(size=(ntx, nele, nt)).astype(np.float32)
    return geo, rf, np.float32(0.0), np.float32(1 / 20e6), nt


def _diverging_3d():
    from pycbf_gb300 import phantom
    w = phantom.matrix_dw_synthetic(nside=8, nvs=2, nt=1024, nvox=(12, 12, 24), n_speckle=300,
                                    lims=((-2e-3, 2e-3), (-2e-3, 2e-3), (5e-3, 15e-3)),
                                    device="cpu")
    return w.geometry, w.rf, w.t0, w.dt, w.nt


def _oracle_synthetic(geo, rf, t0, dt, nt, interp, sumtype):
    keys = ("ovectx", "nvectx", "doftx", "alatx", "t0tx", "ovecrx", "nvecrx", "alarx", "c0",
            "pnts")
    tabs = oracle.synth_tables(*(geo[k] for k in keys))
    if interp in ("nearest", "linear"):
        kind = "nearest" if interp == "nearest" else "linear_floor"
        return oracle.das_tabbed(rf, *tabs, t0, dt, nt, interp=kind, thresh=0.01, sumtype=sumtype)
    # the reference's Synthetic korder kernel receives k as 0 (an int32 in a float parameter)
    return oracle.das_poly(rf, *tabs, t0, dt, nt, interp=interp, k=0, thresh=0.01,
                           sumtype=sumtype, fused=False)


@pytest.mark.parametrize("geometry", ["focused_2d", "diverging_3d"])
@pytest.mark.parametrize("interp", ["nearest", "linear", "akima", "makima", "korder_cubic"])
def test_synthetic_equals_reference_kernels(geometry, interp):
    """Delays and masks computed per tap (calc_tautx_apodtx / calc_taurx_apodrx)
    in geometries whose acceptance angles are far from the float resolution of
    the cosine: every per-channel output equal."""
    geo, rf, t0, dt, nt = _focused_2d() if geometry == "focused_2d" else _diverging_3d()
    ref = oracle.das_synthetic_refgpu(rf, geo, t0, dt, nt, interp, k=8, sumtype="none")
    np.testing.assert_array_equal(_oracle_synthetic(geo, rf, t0, dt, nt, interp, "none"), ref)


@pytest.mark.parametrize("power", [False, True])
@pytest.mark.parametrize("sumlags", [True, False])
def test_dmas_equals_reference_kernel(golden, power, sumlags):
    """calc_dmas (pycbf/gpu/__advanced_engines__.cu:17-61) over every (lag,
    image, pixel): the oracle with the lags at the kernel's positions
    0..nlag-1 agrees within float summation (the kernel adds in float in
    thread order, the oracle in double)."""
    g = golden("coherence_small.npz")
    nrx, nx, nz = g["im"].shape
    im = g["im"].reshape(nrx, nx * nz)
    nlag = int(g["dmas_nlag"]) + 1
    ref = oracle.dmas_refgpu(im, nlag, power=power, sumlags=sumlags).reshape(-1)
    orc = oracle.dmas(im, np.arange(nlag), power=power, sumlags=sumlags).reshape(-1)
    assert oracle.rel_l2(orc, ref) <= 1e-6
    assert np.abs(orc - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["pw_small", "edge"])
@pytest.mark.parametrize("interp,k", POLY)
def test_device_contraction_stays_within_the_parity_bar(golden, name, interp, k):
    """The kernels are checked against the oracle with the multiply-adds the
    device contracts fused; the reference's host build rounds them alone.
    The two oracle modes differ by cancellation in x - x0 - dx*n (korder) at
    most ~3e-6, inside the 1e-5 image bar, and take the same taps."""
    args = _tabbed_args(golden(f"tabbed_{name}.npz"))
    fused = oracle.das_poly(*args, interp=interp, k=k, fused=True)
    plain = oracle.das_poly(*args, interp=interp, k=k, fused=False)
    assert oracle.rel_l2(fused, plain) <= 1e-5
    np.testing.assert_array_equal(fused != 0, plain != 0)


SYNTH_KEYS = ("ovectx", "nvectx", "doftx", "alatx", "t0tx", "ovecrx", "nvecrx", "alarx", "c0",
              "pnts")


def _mask_flips(w):
    """Taps whose inclusion differs between the reference's kernels built with and
    without contracted multiply-adds, and between the oracle's cosine compare and
    the uncontracted build; the image differences beside them."""
    g = w.geometry
    run = lambda contracted: oracle.das_synthetic_refgpu(w.rf, g, w.t0, w.dt, w.nt, "linear",
                                                         sumtype="none", contracted=contracted)
    plain, fused = run(False), run(True)
    tabs = oracle.synth_tables(*(g[k] for k in SYNTH_KEYS))
    orc = oracle.das_tabbed(w.rf, *tabs, w.t0, w.dt, w.nt, interp="linear_floor", thresh=0.01,
                            sumtype="none")
    ntx, nrx = np.shape(g["ovectx"])[0], np.shape(g["ovecrx"])[0]
    img = lambda a: a.reshape(ntx, nrx, -1).sum((0, 1))
    flips = lambda a, b: int(((a != 0) != (b != 0)).sum())
    return (flips(plain, fused), oracle.rel_l2(img(fused), img(plain)), flips(plain, orc),
            oracle.rel_l2(img(orc), img(plain)), plain.size)


@pytest.mark.skipif(oracle.build_refgpu(contracted=True) is None,
                    reason="the contracted build of the reference's kernels is not available")
def test_far_virtual_source_masks_depend_on_rounding():
    """Plane waves modelled as virtual sources 10 m behind the array (the
    192-element Synthetic workload's geometry, here 48 elements and 9 transmits)
    have acceptance angles of ~4.5e-4 rad: |proj/mag| sits within a few float
    steps of 1, and the reference's own decision acos(|proj/mag|) > ala
    (pycbf/gpu/__engines__.cu:412,427) flips with how multiply-adds are
    contracted.  In 3-D diverging waves nothing flips."""
    from pycbf_gb300 import phantom
    w = phantom.linear_pw_synthetic(nele=48, nsteer=9, nt=1536, nx=48, nz=96, n_speckle=2000,
                                    xlim=(-4.8e-3, 4.8e-3), zlim=(5e-3, 20e-3), device="cpu")
    f_ref, r_ref, f_orc, r_orc, n = _mask_flips(w)
    print(f"far virtual sources: reference contracted vs not {f_ref}/{n} taps, rel-L2 {r_ref:.3g}; "
          f"oracle vs reference {f_orc} taps, rel-L2 {r_orc:.3g}")
    assert f_ref > 0.05 * n and r_ref > 0.1  # the reference disagrees with itself
    w = phantom.matrix_dw_synthetic(nside=8, nvs=2, nt=1024, nvox=(12, 12, 24), n_speckle=300,
                                    lims=((-2e-3, 2e-3), (-2e-3, 2e-3), (5e-3, 15e-3)),
                                    device="cpu")
    f_ref, r_ref, f_orc, r_orc, n = _mask_flips(w)
    assert f_ref == 0 and f_orc == 0

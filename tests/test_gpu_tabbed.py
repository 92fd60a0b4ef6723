"""GPU parity of the Tabbed path against the pinned oracle and the reference's
golden outputs.  The tap set (in-range and apodization decisions, and each
tap's sample index) must match bit-exactly; images within rel-L2 1e-5 and
max-abs 1e-4 of the peak; the float64 error is checked and reported."""
import os

import numpy as np
import pytest
import torch

import pycbf_gb300 as pg
from gpu_util import assert_image_close, report
from oracle import oracle
from pycbf_gb300 import phantom

pytestmark = pytest.mark.gpu
CASES = ["pw_small", "edge", "short2", "short3"]
NCPU = max(1, len(os.sched_getaffinity(0)))


def bf_for(case, kind="cubic", sumtype="tx_and_rx", **kw):
    interp = dict(kind=kind) if isinstance(kind, str) else kind
    return pg.TabbedBeamformer(tautx=case["tautx"], taurx=case["taurx"], apodtx=case["apodtx"],
                               apodrx=case["apodrx"], t0=float(case["t0"]), dt=float(case["dt"]),
                               nt=int(case["nt"]), interp=interp, sumtype=sumtype, **kw)


def oracle_for(case, kind="cubic", sumtype="tx_and_rx", threads=1):
    return oracle.das_tabbed(case["rf"], case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
                             float(case["t0"]), float(case["dt"]), int(case["nt"]), interp=kind,
                             sumtype=sumtype, threads=threads)


@pytest.fixture(scope="module")
def tabbed_small():
    w = phantom.linear_pw_tabbed(nx=64, nz=128, n_speckle=1500, device="cuda")
    return dict(rf=w.rf, tautx=w.tautx, apodtx=w.apodtx, taurx=w.taurx, apodrx=w.apodrx,
                t0=w.t0, dt=w.dt, nt=w.nt)


def test_block_items_deterministic_and_frame_consistent(tabbed_small):
    """Single-frame staged launches split tiles into receive-block items whose
    sums the last block adds in order: repeated calls give the same bits, and
    so does the frame-per-tile path of a multi-frame call."""
    bf = bf_for(tabbed_small, "cubic")
    a, b = bf(tabbed_small["rf"]), bf(tabbed_small["rf"])
    np.testing.assert_array_equal(a, b)
    frames = np.stack([tabbed_small["rf"], tabbed_small["rf"][::-1].copy()])
    np.testing.assert_array_equal(bf(frames)[0], a)
    assert bf.kernel_status() == 0


def test_staged_decisions_near_boundaries():
    """The fast quotients and their boundary tolerance (staged kernel; generic
    kernel for cubic sums), on delays within a few ulp of every knot and
    half-knot: staged against generic bit for bit, and both against the
    oracle's exact decisions (random channel data, so a tap at the wrong
    sample changes the image)."""
    rng = np.random.default_rng(43)
    nt, dt, t0 = 512, np.float32(1 / 31.25e6), np.float32(1.3e-6)
    npx = 8192
    k = rng.integers(-3, nt + 3, size=npx).astype(np.float32)
    frac = rng.choice(np.array([0.0, 0.5], np.float32), size=npx)
    tau = (t0 + dt * (k + frac)).astype(np.float32)
    ulps = rng.integers(-6, 7, size=npx)
    for i in range(npx):
        for _ in range(abs(int(ulps[i]))):
            tau[i] = np.nextafter(tau[i], np.float32(np.inf if ulps[i] > 0 else -np.inf))
    nrx = 3
    case = dict(tautx=tau[None, :].copy(), taurx=np.zeros((nrx, npx), np.float32),
                apodtx=np.ones((1, npx), np.float32),
                apodrx=rng.choice(np.array([1, 0.5, -0.25], np.float32), size=(nrx, npx)),
                t0=t0, dt=dt, nt=nt)
    rf = rng.normal(size=(1, nrx, nt)).astype(np.float32)
    for kind in ("cubic", "linear", "nearest"):
        staged = bf_for(case, kind, pixel_order="natural")
        plain = bf_for(case, kind, pixel_order="natural", stage_channels=False)
        assert staged._plan is not None
        a = plain(rf)
        np.testing.assert_array_equal(staged(rf), a)
        assert staged.kernel_status() == 0
        # both take fast quotients for cubic sums: against the oracle's exact
        # decisions a tap at the wrong knot would move its pixel by O(1)
        ref = oracle.das_tabbed(rf, case["tautx"], case["apodtx"], case["taurx"],
                                case["apodrx"], float(t0), float(dt), nt, interp=kind)
        assert_image_close(a, ref, rel=1e-5, peak=1e-5, what=f"{kind} near boundaries")


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only", "rx_only", "none"])
def test_cubic_vs_reference_golden(golden, name, sumtype):
    case = golden(f"tabbed_{name}.npz")
    out = bf_for(case, "cubic", sumtype)(case["rf"])
    assert_image_close(out, case[f"ref_cubic_{sumtype}"], what=f"{name}/{sumtype}")


@pytest.mark.parametrize("name", CASES)
def test_nearest_vs_reference_golden(golden, name):
    case = golden(f"tabbed_{name}.npz")
    out = bf_for(case, "nearest")(case["rf"])
    # nearest picks samples: exact up to the summation order
    assert_image_close(out, case["ref_nearest_tx_and_rx"], rel=1e-6, peak=1e-6, what=name)
    out = bf_for(case, "nearest", "rx_only")(case["rf"])
    assert_image_close(out, case["ref_nearest_rx_only"], rel=1e-6, peak=1e-6, what=name)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("kind", ["cubic", "nearest", "linear"])
def test_tap_census_bit_exact_golden_cases(golden, name, kind):
    case = golden(f"tabbed_{name}.npz")
    cnt, isum = bf_for(case, kind).tap_census()
    ok_cnt, ok_isum = oracle.tap_census(case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
                                        float(case["t0"]), float(case["dt"]), int(case["nt"]),
                                        interp="nearest" if kind == "nearest" else "cubic")
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


def test_tap_census_near_boundaries():
    """Delays placed within a few ulp of every knot and half-knot boundary."""
    rng = np.random.default_rng(42)
    nt, dt, t0 = 512, np.float32(1 / 31.25e6), np.float32(1.3e-6)
    npx = 4096
    k = rng.integers(-3, nt + 3, size=npx).astype(np.float32)
    frac = rng.choice(np.array([0.0, 0.5], np.float32), size=npx)
    base = (t0 + dt * (k + frac)).astype(np.float32)
    ulps = rng.integers(-4, 5, size=npx)
    tau = np.array([np.float32(b) for b in base], np.float32)
    for i in range(npx):
        for _ in range(abs(int(ulps[i]))):
            tau[i] = np.nextafter(tau[i], np.float32(np.inf if ulps[i] > 0 else -np.inf))
    case = dict(tautx=tau[None, :].copy(), taurx=np.zeros((2, npx), np.float32),
                apodtx=np.ones((1, npx), np.float32),
                apodrx=rng.choice(np.array([1, 0.01, 0.0099999, -0.02], np.float32), size=(2, npx)),
                t0=t0, dt=dt, nt=nt)
    for kind in ("cubic", "nearest"):
        cnt, isum = bf_for(case, kind).tap_census()
        ok_cnt, ok_isum = oracle.tap_census(case["tautx"], case["apodtx"], case["taurx"],
                                            case["apodrx"], float(t0), float(dt), nt, interp=kind)
        np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
        np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only", "rx_only", "none"])
def test_plane_wave_geometry_small_grid(tabbed_small, sumtype):
    case = tabbed_small
    out = bf_for(case, "cubic", sumtype)(case["rf"])
    ref = oracle_for(case, "cubic", sumtype, threads=NCPU)
    r, m = assert_image_close(out, ref, what=sumtype)
    report(f"tabbed_64x128_cubic_{sumtype}", rel_l2=r, max_abs_peak=m)


def test_small_grid_fp64_error_and_census(tabbed_small):
    case = tabbed_small
    out = bf_for(case, "cubic")(case["rf"])
    ref64 = oracle.das_tabbed_fp64(case["rf"], case["tautx"], case["apodtx"], case["taurx"],
                                   case["apodrx"], case["t0"], case["dt"], case["nt"])
    r64 = oracle.rel_l2(out, ref64)
    # float32 delays carry ~q*2^-24 of rounding relative to dt, so any float32
    # implementation of the reference algorithm sits ~2e-5 from float64; the GPU
    # must be no further from float64 than the reference's own float32 path
    ref32 = oracle_for(case, "cubic", threads=NCPU)
    r32 = oracle.rel_l2(ref32, ref64)
    assert r64 <= 1e-3 and r64 <= 1.25 * r32, (r64, r32)
    report("tabbed_64x128_cubic_vs_fp64", rel_l2=r64,
           max_abs_peak=oracle.max_abs_rel_peak(out, ref64), oracle_f32_rel_l2_vs_fp64=r32)
    cnt, isum = bf_for(case, "cubic").tap_census()
    ok_cnt, ok_isum = oracle.tap_census(case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
                                        case["t0"], case["dt"], case["nt"])
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


@pytest.mark.parametrize("kind", ["nearest", "linear"])
def test_other_kinds_vs_oracle(tabbed_small, kind):
    out = bf_for(tabbed_small, kind)(tabbed_small["rf"])
    ref = oracle_for(tabbed_small, kind, threads=NCPU)
    assert_image_close(out, ref, what=kind)


def test_linear_reference_floor_vs_oracle(tabbed_small):
    out = bf_for(tabbed_small, dict(kind="linear", reference_floor=True))(tabbed_small["rf"])
    ref = oracle_for(tabbed_small, "linear_floor", threads=NCPU)
    assert_image_close(out, ref, rel=1e-6, peak=1e-6, what="linear_floor")


def test_pixel_order_does_not_change_results(tabbed_small):
    a = bf_for(tabbed_small, "cubic", pixel_order="auto")(tabbed_small["rf"])
    b = bf_for(tabbed_small, "cubic", pixel_order="natural")(tabbed_small["rf"])
    np.testing.assert_array_equal(a, b)


def test_frames_batch_equals_single_frames(tabbed_small):
    rng = np.random.default_rng(1)
    frames = np.stack([tabbed_small["rf"], rng.normal(size=tabbed_small["rf"].shape).astype(np.float32),
                       -tabbed_small["rf"]])
    for sumtype in ("tx_and_rx", "tx_only"):
        bf = bf_for(tabbed_small, "cubic", sumtype)
        batch = bf(frames)
        for f in range(3):
            np.testing.assert_array_equal(batch[f], bf(frames[f]))


@pytest.mark.parametrize("storage,tol", [("float16", 1e-3), ("bfloat16", 1e-2)])
def test_reduced_precision_storage(tabbed_small, storage, tol):
    case = tabbed_small
    out = bf_for(case, "cubic", storage=storage)(case["rf"])
    ref64 = oracle.das_tabbed_fp64(case["rf"], case["tautx"], case["apodtx"], case["taurx"],
                                   case["apodrx"], case["t0"], case["dt"], case["nt"])
    r = oracle.rel_l2(out, ref64)
    report(f"tabbed_64x128_cubic_{storage}_vs_fp64", rel_l2=r)
    assert r < tol


def test_torch_io_and_buffer(tabbed_small):
    bf = bf_for(tabbed_small, "cubic")
    rf = torch.as_tensor(tabbed_small["rf"], device="cuda")
    buf = torch.empty(bf.nop, device="cuda")
    out = bf(rf, out_as_numpy=False, buffer=buf)
    assert out.data_ptr() == buf.data_ptr() and out.is_cuda
    np.testing.assert_array_equal(out.cpu().numpy(), bf(tabbed_small["rf"]))
    with pytest.raises(pg.BeamformerException):
        bf(rf, buffer=torch.empty(3, device="cuda"))
    with pytest.raises(pg.BeamformerException):
        bf(rf[:, :5])


def test_full_workload_vs_threaded_oracle():
    """The full 11 x 128 x 2048, 256 x 512 workload against the oracle."""
    w = phantom.linear_pw_tabbed(device="cuda")
    case = dict(rf=w.rf, tautx=w.tautx, apodtx=w.apodtx, taurx=w.taurx, apodrx=w.apodrx,
                t0=w.t0, dt=w.dt, nt=w.nt)
    bf = bf_for(case, "cubic")
    out = bf(case["rf"])
    ref = oracle_for(case, "cubic", threads=NCPU)
    r, m = assert_image_close(out, ref, what="full workload")
    report("tabbed_11x128x2048_cubic_vs_oracle", rel_l2=r, max_abs_peak=m)
    cnt, isum = bf.tap_census()
    ok_cnt, ok_isum = oracle.tap_census(case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
                                        case["t0"], case["dt"], case["nt"])
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)
    # size-independent property: the image is linear in the channel data
    two = bf(2 * case["rf"] - case["rf"][:, ::-1, :])
    lin = 2 * out - bf(np.ascontiguousarray(case["rf"][:, ::-1, :]))
    assert oracle.rel_l2(two, lin) < 1e-5


def test_interp_known_answer_gpu():
    import kat_interp
    d = kat_interp.make_data()
    t0, dt, nt = d["t"][0], d["t"][1] - d["t"][0], len(d["t"])
    tab = dict(tautx=d["tautxrx"], taurx=d["tautxrx"], apodtx=d["apod"], apodrx=d["apod"])
    mk = lambda kind: pg.TabbedBeamformer(**tab, t0=t0, dt=dt, nt=nt, interp={"kind": kind})
    g_near = mk("nearest")(d["rf"])
    g_cubic = mk("cubic")(d["rf"])
    o_cubic = oracle.das_tabbed(d["rf"], d["tautxrx"], d["apod"], d["tautxrx"], d["apod"], t0, dt, nt,
                                interp="cubic", threads=NCPU)
    rmse = kat_interp.rmse_roi(g_near, o_cubic, d)
    assert abs(rmse - kat_interp.NOTEBOOK_RMSE) <= 1e-6 * kat_interp.NOTEBOOK_RMSE, rmse
    err = kat_interp.rmse_roi(g_cubic, o_cubic, d)
    report("kat_gpu", rmse_nearest_vs_cubic=rmse, rmse_gpu_cubic_vs_cpu_cubic=err)
    assert err < 1e-5 * kat_interp.rms_roi(o_cubic, d)


@pytest.mark.parametrize("kind", ["cubic", "nearest", "linear"])
@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only"])
def test_staged_kernel_matches_generic(tabbed_small, kind, sumtype):
    """The TMA-staged kernel and the global-gather kernel give identical bits."""
    staged = bf_for(tabbed_small, kind, sumtype)
    plain = bf_for(tabbed_small, kind, sumtype, stage_channels=False)
    assert staged._plan is not None and plain._plan is None
    a, b = staged(tabbed_small["rf"]), plain(tabbed_small["rf"])
    np.testing.assert_array_equal(a, b)
    assert staged.kernel_status() == 0


@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only", "dmas_ssr"])
def test_staged_mixed_decisions_match_generic(sumtype):
    """Tiles whose taps all contribute next to tiles with delays past the
    record, NaN delays and transmit weights straddling the threshold: the
    staged image equals the exact-decision kernel's bit for bit, for one frame
    (receive-block items) and for two (tile items)."""
    rng = np.random.default_rng(17)
    ntx, nrx, nt, npx = 5, 16, 1024, 4096
    dt, t0 = np.float32(1 / 25e6), np.float32(2e-7)
    base = rng.uniform(100, 900, npx) * dt
    tautx = (base[None] + rng.uniform(0, 20, (ntx, npx)) * dt).astype(np.float32)
    taurx = (base[None] * 0.1 + rng.uniform(0, 20, (nrx, npx)) * dt).astype(np.float32)
    tautx[:, 1024:1100] += np.float32(nt * dt)      # past the record for one tile
    tautx[2, 2048:2060] = np.nan                     # NaN delays in another
    apodtx = np.ones((ntx, npx), np.float32)
    apodtx[3, 3000:3300] = 0.004                     # one transmit below threshold / |apodrx|
    apodrx = rng.choice(np.array([1.0, 0.5, 0.0], np.float32), size=(nrx, npx), p=[0.6, 0.3, 0.1])
    case = dict(tautx=tautx, taurx=taurx, apodtx=apodtx, apodrx=apodrx, t0=t0, dt=dt, nt=nt)
    rf = rng.normal(size=(2, ntx, nrx, nt)).astype(np.float32)
    kw = dict(pixel_order="natural")
    if sumtype == "dmas_ssr":
        mk = lambda **k: pg.TabbedDMASBeamformer(
            tautx=tautx, taurx=taurx, apodtx=apodtx, apodrx=apodrx, t0=float(t0), dt=float(dt),
            nt=nt, lags=np.arange(1, nrx), lagaxis="rx", sumlags=True, dmastype="ssr", **kw, **k)
    else:
        mk = lambda **k: bf_for(case, "cubic", sumtype, **kw, **k)
    staged, plain = mk(), mk(stage_channels=False)
    assert staged._plan is not None and getattr(staged, "_fused", True)
    for frames in (rf[0], rf):
        np.testing.assert_array_equal(staged(frames), plain(frames))
    assert staged.kernel_status() == 0


def test_staged_frames_and_half_storage(tabbed_small):
    rng = np.random.default_rng(2)
    frames = np.stack([tabbed_small["rf"], rng.normal(size=tabbed_small["rf"].shape).astype(np.float32)])
    for storage in ("float32", "float16"):
        a = bf_for(tabbed_small, "cubic", storage=storage)(frames)
        b = bf_for(tabbed_small, "cubic", storage=storage, stage_channels=False)(frames)
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only", "rx_only", "none"])
def test_many_transmits_column_form_vs_oracle(sumtype):
    """ntx > 12: the generic kernel's transmit delays in shared memory and the
    transmit weights read from the table per receive; weights straddling the
    threshold and delays past the record.  Tap census bit-exact, images within
    the parity bar."""
    rng = np.random.default_rng(29)
    ntx, nrx, nt, npx = 23, 10, 1024, 3000
    dt = np.float32(1 / 25e6)
    base = rng.uniform(50, 900, npx) * dt
    case = dict(tautx=(base[None] + rng.uniform(0, 60, (ntx, npx)) * dt).astype(np.float32),
                taurx=(base[None] * 0.2 + rng.uniform(0, 40, (nrx, npx)) * dt).astype(np.float32),
                apodtx=rng.choice(np.array([1.0, 0.3, 0.02, 0.004], np.float32), size=(ntx, npx)),
                apodrx=rng.choice(np.array([1.0, 0.6, 0.0], np.float32), size=(nrx, npx)),
                t0=np.float32(1e-7), dt=dt, nt=nt)
    case["tautx"][:, :40] += np.float32(nt * dt)
    case["rf"] = rng.normal(size=(ntx, nrx, nt)).astype(np.float32)
    bf = bf_for(case, "cubic", sumtype, pixel_order="natural")
    assert bf._plan is None  # ntx > 12: the generic kernel
    assert_image_close(bf(case["rf"]), oracle_for(case, "cubic", sumtype, threads=NCPU),
                       what=f"ntx {ntx} {sumtype}")
    cnt, isum = bf.tap_census()
    ok_cnt, ok_isum = oracle.tap_census(case["tautx"], case["apodtx"], case["taurx"],
                                        case["apodrx"], float(case["t0"]), float(dt), nt)
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


def test_staged_kernel_unstaged_receives():
    """Delays spread over the whole record: no window fits a stage, so every
    receive takes the kernel's global-gather path (with padded transmits)."""
    rng = np.random.default_rng(5)
    ntx, nrx, nt, npx = 11, 24, 2048, 640
    dt = np.float32(4e-8)
    case = dict(tautx=rng.uniform(0, nt * dt * 0.5, (ntx, npx)).astype(np.float32),
                taurx=rng.uniform(0, nt * dt * 0.5, (nrx, npx)).astype(np.float32),
                apodtx=rng.uniform(0.5, 1, (ntx, npx)).astype(np.float32),
                apodrx=rng.uniform(-1, 1, (nrx, npx)).astype(np.float32),
                t0=np.float32(0), dt=dt, nt=nt)
    frames = rng.normal(size=(3, ntx, nrx, nt)).astype(np.float32)
    for kind in ("cubic", "nearest", "linear"):
        a = bf_for(case, kind, pixel_order="natural")(frames)
        b = bf_for(case, kind, pixel_order="natural", stage_channels=False)(frames)
        np.testing.assert_array_equal(a, b)
    ref = oracle.das_tabbed(frames[2], case["tautx"], case["apodtx"], case["taurx"],
                            case["apodrx"], 0.0, float(dt), nt)
    assert_image_close(bf_for(case, "cubic")(frames)[2], ref, what="unstaged")


@pytest.mark.parametrize("name", CASES)
def test_nearest_usf4_vs_reference_golden(golden, name):
    """Nearest with the cubic 4x upsampling of beamform_nearest (pycbf.c:223-253):
    the reference's own compiled output, and the tap set of the oracle."""
    case = golden(f"tabbed_{name}.npz")
    bf = bf_for(case, dict(kind="nearest", usf=4))
    out = bf(case["rf"])
    assert_image_close(out, case["ref_nearest_usf4_tx_and_rx"], what=name)
    cnt, isum = bf.tap_census()
    ok_cnt, ok_isum = oracle.tap_census(case["tautx"], case["apodtx"], case["taurx"], case["apodrx"],
                                        float(case["t0"]), float(case["dt"]), int(case["nt"]),
                                        interp="nearest", usf=4)
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


@pytest.mark.parametrize("usf", [2, 5])
def test_nearest_upsampled_vs_oracle(tabbed_small, usf):
    out = bf_for(tabbed_small, dict(kind="nearest", usf=usf))(tabbed_small["rf"])
    ref = oracle.das_tabbed(tabbed_small["rf"], tabbed_small["tautx"], tabbed_small["apodtx"], tabbed_small["taurx"],
                            tabbed_small["apodrx"], tabbed_small["t0"], tabbed_small["dt"], tabbed_small["nt"],
                            interp="nearest", usf=usf, threads=NCPU)
    r, m = assert_image_close(out, ref, what=f"usf {usf}")
    report(f"tabbed_nearest_usf{usf}", rel_l2=r, max_abs_peak=m)


@pytest.mark.parametrize("interp", [dict(kind="korder_cubic", k=8), dict(kind="korder_cubic", k=16),
                                    dict(kind="korder_cubic", k=8, zero_slopes=True),
                                    dict(kind="akima"), dict(kind="makima")])
def test_gpu_only_interpolators_vs_oracle(tabbed_small, interp):
    """korder / akima / makima (the reference's CUDA interpolators, restated in
    the oracle from __engines__.cu:58-355): tap set bit-exact, image within
    the float32 bar."""
    c = tabbed_small
    bf = bf_for(c, interp)
    out = bf(c["rf"])
    kind = interp["kind"]
    k = 0 if interp.get("zero_slopes") else interp.get("k", 8)
    ref = oracle.das_poly(c["rf"], c["tautx"], c["apodtx"], c["taurx"], c["apodrx"], c["t0"],
                          c["dt"], c["nt"], kind, k=k)
    r, m = assert_image_close(out, ref, what=str(interp))
    report(f"tabbed_{kind}_k{k}", rel_l2=r, max_abs_peak=m)
    cnt, isum = bf.tap_census()
    ok_cnt, ok_isum = oracle.tap_census(c["tautx"], c["apodtx"], c["taurx"], c["apodrx"], c["t0"],
                                        c["dt"], c["nt"], interp=kind)
    np.testing.assert_array_equal(cnt.cpu().numpy(), ok_cnt)
    np.testing.assert_array_equal(isum.cpu().numpy(), ok_isum)


def test_korder_large_k_and_edges(golden):
    """k = 126 (the reference notebook's setting) and k = nt on golden cases
    whose taps reach both ends of the record."""
    for name in ("edge", "pw_small"):
        case = golden(f"tabbed_{name}.npz")
        nt = int(case["nt"])
        k = min(126, nt - nt % 2)
        out = bf_for(case, dict(kind="korder_cubic", k=k))(case["rf"])
        ref = oracle.das_poly(case["rf"], case["tautx"], case["apodtx"], case["taurx"],
                              case["apodrx"], float(case["t0"]), float(case["dt"]), nt,
                              "korder_cubic", k=k)
        assert_image_close(out, ref, what=f"{name} k={k}")


def test_beamform_stream_equals_calls(tabbed_small):
    """Frames streamed from host memory with overlapped copies give the images
    of one call per frame, bit for bit (float32 pinned and pageable, int16,
    4-D frames)."""
    bf = bf_for(tabbed_small, "cubic")
    rng = np.random.default_rng(7)
    rf = tabbed_small["rf"]
    frames = [rf, (rf * 0.5).astype(np.float32), torch.from_numpy(rf[::-1].copy()).pin_memory(),
              rng.normal(size=rf.shape).astype(np.float32)]
    got = list(bf.beamform_stream(frames))
    assert len(got) == len(frames)
    for g, f in zip(got, frames):
        np.testing.assert_array_equal(g, bf(f))
    counts = [np.round(rf / np.abs(rf).max() * 30000).astype(np.int16)] * 3
    for g, f in zip(bf.beamform_stream(counts), counts):
        np.testing.assert_array_equal(g, bf(f))
    four = np.stack([rf, rf[::-1].copy()])
    (g,) = list(bf.beamform_stream([four]))
    np.testing.assert_array_equal(g, bf(four))
    dm = pg.TabbedDMASBeamformer(tautx=tabbed_small["tautx"], taurx=tabbed_small["taurx"],
                                 apodtx=tabbed_small["apodtx"], apodrx=tabbed_small["apodrx"],
                                 t0=float(tabbed_small["t0"]), dt=float(tabbed_small["dt"]),
                                 nt=int(tabbed_small["nt"]), lags=np.arange(1, 4))
    with pytest.raises(pg.BeamformerException):
        list(dm.beamform_stream([rf]))

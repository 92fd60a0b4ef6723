"""GPU-built delay tables against the reference's own table helper (golden
fixture) and the NumPy restatement in the oracle."""
import os
import sys

import numpy as np
import pytest
import torch

from oracle import tables_ref

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_tables_golden as mtg  # noqa: E402


@pytest.mark.parametrize("name", list(mtg.CASES))
def test_oracle_restatement_matches_the_reference_helper(golden, name):
    g = golden("tables_2d.npz")
    steers, ctx, cm, xele, xout, zout, fnum = mtg.inputs()
    r0 = mtg.CASES[name]
    t = tables_ref.make_tabs_and_apods_2d(steers, r0, ctx if r0 == 0 else cm, cm, xele, xout, zout,
                                          fnum)
    for k, v in t.items():
        np.testing.assert_array_equal(np.asarray(v, np.float64).astype(np.float32), g[f"{name}_{k}"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(mtg.CASES))
def test_gpu_tables_match_the_reference_helper(golden, name):
    from pycbf_gb300.tables import make_tabs_and_apods_2d
    g = golden("tables_2d.npz")
    steers, ctx, cm, xele, xout, zout, fnum = mtg.inputs()
    r0 = mtg.CASES[name]
    t = make_tabs_and_apods_2d(steers, r0, ctx if r0 == 0 else cm, cm, xele, xout, zout, fnum)
    for k, v in t.items():
        ref = g[f"{name}_{k}"]
        got = v.cpu().numpy()
        if name == "focused" and k == "apodtx":  # acos on the device vs NumPy's: ties may flip
            assert np.count_nonzero(got != ref) <= 2
        else:
            np.testing.assert_array_equal(got, ref, err_msg=k)


@pytest.mark.gpu
def test_gpu_tables_at_benchmark_size_and_hann():
    """The 128-element, 11-angle, 256 x 512 tables: identical to the oracle's
    float64 restatement rounded to float32, the Hann-weighted receive mask
    within one float32 ulp of NumPy's, and the images they give identical."""
    from pycbf_gb300 import TabbedBeamformer, helpers, phantom
    from pycbf_gb300.tables import make_tabs_and_apods_2d
    xele = helpers.element_positions(128, 0.3e-3)
    steers = np.radians(np.linspace(-10, 10, 11))
    xout, zout = np.linspace(-19e-3, 19e-3, 256), np.linspace(5e-3, 45e-3, 512)
    t = make_tabs_and_apods_2d(steers, 0.0, 1540.0, 1540.0, xele, xout, zout, 1.5, hann=True)
    ref = tables_ref.make_tabs_and_apods_2d(steers, 0.0, 1540.0, 1540.0, xele, xout, zout, 1.5)
    for k in ("tautx", "taurx", "apodtx"):
        np.testing.assert_array_equal(t[k].cpu().numpy(), ref[k].astype(np.float32), err_msg=k)
    _, hann = helpers.rx_tables(1540.0, xele, xout, zout, 1.5, hann=True)
    got = t["apodrx"].cpu().numpy()
    want = hann.astype(np.float32)
    assert np.max(np.abs(got - want)) <= np.spacing(np.float32(1.0))
    w = phantom.linear_pw_tabbed(device="cuda", n_speckle=500)
    args = dict(t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": "cubic"})
    # the workload's transmit apodization is all ones (the reference's plane-wave
    # helper masks the projected aperture instead)
    a = TabbedBeamformer(tautx=t["tautx"], taurx=t["taurx"], apodtx=torch.ones_like(t["apodtx"]),
                         apodrx=t["apodrx"], **args)(w.rf)
    b = TabbedBeamformer(tautx=w.tautx, taurx=w.taurx, apodtx=w.apodtx, apodrx=w.apodrx,
                         **args)(w.rf)
    assert np.max(np.abs(a - b)) <= 1e-5 * np.max(np.abs(b))


def test_host_helpers_match_reference_golden(golden):
    """helpers.pw_tx_tables / rx_tables (the NumPy builders the phantoms and the
    bench use) give the reference helper's plane-wave tables, rounded to
    float32, bit for bit."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_tables_golden as mk

    from pycbf_gb300 import helpers
    g = golden("tables_2d.npz")
    steers, ctx, cm, xele, xout, zout, fnum = mk.inputs()
    tt, at = helpers.pw_tx_tables(steers, ctx, cm, xele, xout, zout)
    tr, ar = helpers.rx_tables(cm, xele, xout, zout, fnum)
    for name, v in (("tautx", tt), ("apodtx", at), ("taurx", tr), ("apodrx", ar)):
        np.testing.assert_array_equal(v.astype(np.float32), g[f"pw_{name}"], err_msg=name)


def test_synthetic_point_parameters_match_reference_golden(golden):
    """helpers.pw_synthetic_points equals the reference's
    calc_tx_synthetic_points_pw_2D + calc_rx_synthetic_points (golden made by
    them, tests/golden/make_synth_points_golden.py) bit for bit."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_synth_points_golden as mk

    from pycbf_gb300 import helpers
    g = golden("synth_points.npz")
    steers, ctx, cm, xele, fnum, rpw = mk.inputs()
    p = helpers.pw_synthetic_points(steers, ctx, cm, xele, fnum, rpw)
    for k in g:
        np.testing.assert_array_equal(np.asarray(p[k], np.float64), g[k].astype(np.float64), err_msg=k)

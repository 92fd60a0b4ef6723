"""The adjoint kernels of the differentiable cubic delay-and-sum against the
float64 autograd reference and central differences (GPU)."""
import numpy as np
import pytest
import torch

from oracle import adjoint_ref
from pycbf_gb300 import SyntheticBeamformer, TabbedBeamformer, adjoint, phantom, sos

pytestmark = pytest.mark.gpu

SMALL = dict(nele=16, nsteer=3, nt=512, nx=24, nz=40, xlim=(-2.4e-3, 2.4e-3), zlim=(4e-3, 12e-3),
             n_speckle=200, n_points=3)


def rel(a, b):
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.fixture(scope="module")
def tab():
    return phantom.linear_pw_tabbed(device="cuda", **SMALL)


@pytest.fixture(scope="module")
def syn():
    return phantom.two_layer_pw_synthetic(device="cuda", z_interface=7e-3, **SMALL)


def _frames(rf):
    r = torch.as_tensor(rf, device="cuda")
    return torch.stack([r, 0.5 * r.flip(-1)]).contiguous()


def _tables(w):
    return [torch.as_tensor(a, device="cuda") for a in (w.tautx, w.taurx, w.apodtx, w.apodrx)]


def test_forward_equals_the_beamformer(tab):
    tautx, taurx, apodtx, apodrx = _tables(tab)
    rf = torch.as_tensor(tab.rf, device="cuda")
    bf = TabbedBeamformer(tautx=tab.tautx, apodtx=tab.apodtx, taurx=tab.taurx, apodrx=tab.apodrx,
                          t0=tab.t0, dt=tab.dt, nt=tab.nt, interp={"kind": "cubic"},
                          sumtype="tx_and_rx", pixel_order="natural")
    img = adjoint.das_tabbed(rf, tautx, taurx, apodtx, apodrx, t0=tab.t0, dt=tab.dt)
    assert torch.equal(img, bf(rf, out_as_numpy=False))
    img2 = bf.differentiable(rf)
    assert torch.equal(img, img2)


@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only"])
def test_tabbed_gradients_match_float64_autograd(tab, sumtype):
    tautx, taurx, apodtx, apodrx = _tables(tab)
    rf = _frames(tab.rf).requires_grad_(True)
    ttx, trx = tautx.clone().requires_grad_(True), taurx.clone().requires_grad_(True)
    out = adjoint.das_tabbed(rf, ttx, trx, apodtx, apodrx, t0=tab.t0, dt=tab.dt, sumtype=sumtype)
    g = torch.randn(out.shape, generator=torch.Generator().manual_seed(1)).cuda()
    (out * g).sum().backward()

    D = lambda t: t.detach().double().cpu().requires_grad_(True)
    rf64, ttx64, trx64 = D(rf), D(ttx), D(trx)
    ref = adjoint_ref.das_tabbed_ref(rf64, ttx64, trx64, apodtx.double().cpu(),
                                     apodrx.double().cpu(), tab.t0, tab.dt, 0.01, sumtype)
    (ref * g.double().cpu()).sum().backward()
    errs = dict(image=rel(out, ref), rf=rel(rf.grad, rf64.grad), tautx=rel(ttx.grad, ttx64.grad),
                taurx=rel(trx.grad, trx64.grad))
    print(sumtype, errs)
    assert errs["image"] <= 1e-5 and errs["rf"] <= 1e-5
    assert errs["tautx"] <= 1e-4 and errs["taurx"] <= 1e-4


def test_tabbed_gradients_match_central_differences(tab):
    tautx, taurx, apodtx, apodrx = _tables(tab)
    rf = _frames(tab.rf)
    gen = torch.Generator().manual_seed(2)
    w = torch.randn((2, tautx.shape[1]), generator=gen).cuda()
    L = lambda r, a, b: float((w * adjoint.das_tabbed(r, a, b, apodtx, apodrx, t0=tab.t0,
                                                       dt=tab.dt)).double().sum())
    rf_g, ttx, trx = rf.clone().requires_grad_(True), tautx.clone().requires_grad_(True), \
        taurx.clone().requires_grad_(True)
    (w * adjoint.das_tabbed(rf_g, ttx, trx, apodtx, apodrx, t0=tab.t0, dt=tab.dt)).sum().backward()
    # channel data: the image is linear in them (h = 1e-3 of the data scale)
    v = torch.randn(rf.shape, generator=gen).cuda()
    h = 1e-3 * float(rf.abs().max())
    fd = (L(rf + h * v, tautx, taurx) - L(rf - h * v, tautx, taurx)) / (2 * h)
    an = float((rf_g.grad.double() * v.double()).sum())
    assert abs(fd - an) <= 1e-3 * abs(an)
    # delays: a step of 1e-2 of the sample interval
    for which in ("tautx", "taurx"):
        base = tautx if which == "tautx" else taurx
        grad = ttx.grad if which == "tautx" else trx.grad
        v = torch.randn(base.shape, generator=gen).cuda()
        h = 1e-2 * tab.dt
        p = (base + h * v, base - h * v)
        if which == "tautx":
            fd = (L(rf, p[0], taurx) - L(rf, p[1], taurx)) / (2 * h)
        else:
            fd = (L(rf, tautx, p[0]) - L(rf, tautx, p[1])) / (2 * h)
        an = float((grad.double() * v.double()).sum())
        assert abs(fd - an) <= 1e-2 * abs(an), (which, fd, an)


def _synth_bf(w, order="natural", storage="float32"):
    g = w.geometry
    return SyntheticBeamformer(ovectx=g["ovectx"], nvectx=g["nvectx"], doftx=g["doftx"],
                               alatx=g["alatx"], t0tx=g["t0tx"], ovecrx=g["ovecrx"],
                               nvecrx=g["nvecrx"], alarx=g["alarx"], c0=g["c0"], pnts=g["pnts"],
                               t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": "cubic"},
                               sumtype="tx_and_rx", pixel_order=order, storage=storage)


def _synth_ref(w, rf, s, sumtype):
    g = w.geometry
    f32 = lambda a: np.asarray(a, np.float32)
    cosalarx = np.cos(f32(g["alarx"]).astype(np.float64)).astype(np.float32)
    return adjoint_ref.das_synth_pw_ref(rf, s, f32(g["pnts"]), f32(g["ovectx"]), f32(g["nvectx"]),
                                        f32(g["ovecrx"]), f32(g["nvecrx"]), cosalarx, w.t0, w.dt,
                                        sumtype)


def test_uniform_slowness_matches_the_synthetic_forward(syn):
    bf = _synth_bf(syn)
    rf = torch.as_tensor(syn.rf, device="cuda")
    img = bf.differentiable(rf)
    ref = bf(rf, out_as_numpy=False)
    # delays D * fl(1/c0) vs fl(D / c0) differ by an ulp: ~1e-5 of the image
    assert rel(img, ref) <= 5e-5


@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only"])
def test_synthetic_gradients_match_float64_autograd(syn, sumtype):
    bf = _synth_bf(syn)
    rf = _frames(syn.rf).requires_grad_(True)
    s = torch.as_tensor(syn.meta["slowness_true"], dtype=torch.float32, device="cuda")
    s = s.clone().requires_grad_(True)
    out = bf.differentiable(rf, slowness=s, sumtype=sumtype)
    g = torch.randn(out.shape, generator=torch.Generator().manual_seed(3)).cuda()
    (out * g).sum().backward()
    rf64 = rf.detach().double().cpu().requires_grad_(True)
    s64 = s.detach().double().cpu().requires_grad_(True)
    ref = _synth_ref(syn, rf64, s64, sumtype)
    (ref * g.double().cpu()).sum().backward()
    errs = dict(image=rel(out, ref), rf=rel(rf.grad, rf64.grad), slowness=rel(s.grad, s64.grad))
    print(sumtype, errs)
    assert errs["image"] <= 1e-5 and errs["rf"] <= 1e-5 and errs["slowness"] <= 1e-4


def test_slowness_gradient_matches_central_differences(syn):
    bf = _synth_bf(syn)
    rf = torch.as_tensor(syn.rf, device="cuda")
    s0 = torch.as_tensor(syn.meta["slowness_true"], dtype=torch.float32, device="cuda")
    gen = torch.Generator().manual_seed(4)
    w = torch.randn((s0.shape[0],), generator=gen).cuda()
    s = s0.clone().requires_grad_(True)
    (w * bf.differentiable(rf, slowness=s)).sum().backward()
    L = lambda ss: float((w * bf.differentiable(rf, slowness=ss)).double().sum())
    tmax = 2 * 12e-3 * float(s0.max())
    for v in (s0, torch.randn(s0.shape, generator=gen).cuda() * s0):
        h = 1e-2 * syn.dt / tmax  # moves the deepest delays by 1e-2 of a sample
        fd = (L(s0 + h * v) - L(s0 - h * v)) / (2 * h)
        an = float((s.grad.double() * v.double()).sum())
        assert abs(fd - an) <= 1e-2 * abs(an), (fd, an)


def test_backward_is_bitwise_reproducible(tab):
    tautx, taurx, apodtx, apodrx = _tables(tab)
    grads = []
    for _ in range(2):
        rf = _frames(tab.rf).requires_grad_(True)
        ttx = tautx.clone().requires_grad_(True)
        out = adjoint.das_tabbed(rf, ttx, taurx, apodtx, apodrx, t0=tab.t0, dt=tab.dt)
        out.sum().backward()
        grads.append((rf.grad.clone(), ttx.grad.clone()))
    assert torch.equal(grads[0][0], grads[1][0]) and torch.equal(grads[0][1], grads[1][1])


def test_pixel_order_and_half_storage(syn):
    rf = torch.as_tensor(syn.rf, device="cuda")
    s0 = torch.as_tensor(syn.meta["slowness_true"], dtype=torch.float32, device="cuda")
    res = {}
    for order, storage in (("natural", "float32"), ("auto", "float32"), ("auto", "float16"),
                           ("auto", "bfloat16")):
        bf = _synth_bf(syn, order, storage)
        r = rf.clone().requires_grad_(True)
        s = s0.clone().requires_grad_(True)
        out = bf.differentiable(r, slowness=s)
        out.sum().backward()
        res[(order, storage)] = (out.detach(), r.grad.float(), s.grad)
    base = res[("natural", "float32")]
    auto = res[("auto", "float32")]
    assert torch.equal(base[0], auto[0])
    assert rel(auto[1], base[1]) <= 1e-6 and rel(auto[2], base[2]) <= 1e-6
    for storage, tol in (("float16", 5e-3), ("bfloat16", 3e-2)):
        o, gr, gs = res[("auto", storage)]
        assert rel(o, base[0]) <= tol and rel(gs, base[2]) <= 2 * tol
        assert rel(gr, base[1]) <= tol   # the channel-data adjoint does not read the data


def test_speed_of_sound_loss_backpropagates(syn):
    bf = _synth_bf(syn, "auto")
    rf = torch.as_tensor(syn.rf, device="cuda")
    mask = bf.rx_mask()
    model = sos.SlownessModel(syn.grid, map_shape=(4, 8), c_init=1540.0)
    img = bf.differentiable(rf, slowness=model(), sumtype="tx_only")
    loss = sos.sos_loss(img, mask, syn.grid, nkern=2)
    loss.backward()
    assert torch.isfinite(loss) and torch.isfinite(model.c.grad) and float(model.c.grad) != 0.0
    assert torch.isfinite(model.dmap.grad).all() and float(model.dmap.grad.abs().sum()) > 0
    # d loss / d c against central differences.  A relative step of 1e-3 moves
    # the deepest delays by ~0.4 sample (0.5 rad of the 5 MHz carrier), where
    # the coherence loss is far from linear (the float64 reference gives
    # 0.00396 there against 0.00190 in the limit); the differences converge
    # by h = 1e-4.
    with torch.no_grad():
        c = float(model.c)

        def at(cc):
            model.c.fill_(cc)
            out = bf.differentiable(rf, slowness=model(), sumtype="tx_only")
            return float(sos.sos_loss(out, mask, syn.grid, nkern=2).double())

        fd = {h: (at(c * (1 + h)) - at(c * (1 - h))) / (2 * h * c) for h in (1e-3, 1e-4, 3e-5)}
        model.c.fill_(c)
    an = float(model.c.grad)
    print("dL/dc analytic", an, "central differences", fd)
    assert abs(fd[1e-4] - an) <= 0.05 * abs(an) and abs(fd[3e-5] - an) <= 0.05 * abs(an)


def test_caller_delay_tables_in_any_pixel_order(tab):
    """Learnable delay tables go through the beamformer in the caller's pixel
    order whatever order the beamformer keeps its own tables in."""
    tautx, taurx, apodtx, apodrx = _tables(tab)
    rf = torch.as_tensor(tab.rf, device="cuda")
    res = []
    for order in ("auto", "natural"):
        bf = TabbedBeamformer(tautx=tab.tautx, apodtx=tab.apodtx, taurx=tab.taurx, apodrx=tab.apodrx,
                              t0=tab.t0, dt=tab.dt, nt=tab.nt, interp={"kind": "cubic"},
                              pixel_order=order)
        r = rf.clone().requires_grad_(True)
        ttx, trx = tautx.clone().requires_grad_(True), taurx.clone().requires_grad_(True)
        out = bf.differentiable(r, tautx=ttx, taurx=trx)
        out.sum().backward()
        res.append((out.detach(), r.grad, ttx.grad, trx.grad))
    assert torch.equal(res[0][0], res[1][0])
    assert torch.equal(res[0][2], res[1][2]) and torch.equal(res[0][3], res[1][3])
    assert rel(res[0][1], res[1][1]) <= 1e-6
    ref = TabbedBeamformer(tautx=tab.tautx, apodtx=tab.apodtx, taurx=tab.taurx, apodrx=tab.apodrx,
                           t0=tab.t0, dt=tab.dt, nt=tab.nt, interp={"kind": "cubic"})(rf, out_as_numpy=False)
    assert torch.equal(res[0][0], ref)


@pytest.mark.parametrize("sumtype", ["tx_and_rx", "tx_only"])
def test_planned_delay_gradients_equal_the_generic(tab, sumtype):
    """With the forward's staging plan the delay gradients gather the spline
    records from the plan's staged windows (the staged kernel in its adjoint
    mode): the same taps, products and summation order as the generic kernel,
    so the same bits; the image and the channel-data gradient are unchanged."""
    bf = TabbedBeamformer(tautx=tab.tautx, apodtx=tab.apodtx, taurx=tab.taurx, apodrx=tab.apodrx,
                          t0=tab.t0, dt=tab.dt, nt=tab.nt, interp={"kind": "cubic"})
    assert bf._plan is not None and bf._pixel_index is not None
    ktx, kap_tx, krx, kap_rx = bf._tables
    rf = torch.as_tensor(tab.rf, device="cuda")
    res = []
    for plan in (None, bf._plan):
        r = rf.clone().requires_grad_(True)
        ttx, trx = ktx.clone().requires_grad_(True), krx.clone().requires_grad_(True)
        out = adjoint.das_tabbed(r, ttx, trx, kap_tx, kap_rx, t0=tab.t0, dt=tab.dt,
                                 thresh=bf.thresh, sumtype=sumtype, pixel_index=bf._pixel_index,
                                 plan=plan)
        g = torch.randn(out.shape, generator=torch.Generator().manual_seed(4)).cuda()
        (out * g).sum().backward()
        res.append((out.detach(), ttx.grad, trx.grad, r.grad))
    assert torch.equal(res[0][0], res[1][0])
    assert torch.equal(res[0][1], res[1][1]) and torch.equal(res[0][2], res[1][2])
    assert torch.equal(res[0][3], res[1][3])
    assert float(res[1][1].abs().sum()) > 0 and float(res[1][2].abs().sum()) > 0

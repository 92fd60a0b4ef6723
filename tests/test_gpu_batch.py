"""Uneven batches: frames of different beamformers, sizes and storage types in
one persistent launch (replayed as a CUDA graph) give each beamformer's own
image (GPU)."""
import numpy as np
import pytest
import torch

from pycbf_gb300 import SyntheticBeamformer, TabbedBeamformer, phantom
from pycbf_gb300.batch import BatchBeamformer, BatchConfig

pytestmark = pytest.mark.gpu


def _tabbed(w, storage="float32", order="auto"):
    return TabbedBeamformer(tautx=w.tautx, apodtx=w.apodtx, taurx=w.taurx, apodrx=w.apodrx,
                            t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": "cubic"},
                            storage=storage, pixel_order=order)


def _synth(w, storage="float32"):
    g = w.geometry
    return SyntheticBeamformer(ovectx=g["ovectx"], nvectx=g["nvectx"], doftx=g["doftx"],
                               alatx=g["alatx"], t0tx=g["t0tx"], ovecrx=g["ovecrx"],
                               nvecrx=g["nvecrx"], alarx=g["alarx"], c0=g["c0"], pnts=g["pnts"],
                               t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": "cubic"},
                               storage=storage)


@pytest.fixture(scope="module")
def batch():
    small = dict(xlim=(-3e-3, 3e-3), zlim=(4e-3, 14e-3), n_speckle=150, n_points=3)
    wa = phantom.linear_pw_tabbed(nele=16, nsteer=3, nt=512, nx=24, nz=40, device="cuda", **small)
    wb = phantom.linear_pw_tabbed(nele=24, nsteer=13, nt=1024, nx=16, nz=24, device="cuda", **small)
    wc = phantom.linear_pw_synthetic(nele=24, nsteer=5, nt=1024, nx=20, nz=32, device="cuda",
                                     **small)
    wd = phantom.linear_pw_synthetic(nele=32, nsteer=15, nt=2048, nx=12, nz=20, device="cuda",
                                     **small)
    entries = [(_tabbed(wa), wa), (_tabbed(wb), wb), (_synth(wc), wc), (_synth(wd, "float16"), wd),
               (_tabbed(wa, "bfloat16"), wa), (_tabbed(wa, order="natural"), wa)]
    frames = [torch.as_tensor(w.rf, device="cuda") for _, w in entries]
    frames[-1] = 0.5 * frames[-1].flip(-1)  # another frame through the same tables
    singles = [bf(f, out_as_numpy=False).clone() for (bf, _), f in zip(entries, frames)]
    return [bf for bf, _ in entries], frames, singles


def _rel(a, b):
    return float(torch.linalg.norm((a - b).double()) / torch.linalg.norm(b.double()))


@pytest.mark.parametrize("cfg", [BatchConfig(), BatchConfig(2, 0, 8, 2), BatchConfig(4, 1, 4, 3),
                                 BatchConfig(1, 1, 0, 4), BatchConfig(2, 0, 0, 2),
                                 BatchConfig(branches=4), BatchConfig(branches=1)])
def test_batch_matches_single_frames(batch, cfg):
    bfs, frames, singles = batch
    bb = BatchBeamformer(bfs, config=cfg)
    outs = bb(frames)
    for k, (o, s, bf) in enumerate(zip(outs, singles, bfs)):
        if cfg.branches > 0 or cfg.tx_chunk == 0 or bf.ntx <= cfg.tx_chunk:
            assert torch.equal(o, s), (k, _rel(o, s))  # same operations in the same order
        else:
            assert _rel(o, s) <= 1e-6, (k, _rel(o, s))


@pytest.mark.parametrize("storage", ["float32", "float16", "bfloat16"])
@pytest.mark.parametrize("big", [False, True])
def test_one_storage_type_queue_matches_single_frames(batch, storage, big):
    """A batch of one storage type runs the queue kernel compiled for that type
    alone (the shared-memory column form for every ntx), with all jobs at
    ntx <= 12 (big=False: a column of at most 12 transmits) or with larger
    ones: bitwise the single-frame images."""
    small = dict(xlim=(-3e-3, 3e-3), zlim=(4e-3, 14e-3), n_speckle=150, n_points=3)
    wa = phantom.linear_pw_tabbed(nele=16, nsteer=3, nt=512, nx=24, nz=40, device="cuda", **small)
    wc = phantom.linear_pw_synthetic(nele=24, nsteer=5, nt=1024, nx=20, nz=32, device="cuda",
                                     **small)
    entries = [(_tabbed(wa, storage), wa), (_synth(wc, storage), wc),
               (_tabbed(wa, storage, order="natural"), wa)]
    if big:
        wb = phantom.linear_pw_tabbed(nele=24, nsteer=13, nt=1024, nx=16, nz=24, device="cuda",
                                      **small)
        wd = phantom.linear_pw_synthetic(nele=32, nsteer=15, nt=2048, nx=12, nz=20, device="cuda",
                                         **small)
        entries += [(_tabbed(wb, storage), wb), (_synth(wd, storage), wd)]
    dt = {"float32": torch.float32, "float16": torch.float16, "bfloat16": torch.bfloat16}[storage]
    frames = [torch.as_tensor(w.rf, device="cuda").to(dt) for _, w in entries]
    singles = [bf(f, out_as_numpy=False).clone() for (bf, _), f in zip(entries, frames)]
    bfs = [bf for bf, _ in entries]
    assert (max(b.ntx for b in bfs) > 12) == big
    for cfg in (BatchConfig(1, 1, 0, 4), BatchConfig(2, 0, 0, 3)):
        outs = BatchBeamformer(bfs, config=cfg)(frames)
        for k, (o, s) in enumerate(zip(outs, singles)):
            assert torch.equal(o, s), (storage, big, cfg, k, _rel(o, s))


def test_graph_replay_follows_the_inputs(batch):
    bfs, frames, singles = batch
    bb = BatchBeamformer(bfs, config=BatchConfig())
    bb(frames)
    first = [o.clone() for o in bb.outputs]
    outs = bb([2.0 * f for f in frames])
    for o, f0 in zip(outs, first):
        assert _rel(o, 2.0 * f0) <= 1e-6
    outs = bb(frames)
    for o, f0 in zip(outs, first):
        assert torch.equal(o, f0)


def test_autotuner_picks_and_caches(batch):
    bfs, frames, singles = batch
    bb = BatchBeamformer(bfs)  # autotunes
    # the queue form and two branch counts at least
    assert isinstance(bb.config, BatchConfig) and len(bb.timings) >= 3
    assert {c.branches for c in bb.timings} >= {0, 4, 8}
    assert bb.config == min(bb.timings, key=bb.timings.get)
    bb2 = BatchBeamformer(bfs)
    assert bb2.config == bb.config
    outs = bb2(frames)
    for o, s in zip(outs, singles):
        assert _rel(o, s) <= 1e-6


@pytest.mark.slow
def test_uneven_64_frame_batch_storage_errors_against_fp64():
    """64 seeded frames (ntx 1..75, nrx 64..192, nt 1024..4096, grids 128x128 ..
    512x1024, Tabbed and Synthetic) in float32, float16 and bfloat16 storage;
    per frame, the image on 64 random pixels against the float64 oracle."""
    from oracle import oracle
    from gpu_util import report
    from pycbf_gb300.batch import beamformers_for

    frames = phantom.batch_frames(n=64, device="cuda")
    rng = np.random.default_rng(7)
    subsets, refs = [], []
    for f in frames:
        np_ = f["nx"] * f["nz"]
        sub = np.sort(rng.choice(np_, 64, replace=False))
        rf = f["rf"].cpu().numpy()
        if f["kind"] == "tabbed":
            tabs = [f[k][:, torch.as_tensor(sub, device="cuda")].cpu().numpy()
                    for k in ("tautx", "apodtx", "taurx", "apodrx")]
        else:
            g = f["geometry"]
            tabs = oracle.synth_tables(g["ovectx"], g["nvectx"], g["doftx"], g["alatx"], g["t0tx"],
                                       g["ovecrx"], g["nvecrx"], g["alarx"], g["c0"],
                                       g["pnts"][sub])
        refs.append(oracle.das_fp64_columns(rf, *tabs, f["t0"], f["dt"]))
        subsets.append(torch.as_tensor(sub, device="cuda"))
    errs = {}
    images32 = None
    for storage in ("float32", "float16", "bfloat16"):
        bb = BatchBeamformer(beamformers_for(frames, storage), config=BatchConfig())
        outs = bb([f["rf"] for f in frames])
        errs[storage] = [oracle.rel_l2(o[s].cpu().numpy(), r) for o, s, r in zip(outs, subsets, refs)]
        if storage == "float32":
            images32 = [o.clone() for o in outs]
        else:
            vs32 = [_rel(o, i) for o, i in zip(outs, images32)]
            errs[storage + "_vs_f32"] = vs32
        del bb
    for k, f in enumerate(frames):
        report(f"batch64 frame {k} {f['kind']} {f['ntx']}x{f['nrx']}x{f['nt']} {f['nx']}x{f['nz']}",
               **{f"fp64_{s}": errs[s][k] for s in ("float32", "float16", "bfloat16")},
               f16_vs_f32=errs["float16_vs_f32"][k], bf16_vs_f32=errs["bfloat16_vs_f32"][k])
    print({k: (float(np.median(v)), float(np.max(v))) for k, v in errs.items()})
    # Float32 delays near 60 us resolve 2^-24 * 64 us ~ 3.8 ps, 3e-4 rad of a
    # 12.8 MHz carrier: the float32 path (the reference's C path alike) carries
    # up to a few 1e-4 of image error against float64 from the delays alone.
    assert max(errs["float32"]) <= 1e-3
    assert max(errs["float16"]) <= 1e-3
    assert max(errs["bfloat16"]) <= 1e-2  # 8-bit significands: ~2e-3 per sample

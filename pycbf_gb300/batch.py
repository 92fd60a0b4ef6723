"""Uneven batches of frames replayed as one CUDA graph (no counterpart in the
reference, whose beamformers take one frame shape per instance and launch per
call).

``BatchBeamformer(beamformers)`` takes a list of Tabbed / Synthetic
beamformers, one entry per frame (an instance may appear several times for
several frames); frames may differ in ntx, nrx, nt, pixel count and channel
data storage type.  It owns one input buffer per frame, the spline workspaces
and the output images; a call copies the frames in, replays a CUDA graph and
returns the images (cubic interpolation, summed over transmits and receives,
the 'tx_and_rx' image of each beamformer).  The graph holds either two
launches -- the batched prefilter and the persistent delay-and-sum of
pycbf_gb_batch_run, every frame's tiles taken from one queue -- or every
frame's own single-frame launches (the staged kernel for Tabbed frames with a
plan) on a few concurrent branches.

The form and its launch shape -- branches, pixel tiles per work item, work
order, transmits held in registers per chunk, CTAs per SM -- are chosen by
``autotune``: a coordinate search timed with CUDA events on the batch
itself, cached per batch signature for the life of the process.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass
from typing import Sequence

import numpy as np
import torch

from . import _lib
from .beamformers import BeamformerException, SyntheticBeamformer, TabbedBeamformer

__all__ = ["BatchBeamformer", "BatchConfig", "beamformers_for", "assign_branches"]


@dataclass(frozen=True)
class BatchConfig:
    tiles_per_item: int = 1      # 128-pixel tiles per work item
    order: int = 1               # 0 frame order, 1 largest estimated cost first
    tx_chunk: int = 12           # transmits per register chunk (4, 8, 12); 0: the single-frame body
    ctas_per_sm: int = 4         # CTAs of 128 threads per SM serving the queue
    branches: int = 0            # > 0: instead of the queue, each frame's own single-frame
                                 # launches, on this many concurrent graph branches


# the queue form's own fields first, the branch counts last, so that both forms
# are searched before one of them wins the coordinate search
SEARCH_SPACE = dict(tx_chunk=(12, 0, 8, 4), tiles_per_item=(1, 2, 4), order=(1, 0),
                    ctas_per_sm=(4, 5, 3, 2), branches=(0, 4, 8, 16))
_TUNED: dict = {}


def _ptr(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else None


def assign_branches(costs: Sequence[float], nbranch: int) -> list:
    """Branch of each group: largest cost first onto the least loaded branch
    (ties to the lowest branch index)."""
    load = [0.0] * nbranch
    out = [0] * len(costs)
    for g in sorted(range(len(costs)), key=lambda g: -costs[g]):
        b = min(range(nbranch), key=lambda i: load[i])
        load[b] += costs[g]
        out[g] = b
    return out


def _stream():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


class BatchBeamformer:
    """Many frames of many beamformers per launch; see the module docstring."""

    def __init__(self, beamformers: Sequence, config: BatchConfig | None = None,
                 autotune: bool = True):
        if not beamformers:
            raise BeamformerException("a batch needs at least one beamformer")
        self._lib = _lib.load()
        self.beamformers = list(beamformers)
        self.n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        self.inputs, self.outputs, self._coef, jobs = [], [], [], []
        self._keep = []
        for bf in self.beamformers:
            if not isinstance(bf, (TabbedBeamformer, SyntheticBeamformer)):
                raise BeamformerException("batch entries must be Tabbed or Synthetic beamformers")
            if bf._interp_code != _lib.INTERP["cubic"]:
                raise BeamformerException("batched frames use cubic interpolation")
            synth = isinstance(bf, SyntheticBeamformer)
            info = bf._rfinfo(1, bf.ndimp if synth else 0)
            rf = torch.zeros((bf.ntx, bf.nrx, bf.nt), dtype=bf._torch_dtype, device="cuda")
            need = self._lib.pycbf_gb_workspace_bytes(ct.byref(info), _lib.INTERP["cubic"])
            coef = torch.empty(need, dtype=torch.uint8, device="cuda")
            out = torch.empty(bf.nop, dtype=torch.float32, device="cuda")
            j = _lib.BatchJob()
            j.geom = 1 if synth else 0
            j.rf = info
            j.rfdata, j.coef, j.out = _ptr(rf).value, _ptr(coef).value, _ptr(out).value
            j.pixel_index = _ptr(bf._pixel_index).value if bf._pixel_index is not None else None
            if synth:
                j.geo = ct.pointer(bf._geom)
                self._keep.append(j.geo)
            else:
                tautx, apodtx, taurx, apodrx = bf._tables
                j.tautx, j.apodtx = _ptr(tautx).value, _ptr(apodtx).value
                j.taurx, j.apodrx = _ptr(taurx).value, _ptr(apodrx).value
                j.np = bf.nop
                j.thresh = float(np.float32(bf.thresh))
            self.inputs.append(rf)
            self._coef.append(coef)
            self.outputs.append(out)
            jobs.append(j)
        self._jobs = (_lib.BatchJob * len(jobs))(*jobs)
        self.taps = sum(bf.ntx * bf.nrx * bf.nop for bf in self.beamformers)
        self._plans: dict = {}
        self._streams: list = []
        self._graph = None
        if config is None:
            config = self.autotune() if autotune else BatchConfig()
        self.set_config(config)

    # -- plan / run ----------------------------------------------------------
    def signature(self):
        return tuple((type(bf).__name__, bf.storage, bf.ntx, bf.nrx, bf.nt, bf.nop)
                     for bf in self.beamformers)

    def _plan(self, tiles_per_item: int, order: int):
        key = (tiles_per_item, order)
        if key not in self._plans:
            n = len(self._jobs)
            nbytes = self._lib.pycbf_gb_batch_plan_bytes(self._jobs, n, tiles_per_item)
            buf = torch.empty(max(16, nbytes), dtype=torch.uint8, device="cuda")
            info = _lib.BatchInfo()
            st = self._lib.pycbf_gb_batch_plan(self._jobs, n, tiles_per_item, order, _ptr(buf),
                                               nbytes, ct.byref(info), _stream())
            _lib.check(st, "pycbf_gb_batch_plan")
            self._plans[key] = (buf, info)
        return self._plans[key]

    def _launch_frame(self, k: int):
        """Frame k with the single-frame launches of its beamformer (the staged
        kernel for Tabbed frames with a plan), on the current stream."""
        bf = self.beamformers[k]
        rf, coef, out = self.inputs[k], self._coef[k], self.outputs[k]
        L, stream = self._lib, _stream()
        tabbed = isinstance(bf, TabbedBeamformer)
        info = bf._rfinfo(1, 0 if tabbed else bf.ndimp)
        if tabbed:
            tautx, apodtx, taurx, apodrx = bf._tables
            st = L.pycbf_gb_spline_coefficients(ct.byref(info), _ptr(rf), _ptr(coef), coef.numel(),
                                                stream)
            _lib.check(st, "pycbf_gb_spline_coefficients")
            st = L.pycbf_gb_das_tabbed_prefiltered(
                ct.byref(info), _ptr(coef), _ptr(tautx), _ptr(apodtx), _ptr(taurx), _ptr(apodrx),
                bf.nop, _ptr(bf._pixel_index), float(np.float32(bf.thresh)), 3, _ptr(bf._plan),
                _ptr(out), stream)
            _lib.check(st, "pycbf_gb_das_tabbed_prefiltered")
        else:
            st = L.pycbf_gb_das_synthetic(ct.byref(info), _ptr(rf), ct.byref(bf._geom),
                                          _ptr(bf._pixel_index), _lib.INTERP["cubic"], 3, _ptr(out),
                                          _ptr(coef), coef.numel(), stream)
            _lib.check(st, "pycbf_gb_das_synthetic")

    def _run_branches(self, nbranch: int):
        """Every frame's own launches, frames of one beamformer in order on one
        branch (they share its plan), beamformers spread over nbranch streams by
        their taps (largest first onto the least loaded branch)."""
        while len(self._streams) < nbranch:
            self._streams.append(torch.cuda.Stream())
        streams = self._streams[:nbranch]
        groups: dict = {}
        for k, bf in enumerate(self.beamformers):
            groups.setdefault(id(bf), []).append(k)
        members = list(groups.values())
        costs = [sum(self.beamformers[k].ntx * self.beamformers[k].nrx * self.beamformers[k].nop
                     for k in ks) for ks in members]
        branch = assign_branches(costs, nbranch)
        cur = torch.cuda.current_stream()
        fork = torch.cuda.Event()
        fork.record(cur)
        for st in streams:
            st.wait_event(fork)
        for g in sorted(range(len(members)), key=lambda g: -costs[g]):
            with torch.cuda.stream(streams[branch[g]]):
                for k in members[g]:
                    self._launch_frame(k)
        for st in streams:
            join = torch.cuda.Event()
            join.record(st)
            cur.wait_event(join)

    def _run(self, cfg: BatchConfig):
        if cfg.branches > 0:
            self._run_branches(cfg.branches)
            return
        buf, info = self._plan(cfg.tiles_per_item, cfg.order)
        st = self._lib.pycbf_gb_batch_run(_ptr(buf), ct.byref(info), cfg.tx_chunk,
                                          cfg.ctas_per_sm * self.n_sm, _stream())
        _lib.check(st, "pycbf_gb_batch_run")

    def set_config(self, cfg: BatchConfig):
        """Use cfg and capture the CUDA graph of its launches."""
        self.config = cfg
        self._run(cfg)  # warm (plans, attributes) outside the capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._run(cfg)
        self._graph = g

    # -- autotuning ----------------------------------------------------------
    def time_config(self, cfg: BatchConfig, reps: int = 3) -> float:
        self._run(cfg)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            self._run(cfg)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def autotune(self, reps: int = 3, space: dict | None = None) -> BatchConfig:
        """Coordinate search over SEARCH_SPACE (one parameter at a time, twice
        around), timing the batch itself; results cached per signature."""
        sig = self.signature()
        if sig in _TUNED:
            self.timings = _TUNED[sig][1]
            return _TUNED[sig][0]
        space = space or SEARCH_SPACE
        # with branches the queue's fields do not apply: one config per branch count
        canon = lambda c: BatchConfig(branches=c.branches) if c.branches > 0 else c
        best = BatchConfig()
        best_t = self.time_config(best, reps)
        timings = {best: best_t}
        for _ in range(2):
            for name, values in space.items():
                for v in values:
                    cand = canon(BatchConfig(**{**best.__dict__, name: v}))
                    if cand not in timings:
                        timings[cand] = self.time_config(cand, reps)
                    if timings[cand] < best_t:
                        best, best_t = cand, timings[cand]
        _TUNED[sig] = (best, timings)
        self.timings = timings
        return best

    def launches_per_replay(self) -> int:
        """Kernel launches in one replay of the graph: the batched prefilter and
        the persistent delay-and-sum (queue form), or every frame's own spline
        prefilter and delay-and-sum (branch form)."""
        return 2 if self.config.branches == 0 else 2 * len(self.beamformers)

    # -- use -----------------------------------------------------------------
    def replay(self):
        """Beamform what the input buffers hold (no copies)."""
        self._graph.replay()

    def __call__(self, frames: Sequence, out_as_numpy: bool = False):
        if len(frames) != len(self.inputs):
            raise BeamformerException(f"expected {len(self.inputs)} frames, got {len(frames)}")
        for dst, src, bf in zip(self.inputs, frames, self.beamformers):
            t = src if isinstance(src, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(src))
            if tuple(t.shape) != tuple(dst.shape):
                raise BeamformerException(f"frame shape {tuple(t.shape)} != {tuple(dst.shape)}")
            dst.copy_(t.to(device="cuda", dtype=dst.dtype, non_blocking=True))
        self.replay()
        if out_as_numpy:
            return [o.cpu().numpy() for o in self.outputs]
        return self.outputs


def beamformers_for(frames, storage: str = "float32"):
    """Beamformers for phantom.batch_frames entries (cubic, 'tx_and_rx')."""
    out = []
    for f in frames:
        common = dict(t0=f["t0"], dt=f["dt"], nt=f["nt"], interp={"kind": "cubic"},
                      storage=storage)
        if f["kind"] == "tabbed":
            out.append(TabbedBeamformer(tautx=f["tautx"], apodtx=f["apodtx"], taurx=f["taurx"],
                                        apodrx=f["apodrx"], **common))
        else:
            g = f["geometry"]
            out.append(SyntheticBeamformer(ovectx=g["ovectx"], nvectx=g["nvectx"],
                                           doftx=g["doftx"], alatx=g["alatx"], t0tx=g["t0tx"],
                                           ovecrx=g["ovecrx"], nvecrx=g["nvecrx"],
                                           alarx=g["alarx"], c0=g["c0"], pnts=g["pnts"], **common))
    return out

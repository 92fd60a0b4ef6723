#!/usr/bin/env python
"""Benchmark of the beamforming hot path: pixel x tx x rx samples per second.

Workload (the plain Tabbed DAS, FP32, cubic configuration): 128-element linear
array at 0.3 mm pitch, 11 plane waves over -10..+10 deg, fs 25 MHz, Nt 2048,
c 1540 m/s, seeded channel data (20 points + 5000 speckle, 5 MHz pulse at 60 %
bandwidth, -40 dB noise), 256 x 512 pixel grid; tautx/taurx from the
plane-wave geometry, apodtx ones, apodrx Hann inside an F#1.5 mask.
One step = one frame: spline prefilter + delay-and-sum (two kernel launches).

  value     device-resident throughput (inputs already in HBM), L2 flushed
            (256 MiB write) before every step, CUDA events on the launch stream
  e2e       the same through the public API (TabbedBeamformer.__call__) from
            pinned host memory: H2D of the frame, kernels, D2H of the image
  roofline  the delay-and-sum kernel: algorithmic bytes (0.855 B/tap: tables,
            channel data and image) over its event-timed duration, against the
            measured HBM copy bandwidth; an FP32 roofline beside it
  cpu_baseline  the CPU oracle (a float32 restatement of the reference's C
            path) or the reference's own compiled C, all host cores, ~10 s

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) each rank beamforms its own frames on its own GPU (the
path shards by frame with no exchange); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as ct
import json
import re
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DAS pixel×tx×rx samples/s at ≤1e-3 rel-L2; batched/fp16 & fwd+adj vs plain"
UNIT = "samples/s"
BYTES_PER_TAP_NOTE = "tables 145.8 MB + channel data 11.5 MB + image 0.5 MB per frame"
WORKLOAD = "tabbed_das_fp32_cubic_128el_11pw_2048s_256x512"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--variants", default="all",
                    help="comma list of secondary groups to run: batch8, adjoint, batch64, "
                         "synthetic, tables, demod, ingest (default all)")
    ap.add_argument("--pixel-order", default="auto", choices=["auto", "natural"])
    return ap.parse_args()


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(x: float, device) -> float:
    """The largest x over the ranks of the process group (x itself when there
    is no group or one rank): the slowest replica's time."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_rate(world: int, units_per_rank: float, seconds: float) -> float:
    """Whole-job throughput of `world` replicas, each processing units_per_rank,
    timed by the slowest one (weak scaling)."""
    return world * units_per_rank / seconds


def tabbed_workload(device):
    from pycbf_gb300 import phantom
    return phantom.linear_pw_tabbed(device=device)


def taps_of(w):
    return w.tautx.shape[0] * w.taurx.shape[0] * w.tautx.shape[1]


def algorithmic_bytes(w):
    ntx, np_ = w.tautx.shape
    nrx = w.taurx.shape[0]
    return 4 * (2 * (ntx + nrx) * np_ + ntx * nrx * w.nt + np_)


def fp64_columns(w, cols, dev):
    """Float64 'tx_and_rx' image of the Tabbed workload at the pixel columns
    `cols`: the natural cubic spline of every channel solved in float64, each
    tap decided as the float32 C path decides it (|fl(apodtx apodrx)| >=
    0.01, t0 <= fl(tautx + taurx) <= fl(t0 + fl(dt (nt-1)))) and evaluated at
    the float64 delay sum.  The accuracy yardstick of the FP64 errors below
    (pycbf/cpu/pycbf.c:68-166 and 179-207 carried out in double)."""
    import numpy as np
    import torch
    f64 = torch.float64
    rf = torch.as_tensor(w.rf, device=dev, dtype=f64)
    ntx, nrx, nt = rf.shape
    y = rf.reshape(-1, nt).T                                        # (nt, nch)
    # natural spline: 0.5 z_i-1 + 2 z_i + 0.5 z_i+1 = (y_i+1 - 2 y_i + y_i-1) / 2, z = y'' dt^2 / 6,
    # solved on the host by the Thomas algorithm (all channels at once)
    yh = np.asarray(w.rf, dtype=np.float64).reshape(-1, nt).T
    d = 0.5 * (yh[2:] - 2.0 * yh[1:-1] + yh[:-2])
    n = nt - 2
    cp = np.empty(n)
    dp = np.empty_like(d)
    cp[0], dp[0] = 0.25, d[0] / 2.0
    for i in range(1, n):
        m = 2.0 - 0.5 * cp[i - 1]
        cp[i] = 0.5 / m
        dp[i] = (d[i] - 0.5 * dp[i - 1]) / m
    zh = np.zeros_like(yh)
    zh[n] = dp[n - 1]
    for i in range(n - 2, -1, -1):
        zh[i + 1] = dp[i] - cp[i] * zh[i + 2]
    z = torch.as_tensor(zh, device=dev)
    yz = torch.stack([y.T.reshape(ntx, nrx, nt), z.T.reshape(ntx, nrx, nt)])
    t32 = lambda a: torch.as_tensor(np.ascontiguousarray(a[:, cols]), device=dev)
    ttx, atx, trx, arx = t32(w.tautx), t32(w.apodtx), t32(w.taurx), t32(w.apodrx)
    t0 = np.float32(w.t0)
    xmax = np.float32(t0 + np.float32(np.float32(w.dt) * np.float32(nt - 1)))
    x32 = ttx[:, None, :] + trx[None, :, :]                          # float32 sums, as the C path
    ok = ((atx[:, None, :] * arx[None, :, :]).abs() >= np.float32(0.01)) & (x32 >= float(t0)) \
        & (x32 <= float(xmax))
    q = ((ttx.to(f64)[:, None, :] + trx.to(f64)[None, :, :]) - float(t0)) / float(np.float32(w.dt))
    j = torch.clamp(torch.floor(q), 0, nt - 2).long()
    a, b = (j + 1) - q, q - j
    ti = torch.arange(ntx, device=dev)[:, None, None]
    ri = torch.arange(nrx, device=dev)[None, :, None]
    g = lambda k, jj: yz[k][ti, ri, jj]
    s = a * g(0, j) + b * g(0, j + 1) + (a ** 3 - a) * g(1, j) + (b ** 3 - b) * g(1, j + 1)
    apod = atx.to(f64)[:, None, :] * arx.to(f64)[None, :, :]
    return torch.where(ok, apod * s, torch.zeros_like(s)).sum((0, 1))


# Algorithmic work per unit (fixed here, used by every roofline entry):
#   bytes: the compulsory traffic of one call -- delay/apodization tables (Tabbed,
#          float32, read once), channel data in its storage type (read once per
#          frame), pixel coordinates (Synthetic, float32), images (float32, written
#          once); intermediates are not counted
#   FLOPs: 20 per contributing cubic tap + 2 per tap (weight product and threshold),
#          + 13 per (transmit, pixel) and (receive, pixel) delay of the Synthetic
#          geometry (distance, projection, square root, division), + 3 per (pixel,
#          receive) for DMAS (signed root, two multiply-adds), + for SLSC per pixel
#          2 K sum_m (nrx - m) for the lag products and 4 K nrx for the per-element
#          means and norms over the K = 2 nkern + 1 sample kernel; the adjoint adds
#          26 per contributing tap (interpolation transpose and delay derivative) +
#          2 per tap.
def roofline_of(seconds, alg_bytes, flops, hbm_peak, fp32_peak, kernel, note=""):
    t_hbm, t_fp32 = alg_bytes / (hbm_peak * 1e9), flops / (fp32_peak * 1e12)
    out = {"bound": "hbm" if t_hbm >= t_fp32 else "fp32",
           "hbm": {"achieved_gbs": alg_bytes / seconds / 1e9,
                   "frac": alg_bytes / seconds / 1e9 / hbm_peak},
           "fp32": {"achieved_tflops": flops / seconds / 1e12,
                    "frac": flops / seconds / 1e12 / fp32_peak},
           "algorithmic_bytes": int(alg_bytes), "flops": int(flops), "kernel": kernel}
    out["frac"] = out["hbm"]["frac"] if out["bound"] == "hbm" else out["fp32"]["frac"]
    if note:
        out["note"] = note
    return out


def das_flops(contrib, taps, delays=0, extra=0):
    return 20 * contrib + 2 * taps + 13 * delays + extra


def rel_l2_t(a, b) -> float:
    import torch
    a, b = torch.as_tensor(a).double().ravel(), torch.as_tensor(b).double().ravel().to(a.device)
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


# ---------------------------------------------------------------------------
# CPU side
# ---------------------------------------------------------------------------
def cpu_baseline(w, seconds):
    from oracle import oracle
    threads = max(1, len(os.sched_getaffinity(0)))
    kind = "port"
    use_ref = False
    if oracle.ref_lib() is not None:
        kind, use_ref = "reference", True
    taps = taps_of(w)
    args = (w.rf, w.tautx, w.apodtx, w.taurx, w.apodrx, w.t0, w.dt, w.nt)
    n = 0
    t = time.perf_counter()
    while True:
        oracle.das_tabbed(*args, interp="cubic", threads=threads, use_ref=use_ref)
        n += 1
        el = time.perf_counter() - t
        if el >= seconds:
            break
    return {"value": taps * n / el, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{n} full frames of the workload ({taps} taps each) in {el:.1f} s, "
                      f"{'reference pycbf.c per channel' if use_ref else 'oracle'}, "
                      f"{threads} threads over transmits"}


def run_reference_arm(a):
    rank, world, _ = rank_info()
    if rank != 0:
        return
    w = tabbed_workload("cpu")
    from oracle import oracle
    threads = max(1, len(os.sched_getaffinity(0)))
    use_ref = oracle.ref_lib() is not None
    kind = "reference" if use_ref else "port"
    args = (w.rf, w.tautx, w.apodtx, w.taurx, w.apodrx, w.t0, w.dt, w.nt)
    run = lambda: oracle.das_tabbed(*args, interp="cubic", threads=threads, use_ref=use_ref)
    for _ in range(a.warmup):
        run()
    times = []
    for _ in range(a.steps):
        t = time.perf_counter()
        run()
        times.append(time.perf_counter() - t)
    total = sum(times)
    taps = taps_of(w)
    value = taps * a.steps / total
    cores = threads
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * total / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded phantom)",
        "config": {"workload": WORKLOAD, "global_batch": 1, "frames_per_step": 1},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"one full frame per step ({taps} taps), "
                                   f"{'reference pycbf.c' if use_ref else 'CPU oracle restating pycbf.c'}, "
                                   f"{threads} threads over transmits"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.file.flush()
        rows = []
        with open(self.file.name) as fp:
            for line in fp:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def main_ours(a):
    import torch
    import torch.distributed as dist

    import pycbf_gb300 as pg
    from pycbf_gb300 import _lib

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    L = _lib.load()

    w = tabbed_workload(dev)
    taps = taps_of(w)
    bf = pg.TabbedBeamformer(tautx=w.tautx, taurx=w.taurx, apodtx=w.apodtx, apodrx=w.apodrx,
                             t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": "cubic"},
                             pixel_order=a.pixel_order)
    cnt, _ = bf.tap_census()
    n_contrib = int(cnt.sum().item())
    rf = torch.as_tensor(w.rf, device=dev).contiguous()
    info = bf._rfinfo(None)
    ws, nws = bf._workspace_for(info)
    out = torch.empty(bf.nop, device=dev)
    tautx, apodtx, taurx, apodrx = bf._tables
    pidx = ct.c_void_p(bf._pixel_index.data_ptr()) if bf._pixel_index is not None else None
    P = lambda t: ct.c_void_p(t.data_ptr())
    args_spline = (ct.byref(info), P(rf), P(ws), nws)
    plan = ct.c_void_p(bf._plan.data_ptr()) if bf._plan is not None else None
    args_das = (ct.byref(info), P(ws), P(tautx), P(apodtx), P(taurx), P(apodrx), bf.nop, pidx,
                ct.c_float(0.01), 3, plan, P(out))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > L2
    stream = torch.cuda.current_stream()
    sp = ct.c_void_p(stream.cuda_stream)

    def step(ev):
        flush.zero_()
        ev[0].record(stream)
        _lib.check(L.pycbf_gb_spline_coefficients(*args_spline, sp), "spline")
        ev[1].record(stream)
        _lib.check(L.pycbf_gb_das_tabbed_prefiltered(*args_das, sp), "das")
        ev[2].record(stream)

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(a.steps)]
    for _ in range(a.warmup):
        step(evs[0])
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    for k in range(a.steps):
        step(evs[k])
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    spline_ms = [e[0].elapsed_time(e[1]) for e in evs]
    das_ms = [e[1].elapsed_time(e[2]) for e in evs]
    total_ms = max_over_ranks(sum(s + d for s, d in zip(spline_ms, das_ms)), dev)
    value = replicas_rate(world, taps * a.steps, total_ms * 1e-3)

    # end to end through the public API, pinned host input, numpy output
    rf_host = torch.from_numpy(w.rf).pin_memory()
    for _ in range(max(1, a.warmup)):
        bf(rf_host)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t = time.perf_counter()
    for _ in range(a.steps):
        img = bf(rf_host)
    e2e_s = max_over_ranks(time.perf_counter() - t, dev)
    e2e = {"value": replicas_rate(world, taps * a.steps, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": int(rf_host.numel() * rf_host.element_size()),
           "d2h_bytes_per_step": int(img.size * img.itemsize),
           "ms_per_step": 1e3 * e2e_s / a.steps}

    # the same frames through beamform_stream: each frame's host-to-device copy and
    # its image's device-to-host copy overlap the neighbouring frames' beamforms
    for _ in bf.beamform_stream([rf_host] * max(1, a.warmup)):
        pass
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t = time.perf_counter()
    imgs = list(bf.beamform_stream([rf_host] * a.steps))
    es = max_over_ranks(time.perf_counter() - t, dev)
    e2e_stream = {"value": replicas_rate(world, taps * a.steps, es), "unit": UNIT,
                  "h2d_bytes_per_step": int(rf_host.numel() * rf_host.element_size()),
                  "d2h_bytes_per_step": int(imgs[-1].size * imgs[-1].itemsize),
                  "ms_per_step": 1e3 * es / a.steps,
                  "api": "TabbedBeamformer.beamform_stream: a sequence of host frames, copies "
                         "of neighbouring frames overlapped with the beamform"}

    # roofline of the delay-and-sum kernel
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fp:
            peaks = json.load(fp)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    das_s = statistics.mean(das_ms) * 1e-3
    alg_bytes = algorithmic_bytes(w)
    achieved = alg_bytes / das_s / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": None,
                "kernel": ("das_staged_kernel<cubic, tx_and_rx, f32>" if bf._plan is not None
                           else "das_kernel<tabbed, cubic, tx_and_rx, f32>"),
                "kernel_ms": 1e3 * das_s, "spline_ms": statistics.mean(spline_ms),
                "peak_source": "measured" if peaks.get("hbm_gbs") else "fallback",
                "algorithmic_bytes": alg_bytes}
    # DRAM bytes and warp instructions of one launch from the committed ncu summary
    # of this kernel and workload; the kernel is issue-bound, so the share of the
    # schedulers' issue slots it uses is reported beside the HBM fraction
    prof = os.path.join(ROOT, "profiles", "das_tabbed_cubic_11x128x2048.md")
    if os.path.exists(prof):
        with open(prof) as fp:
            text = fp.read()
        m = re.search(r"dram bytes per launch \(read \+ write\): (\d+)", text)
        if m:
            roofline["traffic"] = int(m.group(1))
        m = re.search(r"\| smsp__inst_executed\.sum \| ([0-9.]+) M \|", text)
        sm_mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
        if m and sm_mhz:
            n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
            slots = 4 * n_sm * sm_mhz * 1e6 * das_s
            roofline["issue"] = {"warp_instructions": float(m.group(1)) * 1e6,
                                 "frac": float(m.group(1)) * 1e6 / slots,
                                 "note": "instructions from the profile, one issue per scheduler "
                                         "per cycle at the sampled SM clock"}
    # FP32 roofline: algorithmic FLOPs (20 per contributing cubic tap, 2 per tap for the
    # weight product and threshold) over the kernel time, against the FMA probe
    probe_out = torch.empty(152 * 8 * 256, device=dev)
    iters = 4096
    L.pycbf_gb_fp32_probe(P(probe_out), 152 * 8, iters, sp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    L.pycbf_gb_fp32_probe(P(probe_out), 152 * 8, iters, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    fp32_peak = 152 * 8 * 256 * iters * 16 / (e0.elapsed_time(e1) * 1e-3) / 1e12
    flops = 20 * n_contrib + 2 * taps
    fp32 = {"achieved": flops / das_s / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": flops / das_s / 1e12 / fp32_peak, "flops_per_launch": flops,
            "contributing_taps": n_contrib, "peak_source": "measured (FMA probe)"}

    # float64 yardstick on 512 seeded pixels of the workload
    import numpy as np
    cols = np.sort(np.random.default_rng(2).choice(bf.nop, 512, replace=False))
    f64 = fp64_columns(w, cols, dev)
    fp64_plain = rel_l2_t(torch.as_tensor(np.asarray(img, np.float64)[cols], device=dev), f64)
    roofline["fp64_rel_l2"] = fp64_plain

    ctx = {"hbm_peak": hbm_peak, "fp32_peak": fp32_peak, "cols": cols, "f64": f64,
           "contrib": n_contrib}
    variants = {}
    if not a.no_variants:
        variants = run_variants(a, w, dev, taps, ctx)
        for k in ("demod_256x512", "demod_512x1024"):
            if k in variants:
                variants[k]["iq_fp32_frac"] = variants[k]["iq_tflops"] / fp32_peak

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": total_ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded phantom, 20 points + 5000 speckle)",
        "config": {"workload": WORKLOAD, "global_batch": world, "frames_per_step": 1,
                   "interp": "cubic", "pixel_order": a.pixel_order,
                   "l2": "flushed (256 MiB write) before each step",
                   "parallelism": f"replicas x{world}"},
        "e2e": e2e, "e2e_stream": e2e_stream, "roofline": roofline, "fp32_roofline": fp32,
        "gpu_launches": 2 * a.steps, "clocks": clk,
        "wall_s_timed": t_wall, "variants": variants,
    }
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, a.cpu_seconds)
    # the target numbers in one compact key, last on the line: the plain FP32
    # forward, the batched FP16-storage forward and the forward + adjoint in
    # samples/s, their ratios to the plain forward and their FP64 errors
    tg = {"plain_fp32": {"value": value, "fp64_rel_l2": fp64_plain,
                         "hbm_frac": roofline["frac"], "fp32_frac": fp32["frac"]}}
    for key in ("fp16_batch8", "fwd_adj_tabbed"):
        v = variants.get(key)
        if v:
            tg[key] = {"value": v["value"], "vs_plain": v["value"] / value,
                       "fp64_rel_l2": v.get("fp64_rel_l2")}
    line["target_summary"] = tg
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def run_variants(a, w, dev, taps, ctx):
    """Secondary lines: batched frames with FP16/BF16 storage, and nearest."""
    import numpy as np
    import torch

    import pycbf_gb300 as pg
    res = {}
    want = (lambda g: True) if a.variants == "all" else (lambda g: g in a.variants.split(","))
    nfr = 8
    rng = np.random.default_rng(0)
    scales = [1.0] + [float(np.float32(rng.uniform(0.5, 1.5))) for _ in range(nfr - 1)]
    frames = np.stack([w.rf] + [w.rf * np.float32(sc) for sc in scales[1:]])
    hbm, fp32p, cols, f64 = ctx["hbm_peak"], ctx["fp32_peak"], ctx["cols"], ctx["f64"]
    ntx, nrx, nt = w.rf.shape
    np_ = w.tautx.shape[1]
    table_bytes = 4 * 2 * (ntx + nrx) * np_
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    batch8 = (("fp32_batch8", "float32", "cubic", nfr), ("fp16_batch8", "float16", "cubic", nfr),
              ("bf16_batch8", "bfloat16", "cubic", nfr), ("nearest_fp32", "float32", "nearest", 1))
    for name, storage, kind, nf in batch8 if want("batch8") else ():
        bf = pg.TabbedBeamformer(tautx=w.tautx, taurx=w.taurx, apodtx=w.apodtx, apodrx=w.apodrx,
                                 t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": kind}, storage=storage)
        x = torch.as_tensor(frames[:nf] if nf > 1 else w.rf, device=dev).to(
            {"float32": torch.float32, "float16": torch.float16, "bfloat16": torch.bfloat16}[storage])
        out = torch.empty(bf._out_shape(nf if nf > 1 else None), device=dev)
        for _ in range(3):
            bf(x, out_as_numpy=False, buffer=out)
        times = []
        for _ in range(max(3, a.steps // 2)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            bf(x, out_as_numpy=False, buffer=out)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
        t = statistics.mean(times)
        res[name] = {"value": taps * nf / t, "unit": UNIT,
                     "ms_per_call": 1e3 * t, "frames_per_call": nf,
                     "storage": storage, "interp": kind, "launches_per_call": 2}
        if kind == "cubic":
            nbytes = table_bytes + nf * (ntx * nrx * nt * x.element_size() + 4 * np_)
            res[name]["roofline"] = roofline_of(
                t, nbytes, nf * das_flops(ctx["contrib"], taps), hbm, fp32p,
                "das_staged_kernel (frame, tile) items + spline_coef_kernel")
            o = out.reshape(nf, -1)[:, torch.as_tensor(cols, device=dev)]
            errs = [rel_l2_t(o[k], scales[k] * f64) for k in range(nf)]
            res[name]["fp64_rel_l2"] = max(errs)
            res[name]["fp64_rel_l2_note"] = "max over the frames, 512 seeded pixels"
    for group, fn in (("adjoint", lambda: run_adjoint_variants(a, w, dev, taps, ctx)),
                      ("batch64", lambda: run_batch_variants(a, dev, ctx)),
                      ("synthetic", lambda: run_synthetic_variants(a, dev, ctx)),
                      ("tables", lambda: run_table_variant(a, dev)),
                      ("demod", lambda: run_demod_variant(a, dev)),
                      ("ingest", lambda: run_ingest_variant(a, w, dev, taps))):
        if want(group):
            res.update(fn())
    return res


def run_ingest_variant(a, w, dev, taps):
    """The headline workload fed int16 channel data (the phantom quantised to
    +-30000 counts): device time with the counts resident (the spline
    prefilter converts them), and end to end through TabbedBeamformer.__call__
    from pinned int16 host memory (half the host-to-device bytes of float32)."""
    import numpy as np
    import torch

    import pycbf_gb300 as pg
    rf = np.asarray(w.rf, np.float64)
    rfi = np.round(rf / np.abs(rf).max() * 30000).astype(np.int16)
    bf = pg.TabbedBeamformer(tautx=w.tautx, taurx=w.taurx, apodtx=w.apodtx, apodrx=w.apodrx,
                             t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": "cubic"})
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    x = torch.as_tensor(rfi, device=dev)
    out = torch.empty(bf._out_shape(None), device=dev)
    for _ in range(3):
        bf(x, out_as_numpy=False, buffer=out)
    times = []
    for _ in range(max(3, a.steps)):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bf(x, out_as_numpy=False, buffer=out)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    host = torch.from_numpy(rfi).pin_memory()
    for _ in range(3):
        bf(host)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(a.steps):
        img = bf(host)
    e2e_s = (time.perf_counter() - t) / a.steps
    return {"int16_ingest": {"value": taps / statistics.mean(times), "unit": UNIT,
                             "ms_per_call": 1e3 * statistics.mean(times), "storage": "int16 -> float32 records",
                             "e2e": {"value": taps / e2e_s, "unit": UNIT, "ms_per_step": 1e3 * e2e_s,
                                     "h2d_bytes_per_step": int(rfi.nbytes),
                                     "d2h_bytes_per_step": int(img.nbytes)}}}


def run_demod_variant(a, dev):
    """IQ demodulation of beamformed images (the examples' fft_tukey_demod,
    1-9 MHz band, Tukey 0.25) and the B-mode display chain (envelope,
    99th percentile, log compression), on the 256 x 512 image of the
    workload's grid (z 5..45 mm) and on a 512 x 1024 image of the same extent.
    FLOPs: 4 per (line, input sample, output sample) of the complex matrix."""
    import numpy as np
    import torch

    from pycbf_gb300.demod import Demodulator
    res = {}
    stream = torch.cuda.current_stream()
    for name, nx, nz in (("demod_256x512", 256, 512), ("demod_512x1024", 512, 1024)):
        dz = 40e-3 / (nz - 1)
        d = Demodulator(nz, 2 * 1e6 / 1540.0, 2 * 9e6 / 1540.0, 1 / dz)
        img = torch.as_tensor(np.random.default_rng(nz).standard_normal((nx, nz)).astype(np.float32),
                              device=dev)
        t, api = {}, {}
        for what, fn in (("iq", lambda: d.iq(img)), ("bmode", lambda: d.bmode(img))):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            # device time: the call captured once in a CUDA graph, replayed
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                fn()
            for _ in range(3):
                g.replay()
            ms, ms_api = [], []
            for _ in range(10):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                g.replay()
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
                # through the Python API (host launch overhead included)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                ms_api.append(e0.elapsed_time(e1))
            t[what], api[what] = statistics.median(ms), statistics.median(ms_api)
        flops = 4 * nx * nz * d.M
        res[name] = {"iq_us": 1e3 * t["iq"], "bmode_us": 1e3 * t["bmode"],
                     "iq_api_us": 1e3 * api["iq"], "bmode_api_us": 1e3 * api["bmode"],
                     "lines": nx, "samples_in": nz, "samples_out": d.M, "flops": flops,
                     "iq_tflops": flops / (t["iq"] * 1e-3) / 1e12,
                     "launches_bmode": 2 if nx * d.M <= (1 << 18) else 8,
                     "timing": "CUDA graph replay; *_api_us: eager Python calls"}
    return res


def run_table_variant(a, dev):
    """The workload's tables (11 plane waves, 128 elements, 256 x 512 pixels,
    Hann-weighted F#1.5 receive mask) built on the GPU, against the same
    float64 NumPy build on the host plus its copy to the device."""
    import numpy as np
    import torch

    from pycbf_gb300 import helpers
    from pycbf_gb300.tables import make_tabs_and_apods_2d
    xele = helpers.element_positions(128, 0.3e-3)
    steers = np.radians(np.linspace(-10, 10, 11))
    xout, zout = np.linspace(-19e-3, 19e-3, 256), np.linspace(5e-3, 45e-3, 512)
    build = lambda: make_tabs_and_apods_2d(steers, 0.0, 1540.0, 1540.0, xele, xout, zout, 1.5,
                                           hann=True, device=dev)
    build()
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        build()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    t = time.perf_counter()
    tx, _ = helpers.pw_tx_tables(steers, 1540.0, 1540.0, xele, xout, zout)
    rx, ap = helpers.rx_tables(1540.0, xele, xout, zout, 1.5, hann=True)
    host = [torch.as_tensor(v.astype(np.float32)).to(dev) for v in (tx, rx, ap)]
    torch.cuda.synchronize()
    host_s = time.perf_counter() - t
    nbytes = 4 * (2 * 11 + 2 * 128) * 256 * 512
    return {"tables_11pw_128el_256x512": {
        "gpu_ms": statistics.median(times), "host_numpy_and_copy_ms": 1e3 * host_s,
        "table_bytes": nbytes,
        "gpu_write_gbs": nbytes / (statistics.median(times) * 1e-3) / 1e9}}


def _synthetic(cls, w, **kw):
    g = w.geometry
    keys = ("ovectx", "nvectx", "doftx", "alatx", "t0tx", "ovecrx", "nvecrx", "alarx", "c0", "pnts")
    return cls(**{k: g[k] for k in keys}, t0=w.t0, dt=w.dt, nt=w.nt, **kw)


def run_synthetic_variants(a, dev, ctx):
    """Synthetic-point workloads with delays computed on the fly.

    synthetic_*: 192 elements at 0.2 mm, 75 plane waves over -18..18 deg (far
    virtual sources), fs 31.25 MHz, Nt 4096, 40 000 speckle + 30 points,
    512 x 1024 pixels: DAS, DMAS (signed square root over all receive
    pairs, fused) and SLSC (lags 1..16, axial kernel 7 pixels = 1 wavelength).
    matrix_3d_fp16: 32 x 32 matrix, 25 diverging waves, Nt 2048, float16 channel
    data, 128 x 128 x 256 voxels, 8 frames per call (2 000 speckle + 50
    points: the content does not change the work)."""
    import numpy as np
    import torch

    import pycbf_gb300 as pg
    from pycbf_gb300 import phantom
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    res = {}
    w = phantom.linear_pw_synthetic(device=dev)
    rf = torch.as_tensor(w.rf, device=dev)
    nx, nz = w.grid
    cub = {"kind": "cubic"}
    nrx = w.geometry["ovecrx"].shape[0]
    cases = {
        "synthetic_das": _synthetic(pg.SyntheticBeamformer, w, interp=cub, sumtype="tx_and_rx"),
        "synthetic_dmas": _synthetic(pg.SyntheticDMASBeamformer, w, interp=cub,
                              lags=np.arange(1, nrx), lagaxis="rx", sumlags=True, dmastype="ssr"),
        "synthetic_slsc": _synthetic(pg.SyntheticSLSCBeamformer, w, interp=cub, grid_shape=(nx, nz),
                              nlag=16, nkern=3),
    }
    hbm, fp32p = ctx["hbm_peak"], ctx["fp32_peak"]
    contrib = int(cases["synthetic_das"].tap_census()[0].sum().item())
    ntx, nrx, np_ = 75, nrx, nx * nz
    io_bytes = rf.numel() * 4 + 4 * 2 * np_ + 4 * np_       # channel data, pixels, image
    base_flops = das_flops(contrib, ntx * nrx * np_, delays=(ntx + nrx) * np_)
    K = 2 * 3 + 1
    slsc_flops = np_ * (2 * K * sum(nrx - m for m in range(1, 17)) + 4 * K * nrx)
    extra = {"synthetic_das": (0, "das_kernel<synthetic, cubic, tx_and_rx, f32> + spline_coef_kernel"),
             "synthetic_dmas": (3 * np_ * nrx, "das_kernel<synthetic, cubic, dmas_ssr, f32> + "
                                               "spline_coef_kernel (all-pairs sum fused)"),
             "synthetic_slsc": (slsc_flops, "das_kernel<synthetic, cubic, tx_only, f32> + "
                                            "slsc_kernel + spline_coef_kernel")}
    launches = {"synthetic_das": 2, "synthetic_dmas": 2, "synthetic_slsc": 3}
    for name, bf in cases.items():
        call = lambda: bf(rf, out_as_numpy=False)
        call()
        t = _event_time(call, 3, flush, stream)
        taps = bf.ntx * bf.nrx * bf.nop
        add, kern = extra[name]
        res[name] = {"value": taps / t, "unit": UNIT, "ms_per_call": 1e3 * t, "taps": taps,
                     "contributing_taps": contrib, "launches_per_call": launches[name],
                     "workload": "synthetic 192el 75pw 4096s 512x1024", "interp": "cubic",
                     "roofline": roofline_of(t, io_bytes, base_flops + add, hbm, fp32p, kern),
                     "tap_set": "far-virtual-source masks by the cosine compare of the oracle "
                                "(the reference's own acos decision is rounding-dependent there)"}
        del bf
    del rf, w, cases
    torch.cuda.empty_cache()
    w = phantom.matrix_dw_synthetic(n_speckle=2000, device=dev)
    bf = _synthetic(pg.SyntheticBeamformer, w, interp=cub, sumtype="tx_and_rx", storage="float16")
    frames = torch.as_tensor(w.rf, device=dev).to(torch.float16)
    frames = torch.stack([frames * (1.0 + 0.1 * k) for k in range(8)]).contiguous()
    call = lambda: bf(frames, out_as_numpy=False)
    call()
    t = _event_time(call, 2, flush, stream)
    taps = 8 * bf.ntx * bf.nrx * bf.nop
    contrib = 8 * int(bf.tap_census()[0].sum().item())
    np_ = bf.nop
    io_bytes = frames.numel() * 2 + 4 * 3 * np_ + 4 * 8 * np_
    flops = das_flops(contrib, taps, delays=8 * (bf.ntx + bf.nrx) * np_)
    res["matrix_3d_fp16"] = {"value": taps / t, "unit": UNIT, "ms_per_call": 1e3 * t,
                             "frames_per_call": 8, "taps": taps, "contributing_taps": contrib,
                             "storage": "float16", "launches_per_call": 2,
                             "workload": "synthetic 3-D 32x32 matrix 25dw 2048s 128x128x256",
                             "roofline": roofline_of(t, io_bytes, flops, hbm, fp32p,
                                                     "das_kernel<synthetic, cubic, tx_and_rx, f16> "
                                                     "+ spline_coef_kernel")}
    return res


def run_batch_variants(a, dev, ctx):
    """64 seeded uneven frames (ntx 1..75, nrx 64..192, nt 1024..4096, grids
    128x128..512x1024, Tabbed and Synthetic) in one persistent launch replayed
    as a CUDA graph, launch shape autotuned, for float32 / float16 / bfloat16
    channel data; the 16-bit images are compared with the float32 ones."""
    import numpy as np
    import torch

    import pycbf_gb300 as pg
    from pycbf_gb300 import phantom
    from pycbf_gb300.batch import BatchBeamformer, beamformers_for
    frames = phantom.batch_frames(n=64, device=dev)
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    reps = max(3, a.steps // 2)
    res, images32 = {}, None
    contrib = None
    for storage in ("float32", "float16", "bfloat16"):
        t0 = time.perf_counter()
        bb = BatchBeamformer(beamformers_for(frames, storage))
        tune_s = time.perf_counter() - t0
        outs = bb([f["rf"] for f in frames])
        t = _event_time(bb.replay, reps, flush, stream)
        if contrib is None:
            contrib = [int(b.tap_census()[0].sum().item()) for b in bb.beamformers]
        esize = {"float32": 4, "float16": 2, "bfloat16": 2}[storage]
        nbytes, flops = 0, 0
        for b, c in zip(bb.beamformers, contrib):
            ntap = b.ntx * b.nrx * b.nop
            nbytes += b.ntx * b.nrx * b.nt * esize + 4 * b.nop
            if isinstance(b, pg.TabbedBeamformer):
                nbytes += 4 * 2 * (b.ntx + b.nrx) * b.nop
                flops += das_flops(c, ntap)
            else:
                nbytes += 4 * b.ndimp * b.nop
                flops += das_flops(c, ntap, delays=(b.ntx + b.nrx) * b.nop)
        entry = {"value": bb.taps / t, "unit": UNIT, "ms_per_call": 1e3 * t, "frames_per_call": 64,
                 "storage": storage, "taps_per_call": bb.taps,
                 "launches_per_call": bb.launches_per_replay(),
                 "config": bb.config.__dict__, "configs_timed": len(bb.timings),
                 "best_ms_by_form": {
                     "queue (one persistent launch)": min(
                         (v for c, v in bb.timings.items() if c.branches == 0), default=float("nan")),
                     "branches (every frame's own launches)": min(
                         (v for c, v in bb.timings.items() if c.branches > 0), default=float("nan"))},
                 "setup_and_autotune_s": tune_s,
                 "roofline": roofline_of(t, nbytes, flops, ctx["hbm_peak"], ctx["fp32_peak"],
                                         "batch_spline_kernel + batch_das_kernel (queue form) or "
                                         "every frame's spline + delay-and-sum (branch form)"),
                 "kinds": {k: sum(f["kind"] == k for f in frames) for k in ("tabbed", "synthetic")}}
        if storage == "float32":
            images32 = [o.clone() for o in outs]
        else:
            rel = [float(torch.linalg.norm((o - i).double()) / torch.linalg.norm(i.double()))
                   for o, i in zip(outs, images32)]
            entry["rel_l2_vs_float32_per_frame"] = {"median": float(np.median(rel)),
                                                    "max": float(np.max(rel))}
        res[f"batch64_{storage}"] = entry
        del bb, outs
        torch.cuda.empty_cache()
    return res


def _event_time(fn, reps, flush, stream):
    import torch
    times = []
    for _ in range(reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    return statistics.mean(times)


def run_adjoint_variants(a, w, dev, taps, ctx):
    """Forward + adjoint against the plain forward.

    fwd_adj_tabbed: the workload above through the differentiable path,
    gradients with respect to the channel data and both delay tables.
    fwd_adj_sos: the same array and grid as Synthetic beamforming in a
    two-layer medium (1450 m/s to 15 mm, 1560 m/s below), per-element images
    with a slowness per pixel, gradients with respect to the channel data and
    the slowness; plus one optimisation step of a global c + 32 x 64 slowness
    map on the lag-1 coherence + sharpness loss.
    """
    import torch

    import pycbf_gb300 as pg
    from pycbf_gb300 import phantom, sos
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    reps = max(3, a.steps // 2)
    res = {}

    bf = pg.TabbedBeamformer(tautx=w.tautx, taurx=w.taurx, apodtx=w.apodtx, apodrx=w.apodrx,
                             t0=w.t0, dt=w.dt, nt=w.nt, interp={"kind": "cubic"})
    rf = torch.as_tensor(w.rf, device=dev)
    tautx = torch.as_tensor(w.tautx, device=dev)
    taurx = torch.as_tensor(w.taurx, device=dev)
    gout = torch.randn((bf.nop,), device=dev)

    def fwd_tab():
        with torch.no_grad():
            bf.differentiable(rf)

    def fwd_adj_tab():
        r = rf.detach().requires_grad_(True)
        t1, t2 = tautx.detach().requires_grad_(True), taurx.detach().requires_grad_(True)
        bf.differentiable(r, tautx=t1, taurx=t2).backward(gout)

    for _ in range(2):
        fwd_tab(), fwd_adj_tab()
    t_f = _event_time(fwd_tab, reps, flush, stream)
    t_fa = _event_time(fwd_adj_tab, reps, flush, stream)
    ntx, nrx, nt = w.rf.shape
    np_ = bf.nop
    nbytes = (4 * 2 * (ntx + nrx) * np_ + 4 * ntx * nrx * nt + 4 * np_      # forward
              + 4 * np_ + 4 * ntx * nrx * nt + 4 * (ntx + nrx) * np_)      # gout, gradients
    flops = das_flops(ctx["contrib"], taps) + 26 * ctx["contrib"] + 2 * taps
    with torch.no_grad():
        img = bf.differentiable(rf)
    fwd_err = rel_l2_t(img.reshape(-1)[torch.as_tensor(ctx["cols"], device=dev)], ctx["f64"])
    res["fwd_adj_tabbed"] = {"value": taps / t_fa, "unit": UNIT, "ms_per_call": 1e3 * t_fa,
                             "forward_ms": 1e3 * t_f, "forward_value": taps / t_f,
                             "grads": ["rf", "tautx", "taurx"], "interp": "cubic",
                             "sumtype": "tx_and_rx", "fp64_rel_l2": fwd_err,
                             "fp64_rel_l2_note": "the forward image of the differentiable path, "
                                                 "512 seeded pixels; gradients are checked "
                                                 "against float64 autograd in the tests",
                             "roofline": roofline_of(t_fa, nbytes, flops, ctx["hbm_peak"],
                                                     ctx["fp32_peak"],
                                                     "spline + das_staged_kernel + adj_delay_kernel "
                                                     "+ adj_scatter_kernel + adj_finalize_kernel")}

    sw = phantom.two_layer_pw_synthetic(device=dev)
    g = sw.geometry
    sbf = pg.SyntheticBeamformer(ovectx=g["ovectx"], nvectx=g["nvectx"], doftx=g["doftx"],
                                 alatx=g["alatx"], t0tx=g["t0tx"], ovecrx=g["ovecrx"],
                                 nvecrx=g["nvecrx"], alarx=g["alarx"], c0=g["c0"],
                                 pnts=g["pnts"], t0=sw.t0, dt=sw.dt, nt=sw.nt,
                                 interp={"kind": "cubic"}, sumtype="tx_only")
    srf = torch.as_tensor(sw.rf, device=dev)
    staps = sbf.ntx * sbf.nrx * sbf.nop
    model = sos.SlownessModel(sw.grid, map_shape=(32, 64), c_init=1540.0, device=dev)
    mask = sbf.rx_mask()
    s_fixed = model().detach()
    gimg = torch.randn((sbf.nrx, sbf.nop), device=dev)

    def fwd_s():
        with torch.no_grad():
            sbf.differentiable(srf, slowness=s_fixed)

    def fwd_adj_s():
        r = srf.detach().requires_grad_(True)
        s = s_fixed.detach().requires_grad_(True)
        sbf.differentiable(r, slowness=s).backward(gimg)

    opt = torch.optim.Adam(model.parameters(), lr=1e-6)

    def train_step():
        opt.zero_grad(set_to_none=True)
        loss = sos.sos_loss(sbf.differentiable(srf, slowness=model()), mask, sw.grid, nkern=2)
        loss.backward()
        opt.step()

    for _ in range(2):
        fwd_s(), fwd_adj_s(), train_step()
    t_f = _event_time(fwd_s, reps, flush, stream)
    t_fa = _event_time(fwd_adj_s, reps, flush, stream)
    t_tr = _event_time(train_step, reps, flush, stream)
    scontrib = int(sbf.tap_census()[0].sum().item())
    sntx, snrx, snt = sw.rf.shape
    snp = sbf.nop
    s_bytes = (4 * sntx * snrx * snt + 4 * 2 * snp + 4 * snp + 4 * snrx * snp     # forward
               + 4 * snrx * snp + 4 * sntx * snrx * snt + 4 * snp)              # gout, gradients
    s_flops = (das_flops(scontrib, staps, delays=(sntx + snrx) * snp) + 26 * scontrib
               + 2 * staps)
    res["fwd_adj_sos"] = {"value": staps / t_fa, "unit": UNIT, "ms_per_call": 1e3 * t_fa,
                          "forward_ms": 1e3 * t_f, "forward_value": staps / t_f,
                          "train_step_ms": 1e3 * t_tr, "grads": ["rf", "slowness"],
                          "workload": "synthetic two-layer 128el 11pw 2048s 256x512, per-element "
                                      "images, 32x64 slowness map + global c",
                          "interp": "cubic", "sumtype": "tx_only",
                          "roofline": roofline_of(t_fa, s_bytes, s_flops, ctx["hbm_peak"],
                                                  ctx["fp32_peak"],
                                                  "spline + das_kernel<slowness> + adj_delay_kernel "
                                                  "+ adj_scatter_kernel + adj_finalize_kernel")}
    return res


def main():
    a = parse()
    if a.impl == "reference":
        run_reference_arm(a)
    else:
        main_ours(a)


if __name__ == "__main__":
    main()

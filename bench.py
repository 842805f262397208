#!/usr/bin/env python
"""Benchmark of the GB300 CT reconstruction hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step): the parallel-beam drop-in at its headline size -- a
512x512 image at 0.5 mm is forward projected (fp_par_2d, ray-driven) to a
720-view sinogram over pi with 729 bins at 0.5 mm, ramp filtered (par) and
backprojected (bp_par_2d) -- on one slice (batch 1).  Steps cycle through a
pool of distinct seeded phantom slices whose total size exceeds the 129 MB L2,
so every step reads its input from HBM.

Reported: slices/s (value) and pixel-view updates/s; ``e2e`` repeats the
workload through the C ABI with the slice copied from pinned host memory and
the reconstruction read back every step; ``roofline`` is the dominant
kernel's algorithmic FP32 FLOP/s (per-kernel pass below) against the FP32
peak; ``cpu_baseline`` times the oracle port
(the reference's CPU algorithm restated in C) on this host's cores.

``roofline.kernel_ms`` comes from a per-kernel pass after the timed region
(each stage 100 times from a CUDA graph, CUDA events around the replay);
``roofline.hbm`` gives the same kernel's algorithmic bytes against the
measured HBM bandwidth; ``roofline.traffic`` is the ncu DRAM traffic per call
recorded in profiles/ncu_traffic.txt.

``extra`` (``--legs`` selects): ``fan_fbp_config1`` the fan FBP at its
headline size (fan weighting -> ramp(fan) -> bp_fan_2d, 720 x 736 -> 512x512);
``batched_fan_config3`` 64 uneven fan sinograms through one batched plan
against 64 plain calls; ``gd_config4`` gradient descent through the
differentiable forward projector (batch 16); ``lowp_config5`` the 2048^2
fan slice from FP32, BF16 and FP16 sinograms (tensor-core filter), with its
error against the FP64 oracle on image strips when the CPU-baseline leg runs;
``fp_methods`` the parallel forward projector's other methods, ray casting
(512^2 -> 720 x 729, FoV radius 128 mm, 0.125-pixel steps) and distance
driven, beside ray driven; ``helical`` 360LI / 180LI rebinning of a
clinical-size helical scan (736 channels x 64 rows, 1152 views per rotation,
pitch 1, 128 slices) with its algorithmic bytes against the measured HBM
bandwidth and the oracle port beside it; ``adjoints`` the FP32 adjoints of
bp_fan_2d (config 1) and bp_par_2d (config 2) beside their forwards, and the
fan FBP chain's sinogram gradient; ``bp_par_2d_sv`` the single-view
backprojection at config 2 (write-bound) against the HBM bandwidth.

``--impl reference`` times the reference's CPU implementation of the same
workload on this host (the compiled reference when its build is present,
else the oracle port), all host threads, one slice per step.

Under torchrun (N > 1) every rank runs the same workload on its own GPU as an
independent replica (no data exchange); value is the sum over ranks of the
slices processed divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FBP slices/s and pixel-view updates/s at rel-L2<=1e-4 vs FP64; batched vs plain"
SM_COUNT = 152
LEGS = ("fan", "batched", "gd", "lowp", "fpmethods", "helical", "adjoints", "sv")
FP32_LANES_PER_SM = 128


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--pool", type=int, default=160, help="distinct slices cycled through")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--legs", default=",".join(LEGS),
                    help="workloads measured after the headline, reported under extra: a comma "
                         "list of " + ", ".join(LEGS) + " (or 'none')")
    a = ap.parse_args()
    a.legs = set() if a.legs == "none" else set(a.legs.split(","))
    if not a.legs <= set(LEGS):
        ap.error(f"--legs: unknown {sorted(a.legs - set(LEGS))}")
    return a


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, backend):
        import torch
        import torch.distributed as dist
        self.ws, self.rank, self.local = dist_env()
        self.dist = dist if self.ws > 1 else None
        if self.dist:
            dist.init_process_group(backend)
        self.torch = torch

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if not self.dist:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64,
                              device="cuda" if self.dist.get_backend() == "nccl" else "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def replica_value(world: int, steps: int, slowest_secs: float) -> float:
    """Whole-job throughput of N independent replicas: every rank processes
    `steps` units; the job takes as long as its slowest rank."""
    return world * steps / slowest_secs


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 20 ms, each stamped
    on arrival; stop() keeps those inside the timed window."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        t = time.perf_counter()
        while not self.lines and time.perf_counter() - t < 5.0:  # sampling has begun
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, windows=()):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.05)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        inside = [ln for ts, ln in self.lines if any(a <= ts <= b for a, b in windows)]
        lines = inside or [ln for _, ln in self.lines]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm),
                "window": "timed regions" if inside else "whole run"}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def par_geometry():
    from ct_recon_extensions_gb300 import synthetic as syn
    return syn.parallel_config_2()


def fan_geometry():
    from ct_recon_extensions_gb300 import synthetic as syn
    return syn.fan_config_1()


def make_pool(kind, g, n, seed0):
    """n distinct float32 inputs (images for the parallel workload, analytic
    sinograms for the fan workload): 16 seeded phantoms, each item a
    distinct scaled copy."""
    from ct_recon_extensions_gb300 import synthetic as syn
    base = []
    for i in range(16):
        e = syn.random_ellipses(seed0 + i)
        if kind == "par":
            base.append(syn.rasterize(e, g["nx"], g["ny"], g["dx"], g["dy"]))
        else:
            base.append(syn.fan_sinogram(e, g["na"], g["ns"], g["ds"], g["orbit"], g["dso"], g["dsd"]))
    return base


class ParPipeline:
    """fp_par_2d -> ramp(par) -> bp_par_2d through the C ABI on preallocated buffers."""

    def __init__(self, g, device):
        import torch
        from ct_recon_extensions_gb300 import _lib
        from ct_recon_extensions_gb300 import torch_ctrecon as tc
        self.torch = torch
        self.lib = _lib.load()
        self.g = g
        self.fp = tc.ParallelProjection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                            g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                            g["offset_x"], g["offset_y"], g["fov"])
        self.ramp = tc.RampFilterOp(g["ns"], g["na"], g["ds"], -1.0, 0)
        self.bp = tc.ParallelBackprojection2DOp(g["ns"], g["na"], g["ds"], g["orbit"],
                                                g["offset_s"], g["orbit_start"], g["nx"], g["ny"],
                                                g["dx"], g["dy"], g["offset_x"], g["offset_y"],
                                                g["fov"])
        self.fplan = self.fp.plan(device, 1)  # per-geometry ray tables, built once
        self.taps = ctypes.c_void_p(self.ramp.taps(device).data_ptr())
        self.bplan = self.bp.plan(device, 1)  # per-geometry tables, scratch and view constants
        f32 = dict(dtype=torch.float32, device=device)
        self.sino = torch.empty((g["na"], g["ns"]), **f32)
        self.filt = torch.empty((g["na"], g["ns"]), **f32)
        self.names = ["fp_par_2d", "ramp_filter", "bp_par_2d"]
        # our kernels per call (fp_par_2d: the plan's one-image projector makes
        # its own transposed copy)
        self.kernels = {"fp_par_2d": 1, "ramp_filter": 1, "bp_par_2d": 1}
        # algorithmic FP32 FLOPs per launch (fixed conventions)
        self.flops = {"fp_par_2d": 6.0 * g["na"] * g["ns"] * g["ny"],
                      "ramp_filter": 2.0 * g["ns"] * g["na"] * g["ns"],
                      "bp_par_2d": 9.0 * g["nx"] * g["ny"] * g["na"]}
        self.bytes = {"fp_par_2d": 4.0 * (g["nx"] * g["ny"] + g["na"] * g["ns"]),
                      "ramp_filter": 8.0 * g["na"] * g["ns"],
                      "bp_par_2d": 4.0 * (g["nx"] * g["ny"] + g["na"] * g["ns"])}
        self.updates = float(g["nx"] * g["ny"] * g["na"])

    def launches(self, img, out, stream):
        L = self.lib
        s = ctypes.c_void_p(stream)
        yield lambda: L.ctr_fp_par_2d_plan_run(self.fplan, ctypes.c_void_p(img.data_ptr()),
                                               ctypes.c_void_p(self.sino.data_ptr()), 1, s)
        yield lambda: L.ctr_ramp_filter_f32(ctypes.byref(self.ramp.p),
                                            ctypes.c_void_p(self.sino.data_ptr()), self.taps,
                                            ctypes.c_void_p(self.filt.data_ptr()), 1, s)
        yield lambda: L.ctr_bp_plan_run(self.bplan, ctypes.c_void_p(self.filt.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), 1, s)


class FanPipeline:
    """fan_weighting -> ramp(fan) -> bp_fan_2d through the C ABI."""

    def __init__(self, g, device):
        import torch
        from ct_recon_extensions_gb300 import _lib
        from ct_recon_extensions_gb300 import torch_ctrecon as tc
        self.lib = _lib.load()
        self.g = g
        self.w = tc.FanWeightingOp(g["ns"], g["na"], g["ds"], g["offset_s"], g["dso"], g["dsd"], 1)
        self.ramp = tc.RampFilterOp(g["ns"], g["na"], g["ds"], g["dsd"], 1)
        self.bp = tc.FanBackprojection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                           g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                           g["offset_x"], g["offset_y"], g["dso"], g["dsd"], g["fov"])
        self.taps = ctypes.c_void_p(self.ramp.taps(device).data_ptr())
        self.bplan = self.bp.plan(device, 1)  # per-geometry tables, scratch and view constants
        f32 = dict(dtype=torch.float32, device=device)
        self.wt = torch.empty((g["na"], g["ns"]), **f32)
        self.filt = torch.empty((g["na"], g["ns"]), **f32)
        self.names = ["fan_weighting", "ramp_filter", "bp_fan_2d"]
        self.kernels = {"fan_weighting": 1, "ramp_filter": 1, "bp_fan_2d": 1}
        self.flops = {"fan_weighting": 1.0 * g["na"] * g["ns"],
                      "ramp_filter": 2.0 * g["ns"] * g["na"] * g["ns"],
                      "bp_fan_2d": 32.0 * g["nx"] * g["ny"] * g["na"]}
        self.bytes = {"fan_weighting": 8.0 * g["na"] * g["ns"],
                      "ramp_filter": 8.0 * g["na"] * g["ns"],
                      "bp_fan_2d": 4.0 * (g["nx"] * g["ny"] + g["na"] * g["ns"])}
        self.updates = float(g["nx"] * g["ny"] * g["na"])

    def launches(self, sino, out, stream):
        L = self.lib
        s = ctypes.c_void_p(stream)
        yield lambda: L.ctr_fan_weighting_f32(ctypes.byref(self.w.p), ctypes.c_void_p(sino.data_ptr()),
                                              ctypes.c_void_p(self.wt.data_ptr()), 1, s)
        yield lambda: L.ctr_ramp_filter_f32(ctypes.byref(self.ramp.p), ctypes.c_void_p(self.wt.data_ptr()),
                                            self.taps, ctypes.c_void_p(self.filt.data_ptr()), 1, s)
        yield lambda: L.ctr_bp_plan_run(self.bplan, ctypes.c_void_p(self.filt.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), 1, s)


class LowpFanPipeline:
    """Sinogram stored in BF16 or FP16: fan weighting + ramp(fan) as one
    tensor-core Toeplitz GEMM call (split kernel + tcgen05 GEMM over `splits`
    BF16 terms per operand, FP32 accumulate), then bp_fan_2d in FP32."""

    def __init__(self, g, device, dtype, splits=3):
        import torch
        from ct_recon_extensions_gb300 import _lib
        from ct_recon_extensions_gb300 import torch_ctrecon as tc
        self.lib = _lib.load()
        self.g = g
        w = tc.FanWeightingOp(g["ns"], g["na"], g["ds"], g["offset_s"], g["dso"], g["dsd"], 1)
        self.tcop = tc.RampFilterTCOp(g["ns"], g["na"], g["ds"], g["dsd"], 1, weighting=w, splits=splits)
        self.plan = self.tcop.plan(device, False, 1)
        self.dt = tc.RampFilterTCOp._DTYPES[dtype]
        self.bp = tc.FanBackprojection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                           g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                           g["offset_x"], g["offset_y"], g["dso"], g["dsd"], g["fov"])
        self.bplan = self.bp.plan(device, 1)  # per-geometry tables, scratch and view constants
        self.filt = torch.empty((g["na"], g["ns"]), dtype=torch.float32, device=device)
        self.names = ["ramp_filter_tc", "bp_fan_2d"]
        self.kernels = {"ramp_filter_tc": 2, "bp_fan_2d": 1}
        info = self.tcop.info(device)
        self.flops = {"ramp_filter_tc": float(info["mma_flops_per_row"]) * g["na"],
                      "bp_fan_2d": 32.0 * g["nx"] * g["ny"] * g["na"]}
        self.updates = float(g["nx"] * g["ny"] * g["na"])

    def launches(self, sino, out, stream):
        L = self.lib
        s = ctypes.c_void_p(stream)
        yield lambda: L.ctr_ramp_filter_tc_run(self.plan, self.dt, ctypes.c_void_p(sino.data_ptr()),
                                               ctypes.c_void_p(self.filt.data_ptr()), 1, s)
        yield lambda: L.ctr_bp_plan_run(self.bplan, ctypes.c_void_p(self.filt.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), 1, s)


# per-kernel CUDA events are recorded on every KERNEL_EVERY-th timed step only,
# so that their own cost stays out of the step time
KERNEL_EVERY = 8


def run_device(pipe, pool_dev, outs, steps, warmup, dist, per_kernel=True):
    """Time `steps` pipeline steps on device-resident inputs; returns (seconds,
    per-kernel mean ms, launches).  Per-kernel times come from CUDA events
    around each launch of every KERNEL_EVERY-th step of the timed region."""
    import torch
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    P = len(pool_dev)

    def step(k, rec):
        for i, fn in enumerate(pipe.launches(pool_dev[k % P], outs[k % len(outs)], sp)):
            if rec is not None:
                rec[i][0].record(stream)
            st = fn()
            if st != 0:
                raise RuntimeError(f"{pipe.names[i]} failed: {pipe.lib.ctr_last_error().decode()}")
            if rec is not None:
                rec[i][1].record(stream)

    for k in range(warmup):
        step(k, None)
    torch.cuda.synchronize()
    sampled = [k for k in range(steps) if k % KERNEL_EVERY == 0] if per_kernel else []
    ev = {k: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in pipe.names] for k in sampled}
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    t0.record(stream)
    for k in range(steps):
        step(warmup + k, ev.get(k))
    t1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    secs = t0.elapsed_time(t1) / 1e3
    kern = {}
    if per_kernel:
        for i, n in enumerate(pipe.names):
            kern[n] = statistics.fmean(ev[k][i][0].elapsed_time(ev[k][i][1]) for k in sampled)
    return secs, kern, sum(pipe.kernels.values()) * steps


KERNEL_REPS = 100  # back-to-back launches per stage in the per-kernel pass


def stage_ms(launch, reps=KERNEL_REPS):
    """Mean device time of one call of `launch(k, stream)` (k = repetition
    index, so callers can cycle their inputs): `reps` calls captured in a CUDA
    graph, the graph replayed once untimed and once between CUDA events on the
    replay stream, so the mean has no host gaps.  Where capture fails (a call
    that cannot be captured), the calls are issued directly between events."""
    import torch
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for k in range(3):
            launch(k, s.cuda_stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    try:
        with torch.cuda.graph(g, stream=s):
            for k in range(reps):
                launch(k, s.cuda_stream)
        captured = True
    except Exception:
        torch.cuda.synchronize()
        captured = False
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(s):
        if captured:
            g.replay()
            e0.record(s)
            g.replay()
            e1.record(s)
        else:
            e0.record(s)
            for k in range(reps):
                launch(k, s.cuda_stream)
            e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, captured


def pipeline_kernel_pass(pipe, pool_dev, outs):
    """Per-stage mean time of the pipeline (pipe.names order): the first stage
    cycles through the input pool (as the timed steps do), later stages read
    the pipeline's own intermediate buffers."""
    res, graphs = {}, []
    P = len(pool_dev)
    for i, name in enumerate(pipe.names):
        def launch(k, sp, i=i, name=name):
            fn = list(pipe.launches(pool_dev[k % P], outs[k % len(outs)], sp))[i]
            if fn() != 0:
                raise RuntimeError(f"{name}: {pipe.lib.ctr_last_error().decode()}")
        ms, cap = stage_ms(launch)
        res[name] = ms
        graphs.append(cap)
    return res, all(graphs)


def op_call(op, which, x, out, sp):
    """One C-ABI call of a torch_ctrecon operator's forward, adjoint or single
    view into a preallocated output, on stream handle sp (one item)."""
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    from ct_recon_extensions_gb300._lib import call
    s = ctypes.c_void_p(sp)
    p = ctypes.byref(op.p)
    xi, oi = ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr())
    if isinstance(op, tc.FanBackprojection2DOp):
        t = [ctypes.c_void_p(a.data_ptr()) for a in op.tables(x.device)]
        if which == "forward":
            call("ctr_bp_plan_run", op.plan(x.device, 1), xi, oi, 1, s)
        else:
            call("ctr_bp_plan_run_grad", op.plan(x.device, 1), xi, oi, 1, s)
    elif isinstance(op, tc.ParallelBackprojection2DOp):
        t = [ctypes.c_void_p(a.data_ptr()) for a in op.tables(x.device)]
        if which == "forward":
            call("ctr_bp_plan_run", op.plan(x.device, 1), xi, oi, 1, s)
        elif which == "adjoint":
            call("ctr_bp_plan_run_grad", op.plan(x.device, 1), xi, oi, 1, s)
        else:
            call("ctr_bp_par_2d_sv_f32", p, xi, oi, *t, None, 1, s)
    elif isinstance(op, tc.RampFilterOp):
        taps = ctypes.c_void_p(op.taps(x.device).data_ptr())
        call("ctr_ramp_filter_f32" if which == "forward" else "ctr_ramp_filter_grad_f32", p, xi, taps, oi, 1, s)
    elif isinstance(op, tc.FanWeightingOp):
        call("ctr_fan_weighting_f32" if which == "forward" else "ctr_fan_weighting_grad_f32", p, xi, oi, 1, s)
    else:
        raise TypeError(type(op))


def run_adjoints(device, dist):
    """The FP32 adjoints beside their forwards, one image per call: bp_fan_2d
    and its exact adjoint at config 1 (720 x 736 -> 512^2), bp_par_2d and its
    adjoint at config 2 (720 x 729 -> 512^2), and the sinogram gradient of the
    fan FBP chain (bp_fan_2d adjoint -> ramp-filter adjoint -> fan-weighting
    adjoint, the reference's TF gradient wiring), with FP32-pipe throughput
    (the forward's algorithmic FLOPs: 32 per fan update, 9 per parallel one)."""
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    rng = np.random.default_rng(5)
    out = {}
    gf, gp = syn.fan_config_1(), syn.parallel_config_2()
    fan = tc.FanBackprojection2DOp(gf["ns"], gf["na"], gf["ds"], gf["orbit"], gf["offset_s"],
                                   gf["orbit_start"], gf["nx"], gf["ny"], gf["dx"], gf["dy"],
                                   gf["offset_x"], gf["offset_y"], gf["dso"], gf["dsd"], gf["fov"])
    par = tc.ParallelBackprojection2DOp(gp["ns"], gp["na"], gp["ds"], gp["orbit"], gp["offset_s"],
                                        gp["orbit_start"], gp["nx"], gp["ny"], gp["dx"], gp["dy"],
                                        gp["offset_x"], gp["offset_y"], gp["fov"])
    w = tc.FanWeightingOp(gf["ns"], gf["na"], gf["ds"], gf["offset_s"], gf["dso"], gf["dsd"], 1)
    ramp = tc.RampFilterOp(gf["ns"], gf["na"], gf["ds"], gf["dsd"], 1)
    f32 = dict(dtype=torch.float32, device=device)
    pool = 40  # 40 distinct inputs of 1-2 MB: more than L2 per cycle

    def randn(shape):
        return torch.from_numpy(rng.standard_normal(shape).astype(np.float32)).to(device)

    for name, op, g, fl in (("bp_fan_2d", fan, gf, 32.0), ("bp_par_2d", par, gp, 9.0)):
        sinos = [randn((g["na"], g["ns"])) for _ in range(pool)]
        imgs = [randn((g["ny"], g["nx"])) for _ in range(pool)]
        img_out = torch.empty((g["ny"], g["nx"]), **f32)
        sino_out = torch.empty((g["na"], g["ns"]), **f32)
        flops = fl * g["nx"] * g["ny"] * g["na"]
        ms_f, _ = stage_ms(lambda k, sp: op_call(op, "forward", sinos[k % pool], img_out, sp))
        ms_a, _ = stage_ms(lambda k, sp: op_call(op, "adjoint", imgs[k % pool], sino_out, sp))
        out[name] = {"forward_ms": ms_f, "adjoint_ms": ms_a, "adjoint_over_forward": ms_a / ms_f,
                     "forward_tflops": flops / ms_f / 1e9, "adjoint_tflops": flops / ms_a / 1e9}
    imgs = [randn((gf["ny"], gf["nx"])) for _ in range(pool)]
    t1, t2, t3 = (torch.empty((gf["na"], gf["ns"]), **f32) for _ in range(3))

    def chain(k, sp):
        op_call(fan, "adjoint", imgs[k % pool], t1, sp)
        op_call(ramp, "adjoint", t1, t2, sp)
        op_call(w, "adjoint", t2, t3, sp)
    ms_c, _ = stage_ms(chain)
    out["fan_chain_grad"] = {"ms": ms_c, "kernels": 4,
                             "workload": "d loss / d sinogram of fan_weighting -> ramp(fan) -> "
                                         "bp_fan_2d, 720 x 736 -> 512^2"}
    out["workload"] = ("FP32 adjoints vs forwards, one image per call, 100 calls replayed from a "
                       "CUDA graph, inputs cycled over 40 distinct buffers")
    return out


def run_single_view(device, dist):
    """bp_par_2d_sv at config 2: 720 x 729 -> 512 x 512 x 720 FP32 (755 MB out,
    write-bound), one sinogram per call, against the measured HBM bandwidth."""
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    g = syn.parallel_config_2()
    op = tc.ParallelBackprojection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                       g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                       g["offset_x"], g["offset_y"], g["fov"])
    rng = np.random.default_rng(9)
    sinos = [torch.from_numpy(rng.standard_normal((g["na"], g["ns"])).astype(np.float32)).to(device)
             for _ in range(4)]
    out = torch.empty((g["ny"], g["nx"], g["na"]), dtype=torch.float32, device=device)
    ms, _ = stage_ms(lambda k, sp: op_call(op, "single_view", sinos[k % 4], out, sp), reps=20)
    wbytes = 4.0 * g["nx"] * g["ny"] * g["na"]
    rbytes = 4.0 * g["na"] * g["ns"] + 8.0 * g["na"] * (g["nx"] + g["ny"])  # sinogram + FP64 tables
    gbs = (wbytes + rbytes) / ms / 1e6
    peak = hbm_peak_gbs()
    return {"workload": "bp_par_2d_sv 720 views x 729 bins -> 512 x 512 x 720 (FP32), one sinogram per call",
            "ms_per_call": ms, "algorithmic_bytes": wbytes + rbytes, "achieved_gbs": gbs,
            "hbm_peak_gbs": peak, "hbm_frac": gbs / peak, "calls": 20}


def run_batched(device, steps, warmup, dist):
    """The uneven fan batch (64 items, image 256^2..1024^2, 360..2304 views,
    512..1024 channels): one plan run (batched filter launch + one persistent
    backprojection launch, replayed from a CUDA graph) per step, against the
    same items through the plain per-item drop-in (3 launches an item)."""
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300.batch import FanFBPBatch
    items = syn.batched_config_3()
    geoms = [{k: v for k, v in it.items() if k != "seed"} for it in items]
    sinos = [syn.fan_sinogram_torch(syn.random_ellipses(it["seed"]), g["na"], g["ns"], g["ds"],
                                    g["orbit"], g["dso"], g["dsd"], device).contiguous()
             for it, g in zip(items, geoms)]
    outs = [torch.empty((g["ny"], g["nx"]), dtype=torch.float32, device=device) for g in geoms]
    updates = float(sum(g["nx"] * g["ny"] * g["na"] for g in geoms))
    stream = torch.cuda.current_stream()

    def timed(fn, k):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        dist.barrier()
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(k):
            fn()
        t1.record(stream)
        torch.cuda.synchronize()
        dist.barrier()
        return dist.max(t0.elapsed_time(t1) / 1e3)

    plan = FanFBPBatch(geoms)  # autotuned, CUDA graph
    k = max(3, min(steps, 10))
    b_secs = timed(lambda: plan.run(sinos, outs), k)
    info = plan.info()
    pipes = [FanPipeline(g, device) for g in geoms]
    sp = stream.cuda_stream
    outs_plain = [torch.empty_like(o) for o in outs]

    def plain():
        for pipe, s, o in zip(pipes, sinos, outs_plain):
            for fn in pipe.launches(s, o, sp):
                if fn() != 0:
                    raise RuntimeError(pipe.lib.ctr_last_error().decode())

    p_secs = timed(plain, k)
    # the plan's images against the plain per-item path's (separate buffers)
    plan.run(sinos, outs)
    plain()
    torch.cuda.synchronize()
    diffs = [rel_l2(a.cpu().numpy(), b.cpu().numpy()) for a, b in zip(outs, outs_plain)]
    n = len(geoms)
    plan.close()
    return {
        "workload": "64 fan sinograms of uneven size (image 256^2-1024^2, 360-2304 views, "
                    "512-1024 channels): weighting -> ramp(fan) -> bp_fan_2d",
        "slices_per_s": n * k / b_secs, "updates_per_s": updates * k / b_secs,
        "plain_slices_per_s": n * k / p_secs, "speedup_vs_plain": p_secs / b_secs,
        "rel_l2_plan_vs_plain_max": max(diffs),
        "plan": {key: info[key] for key in ("tile_rows", "view_block", "ctas", "autotuned",
                                            "tuned_ms", "graph", "launches_per_run")},
        "gpu_launches": int(info["launches_per_run"]) * k, "runs": k,
    }


def run_fp_methods(device, steps, warmup, dist):
    """The parallel forward projector by method on the headline geometry
    (512^2 at 0.5 mm -> 720 views x 729 bins over pi): ray casting with a 128 mm
    FoV radius and 0.125-pixel steps (its samples counted from the prep's step
    counts), distance driven and ray driven, one image per call."""
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    g = dict(syn.parallel_config_2(), fov=128.0)
    img = torch.from_numpy(syn.rasterize(syn.random_ellipses(4100), g["nx"], g["ny"], g["dx"],
                                         g["dy"])).float().to(device)
    out = {}
    for method in ("raycasting", "disdriven", "raydriven"):
        op = tc.ParallelProjection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                       g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                       g["offset_x"], g["offset_y"], g["fov"], method=method)
        for _ in range(max(1, warmup)):
            op.forward(img)
        k = max(3, min(steps, 50))
        stream = torch.cuda.current_stream()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        dist.barrier()
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(k):
            op.forward(img)
        t1.record(stream)
        torch.cuda.synchronize()
        dist.barrier()
        ms = dist.max(t0.elapsed_time(t1)) / k
        row = {"ms_per_call": ms, "projections_per_s": 1e3 / ms, "calls": k}
        if method == "raycasting":
            steps_total = float(op.tables(img.device)[2].to(torch.int64).sum())
            row.update({"samples_per_call": steps_total, "gsamples_per_s": steps_total / ms / 1e6,
                        "step_size": op.step_size, "fov_mm": g["fov"], "gpu_launches": k})
        elif method == "disdriven":
            row.update({"line_footprints_per_s": g["na"] * g["ns"] * g["ny"] / ms * 1e3,
                        "gpu_launches": k})
        else:
            row.update({"gpu_launches": 2 * k})
        out[method] = row
    out["workload"] = ("fp_par_2d by method, 512^2 @0.5 mm -> 720 x 729 over pi; ray casting: "
                       "FoV radius 128 mm, 0.125-pixel steps; distance driven; ray driven")
    return out


def helical_scan():
    """A clinical-size helical scan: 736 channels x 64 rows, 1152 views per
    rotation, pitch 1 (the couch moves nt * dso / dsd per rotation, the row unit
    of the reference's z -> row mapping), 128 slices of 1 mm over one rotation
    of couch travel (9 views apart), views enough for 360LI around every slice."""
    from ct_recon_extensions_gb300._lib import HelicalParam
    ns, nt, vpr, dso, dsd = 736, 64, 1152, 595.0, 1085.6
    cm = nt * dso / dsd / vpr
    nz, step = 128, 9
    c0 = vpr + 8                      # first slice's nearest view (360LI needs c0 - vpr >= 0)
    na = c0 + step * (nz - 1) + vpr + 8
    return HelicalParam(ns=ns, nt=nt, na=na, ds=1.2858, dt=1.0, offset_s=1.25, offset_t=0.0,
                        orbit_start=0.0, orbit=2 * math.pi / vpr, couch_begin=0.0, couch_mov=cm,
                        view_per_rot=vpr, nz=nz, dz=step * cm, z0=c0 * cm + 0.1 * cm,
                        thickness=1.0, dso=dso, dsd=dsd)


def helical_bytes(h, method, itemsize):
    """Algorithmic bytes of one rebinning call: the output plus every input row
    some sample reads (per view, the union over slices of the thick-slice rows,
    taken at the extreme fan angles)."""
    center_s = (h.ns - 1) / 2.0 + h.offset_s
    gam = (np.array([0.0, h.ns - 1]) - center_s) * h.ds / h.dsd
    cgs = np.concatenate([np.cos(gam), [1.0]])
    ct = (h.nt - 1) / 2.0 + h.offset_t
    lo_v = np.full(h.na, h.nt, np.int64)
    hi_v = np.zeros(h.na, np.int64)
    z = h.z0
    for _ in range(h.nz):
        c = int(round((z - h.couch_begin) / h.couch_mov))
        lo, hi = (c - h.view_per_rot, c + h.view_per_rot - 1) if method == "360" else \
            (c - h.view_per_rot // 2, c - h.view_per_rot // 2 + h.view_per_rot - 1)
        v = np.arange(max(lo - 1, 0), hi + 1)
        zd = z - h.couch_begin - v * h.couch_mov
        for cg in cgs:
            top = np.clip(ct - (zd + h.thickness / 2) / h.dso * cg * h.dsd, 0, h.nt)
            bot = np.clip(ct - (zd - h.thickness / 2) / h.dso * cg * h.dsd, 0, h.nt)
            r0, r1 = np.floor(top).astype(np.int64), np.ceil(bot).astype(np.int64)
            ok = r1 > r0
            lo_v[v[ok]] = np.minimum(lo_v[v[ok]], r0[ok])
            hi_v[v[ok]] = np.maximum(hi_v[v[ok]], r1[ok])
        z += h.dz
    rows = np.maximum(hi_v - lo_v, 0).sum()
    return int(rows) * h.ns * itemsize + h.nz * h.view_per_rot * h.ns * itemsize


def run_helical(device, steps, warmup, dist, cpu):
    """Helical rebinning (360LI and 180LI) of one clinical-size scan per call,
    T=float (FP64 arithmetic inside, as the reference), input larger than L2;
    with `cpu`, the oracle port on the host cores over a 2-slice sample."""
    import torch
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    h = helical_scan()
    gen = torch.Generator(device=device).manual_seed(11)
    x = 1 + 0.1 * torch.randn((1, h.na, h.nt, h.ns), generator=gen, device=device)
    peak = hbm_peak_gbs()
    out = {"workload": (f"helical scan {h.na} views x {h.nt} rows x {h.ns} ch, "
                        f"{h.view_per_rot} views/rotation, pitch 1 -> {h.nz} slices x "
                        f"{h.view_per_rot} x {h.ns}, T=float")}
    for method in ("360", "180"):
        op = tc.HelicalInterpolationOp(h.ns, h.nt, h.na, h.ds, h.dt, h.offset_s, h.offset_t,
                                       h.orbit_start, h.orbit, h.couch_begin, h.couch_mov,
                                       h.view_per_rot, h.nz, h.dz, h.z0, h.thickness, h.dso,
                                       h.dsd, method)
        res = torch.empty((1, h.nz, h.view_per_rot, h.ns), device=device)
        status = torch.zeros(h.nz, dtype=torch.int32, device=device)
        for _ in range(max(3, warmup)):
            op.launch(x, res, status)
        k = max(3, min(steps, 20))
        stream = torch.cuda.current_stream()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        dist.barrier()
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(k):
            op.launch(x, res, status)
        t1.record(stream)
        torch.cuda.synchronize()
        dist.barrier()
        ms = dist.max(t0.elapsed_time(t1)) / k
        nbytes = helical_bytes(h, method, 4)
        row = {"ms_per_call": ms, "slices_per_s": h.nz / ms * 1e3,
               "outputs_per_s": h.nz * h.view_per_rot * h.ns / ms * 1e3,
               "algorithmic_bytes": nbytes, "achieved_gbs": nbytes / ms / 1e6,
               "hbm_peak_gbs": peak, "hbm_frac": nbytes / ms / 1e6 / peak,
               "status_words_nonzero": int((status != 0).sum()), "gpu_launches": k}
        if cpu:
            from oracle import Heli, Oracle
            nthreads = os.cpu_count() or 1
            sub = Heli(**{f: getattr(h, f) for f, _ in Heli._fields_})
            sub.nz = 2
            xs = x[0].cpu().numpy()
            port = Oracle("port", threads=nthreads)
            port.helical(xs, sub, method)
            t = time.perf_counter()
            port.helical(xs, sub, method)
            dt = time.perf_counter() - t
            row["cpu_port"] = {"slices_per_s": 2 / dt, "threads": nthreads,
                               "sample": "2 slices of the same scan (slices are independent)"}
            row["gpu_over_cpu"] = row["slices_per_s"] / row["cpu_port"]["slices_per_s"]
        out[method] = row
    return out


def hbm_peak_gbs():
    """The HBM copy bandwidth measured on this GPU type, from MEASURED_PEAKS.json
    beside this file, else the fallback."""
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def run_gd(device, steps, warmup, dist):
    """The differentiable pair: gradient descent on ||A x - y||^2 for a batch of
    16 images of 512^2 (parallel, 720 views, 729 bins), y = A x_true + Gaussian
    noise (1 % of max), step 1/||A^T A||.  A step = forward projection of the
    batch, residual, backward through torch.autograd (the adjoint kernel),
    update."""
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300 import torch_ctrecon as tc
    g = syn.parallel_config_2()
    op = tc.ParallelProjection2DOp(g["ns"], g["na"], g["ds"], g["orbit"], g["offset_s"],
                                   g["orbit_start"], g["nx"], g["ny"], g["dx"], g["dy"],
                                   g["offset_x"], g["offset_y"], g["fov"])
    B = 16
    xt = torch.from_numpy(np.stack([syn.rasterize(syn.random_ellipses(4000 + i), g["nx"], g["ny"],
                                                  g["dx"], g["dy"]) for i in range(B)])).float().to(device)
    with torch.no_grad():
        y = op.forward(xt)
        gen = torch.Generator(device=device).manual_seed(4)
        y += 0.01 * y.max() * torch.randn(y.shape, generator=gen, device=device)
        v = torch.ones_like(xt)  # step 1/L, L = ||A^T A|| by power iteration
        for _ in range(10):
            v = op.adjoint(op.forward(v))
            L = float(v.norm()) / math.sqrt(v.numel())
            v *= math.sqrt(v.numel()) / float(v.norm())
    x = torch.zeros_like(xt, requires_grad=True)
    lr = 1.0 / L
    stream = torch.cuda.current_stream()
    ev = []

    def step(rec):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if rec else None
        if rec:
            e[0].record(stream)
        ax = tc.apply(op, x)
        if rec:
            e[1].record(stream)
        loss = 0.5 * (ax - y).pow(2).sum()
        if rec:
            e[2].record(stream)
        loss.backward()
        if rec:
            e[3].record(stream)
            ev.append(e)
        with torch.no_grad():
            x.sub_(lr * x.grad)
            x.grad = None
        return loss.detach()

    l0 = None
    for _ in range(warmup):
        lw = step(False)
        l0 = float(lw) if l0 is None else l0
    k = max(3, min(steps, 20))
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(k):
        loss = step(True)
    t1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    secs = dist.max(t0.elapsed_time(t1) / 1e3)
    fwd = statistics.fmean(e[0].elapsed_time(e[1]) for e in ev)
    bwd = statistics.fmean(e[2].elapsed_time(e[3]) for e in ev)
    return {
        "workload": "gradient descent on ||Ax - y||^2, batch 16 x 512^2, fp_par_2d 720 x 729 "
                    "and its adjoint through torch.autograd",
        "steps_per_s": k / secs, "images_per_s": B * k / secs,
        "forward_batch_ms": fwd, "backward_batch_ms": bwd,
        "loss_first": l0, "loss_last": float(loss), "steps": k,
        "gpu_launches": k * (3 + 1),
    }


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


LOWP_STRIPS = ((256, 16), (900, 16), (1400, 16), (1800, 16))  # (first row, rows) of the check


def lowp_check(g, stored, imgs):
    """FP64 oracle of the large fan FBP (fan weighting -> ramp(fan) ->
    bp_fan_2d, the port on all host cores) on 4 strips of 16 image rows,
    against each path's image: the oracle of the stored sinogram (the kernels'
    error) and of the exact FP64 sinogram (storage included).  The strips are
    sub-images whose pixel centres are the full image's rows."""
    from oracle import Geom, Oracle
    orc = Oracle("port", threads=os.cpu_count() or 1)

    def strips(sino64):
        w = orc.fan_weighting(sino64, g["ds"], g["offset_s"], g["dso"], g["dsd"], 1)
        f = orc.ramp_filter(w, g["ds"], g["dsd"], 1)
        out = []
        for r0, k in LOWP_STRIPS:
            off_y = (g["ny"] - 1) / 2 + g["offset_y"] - r0 - (k - 1) / 2
            gs = Geom.make(g["ns"], g["na"], g["ds"], g["orbit"], g["nx"], k, g["dx"], g["dy"],
                           g["offset_s"], g["orbit_start"], g["offset_x"], off_y, g["dso"], g["dsd"],
                           g["fov"])
            out.append(orc.bp_fan_2d(f, gs))
        return np.concatenate(out)

    def rows(img):
        return np.concatenate([img[r0:r0 + k] for r0, k in LOWP_STRIPS]).astype(np.float64)

    t0 = time.perf_counter()
    exact = strips(stored["exact"])
    res = {}
    for name, img in imgs.items():
        same = strips(stored[name])
        got = rows(img)
        res[name] = {"rel_l2_vs_fp64": rel_l2(got, same),
                     "max_abs_vs_fp64": float(np.abs(got - same).max()),
                     "rel_l2_vs_fp64_exact_sinogram": rel_l2(got, exact),
                     "max_abs_vs_fp64_exact_sinogram": float(np.abs(got - exact).max())}
    res["image_max_abs"] = float(np.abs(exact).max())
    res["oracle"] = (f"FP64 port on {os.cpu_count()} threads, rows "
                     + ", ".join(f"{r0}-{r0 + k - 1}" for r0, k in LOWP_STRIPS)
                     + f" of {g['ny']} ({sum(k for _, k in LOWP_STRIPS) * g['nx']} pixels), "
                     f"{time.perf_counter() - t0:.1f} s")
    return res


def run_lowp(device, steps, warmup, dist, check):
    """The large reduced-precision slice: 2048^2 at 0.25 mm from 2304 fan views
    over 2pi x 1472 channels.  The sinogram is stored in FP32 (plain path:
    fan_weighting -> ramp_filter on the FP32 pipe -> bp_fan_2d) and in BF16
    and FP16 (weighting + filter as the tensor-core Toeplitz GEMM with
    hi/mid/lo operands, then bp_fan_2d in FP32); bf16_hilo is the BF16 path
    with the 2-term (hi/lo, 3-product) split.  Each path runs on 4 distinct sinograms; with `check`
    its error against the FP64 oracle is measured on image strips."""
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    g = syn.large_config_5()
    k = max(3, min(steps, 20))
    base = syn.fan_sinogram(syn.random_ellipses(5000), g["na"], g["ns"], g["ds"], g["orbit"], g["dso"],
                            g["dsd"], dtype=np.float64)
    outs = [torch.empty((g["ny"], g["nx"]), dtype=torch.float32, device=device) for _ in range(2)]
    paths = {"f32": (lambda: FanPipeline(g, device), torch.float32),
             "bf16": (lambda: LowpFanPipeline(g, device, torch.bfloat16, 3), torch.bfloat16),
             "f16": (lambda: LowpFanPipeline(g, device, torch.float16, 3), torch.float16),
             "bf16_hilo": (lambda: LowpFanPipeline(g, device, torch.bfloat16, 2), torch.bfloat16)}
    res, imgs, stored = {}, {}, {"exact": base}
    peak_tc = bf16_peak_tflops()
    for name, (make, dt) in paths.items():
        pipe = make()
        pool = [torch.from_numpy(base * (1.0 + 1e-3 * i)).to(device=device, dtype=dt) for i in range(4)]
        secs, kern, launches = run_device(pipe, pool, outs, k, warmup, dist)
        secs = dist.max(secs)
        r = {"slices_per_s": dist.ws * k / secs, "ms_per_slice": 1e3 * secs / k, "kernel_ms": kern,
             "gpu_launches": launches, "storage": str(dt).replace("torch.", "")}
        if name == "f32":
            r["filter"] = "fan_weighting + ramp_filter, FP32 pipe (direct convolution)"
        else:
            fl = pipe.flops["ramp_filter_tc"]
            tfl = fl / (kern["ramp_filter_tc"] / 1e3) / 1e12
            r["filter"] = ("weighting + ramp as a Toeplitz GEMM on tcgen05, FP32 accumulate (split kernel"
                           " + GEMM kernel): " + ("BF16 hi/mid/lo, 6 term products" if pipe.tcop.splits == 3
                                                  else "BF16 hi/lo, 3 term products"))
            r["filter_tc"] = {"mma_flops": fl, "tflops": tfl, "peak": peak_tc[0], "frac": tfl / peak_tc[0],
                              "peak_source": peak_tc[1], "unit": "TFLOP/s"}
        if check:
            run = list(pipe.launches(pool[0], outs[0], torch.cuda.current_stream().cuda_stream))
            for fn in run:
                if fn() != 0:
                    raise RuntimeError(pipe.lib.ctr_last_error().decode())
            imgs[name] = outs[0].cpu().numpy()
            stored[name] = pool[0].to(torch.float64).cpu().numpy()
        res[name] = r
        if hasattr(pipe, "tcop"):
            torch.cuda.synchronize()
            pipe.tcop.close()
        del pool
    out = {"workload": "fan FBP, 2304 views over 2pi x 1472 ch at 0.6429 mm -> 2048x2048 at 0.25 mm; "
                       "sinogram stored in FP32, BF16, FP16; backprojection accumulates in FP32",
           "paths": res, "steps": k,
           "speedup_bf16_vs_f32": res["bf16"]["slices_per_s"] / res["f32"]["slices_per_s"]}
    if check:
        acc = lowp_check(g, stored, imgs)
        for name in imgs:
            res[name].update(acc[name])
        out["image_max_abs"] = acc["image_max_abs"]
        out["check"] = acc["oracle"]
    return out


def bf16_peak_tflops():
    """The dense BF16 tensor peak measured on this GPU type (cuBLAS 8192^3,
    burst), from MEASURED_PEAKS.json beside this file, else the fallback."""
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"]), "measured: cuBLAS bf16 8192^3 burst"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback: 1.9 PFLOP/s bf16 burst"


def run_e2e(pipe, pool_host, steps, warmup, in_shape, out_shape, device):
    """Through the C ABI with host buffers: every step copies its input slice
    from pinned host memory to the device, runs the pipeline's operators and
    copies the result back to pinned host memory.  The library's HostStreamer
    overlaps the copies of neighbouring steps with the compute (2 device
    buffer pairs, separate copy-in / compute / copy-out streams).  Timed on
    the host from the first step's copy to the last result on the host."""
    import torch
    from ct_recon_extensions_gb300.host_stream import HostStreamer

    def step(din, dout, s):
        for fn in pipe.launches(din, dout, s):
            if fn() != 0:
                raise RuntimeError(pipe.lib.ctr_last_error().decode())

    hs = HostStreamer(step, in_shape, out_shape, device, depth=2)
    P = len(pool_host)
    hout = [torch.empty(out_shape, dtype=torch.float32, pin_memory=True) for _ in range(4)]
    hs.run([pool_host[k % P] for k in range(warmup)], [hout[k % 4] for k in range(warmup)])
    torch.cuda.synchronize()
    ins = [pool_host[(warmup + k) % P] for k in range(steps)]
    outs = [hout[k % 4] for k in range(steps)]
    t = time.perf_counter()
    hs.run(ins, outs)
    secs = time.perf_counter() - t
    return secs, hs.din[0].numel() * 4, hs.dout[0].numel() * 4


def fp32_peak_tflops(device):
    """Measured FP32 (non-tensor) throughput: cuBLAS SGEMM with TF32 off,
    best of 5 at 8192^3."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device=device)
        b = torch.randn(n, n, device=device)
        c = a @ b
        torch.cuda.synchronize()
        best = math.inf
        for _ in range(5):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        del a, b, c
        return 2.0 * n ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def read_traffic():
    """Per-launch DRAM bytes measured by ncu, from profiles/ncu_traffic.txt
    (lines: '<kernel> <bytes per launch> <workload>')."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    out = {}
    if os.path.exists(path):
        for ln in open(path):
            f = ln.split()
            if len(f) >= 2 and not ln.startswith("#"):
                try:
                    out[f[0]] = float(f[1])
                except ValueError:
                    pass
    return out


# ---------------------------------------------------------------------------
# CPU side (oracle port / reference build)
# ---------------------------------------------------------------------------

def cpu_slices_per_s(kind, g, n_slices, threads):
    """Time the reference CPU algorithm of one step on n_slices slices."""
    from oracle import Geom, Oracle, REF_LIB
    from ct_recon_extensions_gb300 import synthetic as syn
    use_ref = kind == "reference" and os.path.exists(REF_LIB)
    gm = Geom.make(**g)
    e = syn.random_ellipses(2000)
    img = syn.rasterize(e, g["nx"], g["ny"], g["dx"], g["dy"])
    if use_ref:
        # the reference's own code is single-threaded per call: run one slice per thread
        from concurrent.futures import ThreadPoolExecutor
        orc = Oracle("reference")

        def one(_):
            s = orc.fp_par_2d(img, gm)
            return orc.bp_par_2d(orc.ramp_filter(s, gm.ds, -1.0, 0), gm)
        t = time.perf_counter()
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(one, range(n_slices)))
        secs = time.perf_counter() - t
        return n_slices / secs, "reference", threads
    orc = Oracle("port", threads=threads)
    t = time.perf_counter()
    for _ in range(n_slices):
        s = orc.fp_par_2d(img, gm)
        orc.bp_par_2d(orc.ramp_filter(s, gm.ds, -1.0, 0), gm)
    secs = time.perf_counter() - t
    return n_slices / secs, "port", threads


def cpu_configs(threads):
    """The oracle port (the reference's CPU algorithm restated in C, T=float)
    on a bounded sample of each configuration, with all host threads (rows
    split across threads) and, for configs 1 and 2, one thread.  Config 3
    times its first items and is scaled by pixel-view updates; config 5 runs
    weighting and filter in full and backprojects one 16-row strip, scaled to
    the 2048 rows."""
    from oracle import Geom, Oracle
    from ct_recon_extensions_gb300 import synthetic as syn

    def geom(g, ny=None, off_y=None):
        return Geom.make(g["ns"], g["na"], g["ds"], g["orbit"], g["nx"], g["ny"] if ny is None else ny,
                         g["dx"], g["dy"], g["offset_s"], g["orbit_start"], g["offset_x"],
                         g["offset_y"] if off_y is None else off_y, g.get("dso", -1.0), g.get("dsd", -1.0),
                         g["fov"])

    def timed(fn):
        t = time.perf_counter()
        fn()
        return time.perf_counter() - t

    res = {}
    g1 = syn.fan_config_1()
    s1 = syn.fan_sinogram(syn.random_ellipses(1000), g1["na"], g1["ns"], g1["ds"], g1["orbit"], g1["dso"],
                          g1["dsd"])
    c1 = {}
    for nt in (threads, 1):
        orc = Oracle("port", threads=nt)
        c1[f"slices_per_s_{nt}t"] = 1.0 / timed(lambda: orc.fbp_fan(s1, geom(g1)))
    res["fan_fbp_config1"] = dict(c1, sample="1 slice")
    g2 = par_geometry()
    c2 = {}
    for nt in (threads, 1):
        v, _, _ = cpu_slices_per_s("port", g2, 1, nt)
        c2[f"slices_per_s_{nt}t"] = v
    res["parallel_config2"] = dict(c2, sample="1 slice")
    items = syn.batched_config_3()
    upd_all = sum(it["nx"] * it["ny"] * it["na"] for it in items) / len(items)
    orc = Oracle("port", threads=threads)
    done, upd, secs = 0, 0.0, 0.0
    while upd < 4e8 and done < len(items):
        it = items[done]
        sino = syn.fan_sinogram(syn.random_ellipses(it["seed"]), it["na"], it["ns"], it["ds"], it["orbit"],
                                it["dso"], it["dsd"])
        secs += timed(lambda: orc.fbp_fan(sino, geom(it)))
        upd += it["nx"] * it["ny"] * it["na"]
        done += 1
    res["batched_fan_config3"] = {f"slices_per_s_{threads}t": upd / secs / upd_all,
                                  "sample": f"first {done} of {len(items)} items, scaled by updates"}
    img = syn.rasterize(syn.random_ellipses(4000), g2["nx"], g2["ny"], g2["dx"], g2["dy"])
    G2 = geom(g2)
    sec4 = timed(lambda: orc.fp_par_2d_grad(orc.fp_par_2d(img, G2), G2))
    res["gd_config4"] = {f"images_per_s_{threads}t": 1.0 / sec4,
                         "sample": "1 image: fp_par_2d and its adjoint"}
    g5 = syn.large_config_5()
    s5 = syn.fan_sinogram(syn.random_ellipses(5000), g5["na"], g5["ns"], g5["ds"], g5["orbit"], g5["dso"],
                          g5["dsd"])
    out = {}

    def filt():
        w = orc.fan_weighting(s5, g5["ds"], g5["offset_s"], g5["dso"], g5["dsd"], 1)
        out["f"] = orc.ramp_filter(w, g5["ds"], g5["dsd"], 1)
    secf = timed(filt)
    k, r0 = 16, 1000
    gs = geom(g5, ny=k, off_y=(g5["ny"] - 1) / 2 + g5["offset_y"] - r0 - (k - 1) / 2)
    secb = timed(lambda: orc.bp_fan_2d(out["f"], gs)) * g5["ny"] / k
    res["lowp_config5"] = {f"slices_per_s_{threads}t": 1.0 / (secf + secb),
                           "sample": "weighting + filter in full, one 16-row strip of the backprojection "
                                     "scaled to 2048 rows (FP32 storage)"}
    return res


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    try:
        oracle.build(ref_src="")
    except Exception as e:  # pragma: no cover
        print(json.dumps({"impl": "reference", "unavailable": f"oracle build failed: {e}"}))
        return
    g = par_geometry()
    threads = os.cpu_count() or 1
    kind = "reference" if os.path.exists(oracle.REF_LIB) else "port"
    # warm-up steps, then `steps` timed steps of one slice each
    for _ in range(min(args.warmup, 3)):
        cpu_slices_per_s(kind, g, 1, threads)
    t = time.perf_counter()
    steps = max(1, min(args.steps, 20))
    v, k, c = cpu_slices_per_s(kind, g, steps, threads)
    secs = time.perf_counter() - t
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "slices/s",
        "n_gpus": ws, "steps": steps, "warmup": min(args.warmup, 3),
        "ms_per_step": 1e3 * secs / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded random-ellipse phantom)",
        "config": {"workload": "parallel drop-in: fp_par_2d 512x512 @0.5mm -> 720 views x 729 bins "
                               "over pi -> ramp(par) -> bp_par_2d", "batch": 1},
        "cpu_baseline": {"value": v, "unit": "slices/s", "cores": c, "kind": k,
                         "sample": f"{steps} slices, one per step"},
        "e2e": {"value": v, "unit": "slices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "updates_per_s": v * g["nx"] * g["ny"] * g["na"],
    }
    if k == "port":
        line["cpu_baseline"]["note"] = ("the reference's own src/ was not built on this host (its checkout is "
                                        "absent), so the oracle port runs: the reference's CPU algorithm "
                                        "restated in C, bit-exact to fixtures made by the reference build")
    print(json.dumps(line))


# ---------------------------------------------------------------------------

def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    dist = Dist("nccl")
    from ct_recon_extensions_gb300 import build as b
    b.build()
    from ct_recon_extensions_gb300 import _lib
    lib = _lib.load()
    if lib.ctr_device_check() != 0:
        raise SystemExit(lib.ctr_last_error().decode())

    # ---- parallel drop-in (headline) ----
    g = par_geometry()
    pipe = ParPipeline(g, device)
    base = make_pool("par", g, args.pool, 2000 + 100 * rank)
    pool_dev = [torch.from_numpy(base[i % 16] * (1.0 + 1e-3 * i)).to(device) for i in range(args.pool)]
    outs = [torch.empty((g["ny"], g["nx"]), dtype=torch.float32, device=device) for _ in range(4)]

    clk = ClockSampler(local)
    clk.start()
    t_a = time.perf_counter()
    secs, kern, launches = run_device(pipe, pool_dev, outs, args.steps, args.warmup, dist)
    clocks = clk.stop([(t_a, time.perf_counter())])
    secs = dist.max(secs)
    value = replica_value(ws, args.steps, secs)
    # per-kernel pass after the timed region: each stage 100x from a CUDA graph
    kpass, kpass_graph = pipeline_kernel_pass(pipe, pool_dev, outs)

    # ---- e2e through the C ABI with pinned host buffers ----
    pool_host = [t.cpu().pin_memory() for t in pool_dev[:32]]
    e_secs, hb, db = run_e2e(pipe, pool_host, args.steps, args.warmup, (g["ny"], g["nx"]),
                             (g["ny"], g["nx"]), device)
    e_secs = dist.max(e_secs)
    e2e = {"value": replica_value(ws, args.steps, e_secs), "unit": "slices/s", "h2d_bytes_per_step": hb,
           "d2h_bytes_per_step": db}

    extra = {}
    # ---- fan FBP at its headline size ----
    if "fan" in args.legs:
        gf = fan_geometry()
        fpipe = FanPipeline(gf, device)
        fbase = make_pool("fan", gf, 64, 1000 + 100 * rank)
        fpool = [torch.from_numpy(fbase[i % 16] * (1.0 + 1e-3 * i)).to(device) for i in range(64)]
        fouts = [torch.empty((gf["ny"], gf["nx"]), dtype=torch.float32, device=device) for _ in range(4)]
        f_secs, f_kern, f_launches = run_device(fpipe, fpool, fouts, args.steps, args.warmup, dist)
        f_secs = dist.max(f_secs)
        f_pass, _ = pipeline_kernel_pass(fpipe, fpool, fouts)
        fdom = max(f_pass, key=f_pass.get)
        extra["fan_fbp_config1"] = {
            "workload": "fan_weighting -> ramp(fan) -> bp_fan_2d, 720 views x 736 ch -> 512x512",
            "slices_per_s": ws * args.steps / f_secs,
            "updates_per_s": ws * args.steps / f_secs * fpipe.updates,
            "ms_per_step": 1e3 * f_secs / args.steps,
            "kernel_ms": f_pass,
            "kernel_ms_in_run": f_kern,
            "dominant": fdom,
            "dominant_tflops": fpipe.flops[fdom] / (f_pass[fdom] / 1e3) / 1e12,
            "gpu_launches": f_launches,
        }

    # ---- batched uneven fan FBP (config 3) against the plain drop-in ----
    if "batched" in args.legs:
        extra["batched_fan_config3"] = run_batched(device, args.steps, args.warmup, dist)

    # ---- differentiable pair: gradient descent (config 4) ----
    if "gd" in args.legs:
        extra["gd_config4"] = run_gd(device, args.steps, args.warmup, dist)

    # ---- the forward projector's other method (ray casting) ----
    if "fpmethods" in args.legs:
        extra["fp_methods"] = run_fp_methods(device, args.steps, args.warmup, dist)

    # ---- helical rebinning (360LI / 180LI) of a clinical-size scan ----
    if "helical" in args.legs:
        extra["helical"] = run_helical(device, args.steps, args.warmup, dist,
                                       rank == 0 and not args.no_cpu_baseline)

    # ---- FP32 adjoints beside their forwards, and the fan chain's gradient ----
    if "adjoints" in args.legs:
        extra["adjoints"] = run_adjoints(device, dist)

    # ---- single-view backprojection (write-bound) ----
    if "sv" in args.legs:
        extra["bp_par_2d_sv"] = run_single_view(device, dist)

    # ---- reduced-precision large slice (config 5); its FP64 check is CPU
    #      oracle work on rank 0, part of the CPU-baseline leg ----
    if "lowp" in args.legs:
        extra["lowp_config5"] = run_lowp(device, args.steps, args.warmup, dist,
                                         rank == 0 and not args.no_cpu_baseline)

    # ---- roofline of the dominant kernel ----
    peak_meas = fp32_peak_tflops(device)
    clk_max = clocks.get("sm_max_mhz") or 2070.0
    peak_nominal = SM_COUNT * FP32_LANES_PER_SM * 2 * clk_max * 1e6 / 1e12
    dom = max(kpass, key=kpass.get)
    achieved = pipe.flops[dom] / (kpass[dom] / 1e3) / 1e12
    traffic = read_traffic()
    plausible = peak_meas <= 1.1 * peak_nominal
    peak = peak_meas if plausible else peak_nominal
    hbm = hbm_peak_gbs()
    gbs = pipe.bytes[dom] / (kpass[dom] / 1e3) / 1e9
    roofline = {
        "bound": "fp32", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
        "frac": achieved / peak, "traffic": traffic.get(dom),
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per call, "
                          "profiles/ncu_traffic.txt (not measured in this run)",
        "algorithmic_bytes": pipe.bytes[dom],
        "peak_source": ("measured: cuBLAS SGEMM 8192^3, TF32 off, best of 5" if plausible else
                        "nominal: 152 SMs x 128 FP32 lanes x 2 x max SM clock"),
        "peak_nominal": peak_nominal,
        "hbm": {"achieved_gbs": gbs, "peak_gbs": hbm, "frac": gbs / hbm,
                "peak_source": "measured: MEASURED_PEAKS.json hbm_gbs (copy)"},
        "kernel_ms": kpass,
        "kernel_ms_source": "per-stage pass after the timed region: 100 calls per stage replayed "
                            "from a CUDA graph, CUDA events around the replay"
                            + ("" if kpass_graph else " (some stage not capturable: issued directly)"),
        "kernel_sum_ms": sum(kpass.values()),
        "kernel_ms_in_run": kern,
    }
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            v, k, c = cpu_slices_per_s("port", g, 2, os.cpu_count() or 1)
            cpu = {"value": v, "unit": "slices/s", "cores": c, "kind": k,
                   "sample": "2 slices of the same workload (fp_par_2d -> ramp -> bp_par_2d)"}
        if "fan_fbp_config1" in extra:
            extra["fan_fbp_config1"]["dominant_frac"] = extra["fan_fbp_config1"]["dominant_tflops"] / peak
        if not args.no_cpu_baseline:
            # the reference's CPU algorithm beside each configuration
            nt = os.cpu_count() or 1
            cc = cpu_configs(nt)
            gpu = {"fan_fbp_config1": ("slices_per_s", f"slices_per_s_{nt}t"),
                   "batched_fan_config3": ("slices_per_s", f"slices_per_s_{nt}t"),
                   "gd_config4": ("images_per_s", f"images_per_s_{nt}t")}
            for leg, (gk, ck) in gpu.items():
                if leg in extra:
                    cc[leg]["gpu_over_cpu"] = extra[leg][gk] / cc[leg][ck]
            if "lowp_config5" in extra:
                cc["lowp_config5"]["gpu_over_cpu"] = (extra["lowp_config5"]["paths"]["bf16"]["slices_per_s"] /
                                                      cc["lowp_config5"][f"slices_per_s_{nt}t"])
            cc["parallel_config2"]["gpu_over_cpu"] = value / cc["parallel_config2"][f"slices_per_s_{nt}t"]
            extra["cpu_oracle_port"] = dict(cc, threads=nt, kind="port")
        line = {
            "metric": METRIC, "value": value, "unit": "slices/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded random-ellipse phantoms, analytic fan sinograms)",
            "config": {"workload": "parallel drop-in: fp_par_2d 512x512 @0.5mm -> 720 views x 729 "
                                   "bins over pi -> ramp(par) -> bp_par_2d", "batch": 1,
                       "pool_slices": args.pool,
                       "l2": f"inputs larger than L2: {args.pool} distinct 1 MiB slices cycled"},
            "updates_per_s": value * pipe.updates,
            "gpu_launches": launches,
            "e2e": e2e, "roofline": roofline, "clocks": clocks, "cpu_baseline": cpu,
            "extra": extra,
        }
        # kernel self-checks (bit 0 window, 1 queue, 2 bounded wait, 3 alignment): a set
        # bit means some launch skipped work, so its numbers would not stand
        flags = ctypes.c_uint()
        lib.ctr_kernel_flags(ctypes.byref(flags), 1)
        line["kernel_flags"] = flags.value
        if flags.value:
            print(f"bench: kernel self-check flags 0x{flags.value:x}", file=sys.stderr)
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()

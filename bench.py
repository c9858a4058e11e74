#!/usr/bin/env python
"""Dose-convolution throughput on GB300 (one JSON line on rank 0).

Workload (default ``ct256_y90_lu177_i131``): a seeded 256^3 CT-like phantom at
1.5 mm (density + activity), dose-point-kernel convolution with three nuclide
kernels (Y-90 21^3, Lu-177 9^3, I-131 11^3, analytic radial profiles) sharing
one forward transform, density-scaled epilogue.  One step = the three dose
maps of one volume; the metric counts output dose voxels (3 x 256^3 per step).
``sphere128_y90`` is the 128^3 / 2 mm / 15^3 single-kernel water case.

value : device-resident inputs, CUDA events on the launching stream around
        each step, L2 flushed (256 MiB write) between steps outside the events.
e2e   : the same workload through the public API
        (KernelConvolutionCalculator.calculate_dose_rate) from pinned host
        tensors: H2D of activity+density and D2H of the dose maps inside the
        timed region.
roofline : the dominant pass, timed live with CUDA events (pvd_plan_profile)
        over the timed steps; algorithmic bytes from the pass byte model.
cpu_baseline : the reference operator (numpy FFT, float64, single thread)
        on one full-size Y-90 convolution, timed on this host.
``--impl reference`` times that CPU path alone as the reference arm.
unet : the learned heterogeneity correction (rank 0 sub-measurement): NN-corrected
        dose of a 128^3 phantom (plain density-scaled conv + tcgen05 U-Net), its
        tensor-core throughput, a training step, the GPU Monte Carlo run to 1 %
        statistical uncertainty on the same phantom, and ``accuracy``: the network
        trained in the same run on in-repo MC pairs, plain vs corrected dose against
        MC on held-out phantoms.

Multi-GPU (torchrun): independent replicas, one volume per rank per step
(weak scaling); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "dose Gvoxel/s: plain conv vs NN-corrected (≤3% vs MC), % of HBM roofline"
UNIT = "Gvoxel/s"

WORKLOADS = {
    "ct256_y90_lu177_i131": dict(shape=(256, 256, 256), voxel_mm=1.5, phantom="ct",
                                 nuclides=["Y90", "Lu177", "I131"], ksize={"Y90": 21, "Lu177": 9, "I131": 11},
                                 density=True),
    "sphere128_y90": dict(shape=(128, 128, 128), voxel_mm=2.0, phantom="sphere", nuclides=["Y90"],
                          ksize={"Y90": 15}, density=False),
}
PASS_NAMES = ["x_fwd", "y_fwd", "z_fwd_mul_inv", "y_inv", "x_inv"]
PASS_KERNELS = ["kf_x_fwd", "kf_y<0>", "kf_z", "kf_y<1>", "kf_x_inv"]
# dram__bytes_read.sum + dram__bytes_write.sum of one launch of a kernel, from one ncu capture of
# that kernel (one launch, --clock-control none) on this workload, keyed by workload, kernel and
# FFT lengths: the figure is reported only when the run's dominant pass and lengths match the key
# (null otherwise), so a changed kernel or length choice never inherits an old capture.
NCU_DRAM_BYTES_PER_LAUNCH = {
    ("ct256_y90_lu177_i131", "kf_x_inv", (280, 288, 280)): 297_638_912 + 166_278_656,
}


def make_inputs(wl):
    from pyvoxeldosimetry_gb300 import phantoms
    if wl["phantom"] == "ct":
        act, rho = phantoms.ct_phantom(wl["shape"], wl["voxel_mm"], seed=2)
    else:
        act = phantoms.sphere_phantom(wl["shape"], wl["voxel_mm"], seed=1)
        rho = None
    return act, (rho if wl["density"] else None)


def byte_model(shape, kmax, nk, density):
    """Algorithmic HBM bytes per STEP of each pass of the pruned 5-pass R2C pipeline at the
    minimal padding P = N + K - 1 (padding beyond that is the implementation's cost), the
    forward part counted once and the z pass / inverse per kernel:
    x_fwd 4V + A; y_fwd A + By; z By + nk (By + S); y_inv nk (By + A);
    x_inv nk (A + 4V) + 4V density (the density rows are read once for all kernels)."""
    n0, n1, n2 = shape
    p = [n + k - 1 for n, k in zip(shape, kmax)]
    h = p[2] // 2 + 1
    v = n0 * n1 * n2
    a = 8 * n0 * n1 * h
    by = 8 * p[1] * n0 * h
    s = 4 * p[0] * p[1] * h
    m = {
        "x_fwd": 4 * v + a,
        "y_fwd": a + by,
        "z_fwd_mul_inv": by + nk * (by + s),
        "y_inv": nk * (by + a),
        "x_inv": nk * (a + 4 * v) + (4 * v if density else 0),
    }
    m["_per_step"] = sum(m.values())
    m["_compulsory_per_step"] = 4 * v * (1 + (1 if density else 0) + nk) + nk * s
    m["_p_min"] = p
    return m


def link_bound(act_h, out_h, e2e_ms, passes, device_ms, reps=5):
    """The host link's share of one end-to-end step: plain pinned copies of the activity
    (up) and of every slot's dose (down), timed alone with CUDA events, and the
    critical path they set: the activity upload precedes the z pass,
    the passes after the forward ones (z, y inverse, the first inverse-x chunk) run
    before the first dose chunk can go back, and the dose copy-back ends the step
    (the density upload overlaps the forward passes)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())

    def timed(dst, src):
        dst.copy_(src, non_blocking=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ts = []
        for _ in range(reps):
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    a_d = torch.empty(act_h.shape, dtype=torch.float32, device=dev)
    o_d = torch.empty(out_h.shape, dtype=torch.float32, device=dev)
    up_ms = timed(a_d, act_h)
    down_ms = timed(out_h, o_d)
    del a_d, o_d
    mid_ms = sum(passes.get(k, 0.0) for k in ("z_fwd_mul_inv", "y_inv")) + passes.get("x_inv", 0.0) / 4
    bound = up_ms + mid_ms + down_ms
    return {"activity_up_ms": up_ms, "activity_up_gb_s": act_h.numel() * 4 / up_ms / 1e6,
            "dose_down_ms": down_ms, "dose_down_gb_s": out_h.numel() * 4 / down_ms / 1e6,
            "critical_path_ms": bound, "e2e_ms": e2e_ms, "e2e_frac_of_link_bound": bound / e2e_ms,
            "device_resident_ms": device_ms,
            "note": "the host link (about 200 GB/s each way on this box, copy engine or SM loads/stores alike) "
                    "bounds the end-to-end step; the passes between the uploads and the copy-back are taken "
                    "from this run's per-pass times"}


def load_peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback (6.8 TB/s)"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms during the timed region."""

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.path = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu_id, f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": float(np.median(loaded)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference_conv(act, rho, kernel):
    """The reference operator (core/kernel_convolution.py:71-74) in float64 on zero-padded
    inputs, cropped, density-divided: the same linear convolution this package computes."""
    from oracle import conv as oc
    d = oc.linear_conv_same(act.astype(np.float64), kernel)
    return oc.density_scale(d, rho)


def cpu_reference_stock(act, kernel):
    """The reference operator exactly as core/kernel_convolution.py:71-74 runs it: float64,
    unpadded (circular), np.fft.ifftn(np.fft.fftn(A) * np.fft.fftn(K, A.shape)).real."""
    from oracle import conv as oc
    return oc.reference_circular_conv(act.astype(np.float64), kernel)


def oracle_errors(act, rho, wl, dose, refs=None):
    """Max / mean error of each nuclide's dose map (numpy [nk, *shape]) against the FP64
    oracle (checker only, outside every timed region); with a density map also the
    error of the energy per voxel D * rho and of the dose in tissue (rho >= 0.2).
    Returns (errors, refs)."""
    from oracle import conv as oc
    if refs is None:
        refs = oc.linear_conv_same_multi(act, reference_kernels(wl), density=rho)
    errs = {nuc: oc.error_stats(dose[i], refs[i], density=rho) for i, nuc in enumerate(wl["nuclides"])}
    return errs, refs


def reference_kernels(wl):
    from pyvoxeldosimetry_gb300.data import nuclides as nd
    out = []
    for nuc in wl["nuclides"]:
        k = nd.analytic_profile(nuc, wl["voxel_mm"], (wl["ksize"][nuc],) * 3)
        out.append(k / k.sum() * nd.gy_per_bq_s_scale(nuc, wl["voxel_mm"]))
    return out


_REF = {}


def _ref_init(workload):
    """Reference-arm worker: the seeded phantom and kernels, built once per process."""
    wl = WORKLOADS[workload]
    _REF["act"], _REF["rho"] = make_inputs(wl)
    _REF["ks"] = reference_kernels(wl)


def _ref_conv(i):
    cpu_reference_conv(_REF["act"], _REF["rho"], _REF["ks"][i % len(_REF["ks"])])
    return i


def _ref_stock(i):
    cpu_reference_stock(_REF["act"], _REF["ks"][i % len(_REF["ks"])])
    return i


def reference_workers(shape) -> int:
    """Host cores to run reference convolutions on: all of them, bounded by the memory
    one float64 FFT convolution of this shape needs (about 10 padded complex volumes)."""
    cores = os.cpu_count() or 1
    per = 10 * 16 * int(np.prod([n + 20 for n in shape]))
    try:
        with open("/proc/meminfo") as f:
            avail = next(int(l.split()[1]) * 1024 for l in f if l.startswith("MemAvailable:"))
        cores = max(1, min(cores, int(0.8 * avail // per)))
    except (OSError, StopIteration, ValueError):
        pass
    return cores


def run_reference(args, wl, rank):
    """Reference arm: the reference's CPU convolution operator on this host's cores.  numpy's
    FFT runs on one thread, so the cores are used the way a reference user would use them for
    many volumes: one full-size nuclide convolution per worker process, all at once; a step is
    one convolution on every worker.  The line's value is the operator exactly as the
    reference runs it (unpadded, circular: core/kernel_convolution.py:71-74); ``padded_linear``
    times the same operator on zero-padded inputs with the density divide, which is the
    linear convolution this package computes (fewer steps: it is only reported)."""
    if rank != 0:
        return
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    workers = reference_workers(wl["shape"])
    vox = int(np.prod(wl["shape"]))

    def timed(ex, fn, steps, warmup):
        for w in range(warmup):
            list(ex.map(fn, range(w * workers, (w + 1) * workers)))
        times = []
        for i in range(steps):
            t0 = time.perf_counter()
            list(ex.map(fn, range(i * workers, (i + 1) * workers)))
            times.append(time.perf_counter() - t0)
        return float(np.sum(times))

    with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn"),
                             initializer=_ref_init, initargs=(args.workload,)) as ex:
        t = timed(ex, _ref_stock, args.steps, args.warmup)
        pad_steps = min(args.steps, 3)
        t_pad = timed(ex, _ref_conv, pad_steps, 1)
    value = vox * workers * args.steps / t / 1e9
    value_pad = vox * workers * pad_steps / t_pad / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded phantom)",
        "config": config_dict(args.workload, wl),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                         "sample": f"per step one full {wl['shape']} convolution on each of {workers} worker "
                                   "processes (nuclides in turn): the reference operator exactly as "
                                   "kernel_convolution.py:71-74 runs it, numpy float64, unpadded circular"},
        "padded_linear": {"value": value_pad, "unit": UNIT, "steps": pad_steps, "cores": workers,
                          "ms_per_step": 1e3 * t_pad / pad_steps,
                          "sample": "the same operator on zero-padded inputs (P = N + K - 1), cropped, density "
                                    "divide: the linear density-scaled convolution the GPU arm computes"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def max_over_ranks(ms: float, device=None) -> float:
    """Elapsed time of the slowest rank (the job's time); identity without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world: int, units_per_rank_step: int, steps: int, max_ms: float) -> float:
    """Whole-job Gvoxel/s: every rank processes its own replica each step (weak scaling)."""
    return world * units_per_rank_step * steps / (max_ms / 1e3) / 1e9


def measure_mc(device, n_hist=10_000_000, reps=3):
    """GPU Monte Carlo throughput: Lu-177 (beta + gammas) on a 128^3 CT-like phantom at 3 mm."""
    import torch
    from pyvoxeldosimetry_gb300 import phantoms
    from pyvoxeldosimetry_gb300.core.monte_carlo import McPlan, physics_tables
    act, rho = phantoms.ct_phantom((128, 128, 128), 3.0, seed=4)
    a = torch.from_numpy(act).to(device)
    r = torch.from_numpy(rho).to(device)
    plan = McPlan(act.shape, (3.0, 3.0, 3.0), physics_tables("Lu177"), device)
    plan.run(a, r, n_hist // 10, 1, dose=True)
    ms = []
    for i in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _, _, st = plan.run(a, r, n_hist, 100 + i, dose=True, stats=False)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    plan.close()
    t = float(np.median(ms))
    return {"value": n_hist / (t / 1e3) / 1e6, "unit": "Mhistories/s", "ms_per_run": t, "histories": n_hist,
            "workload": "Lu-177 beta+gamma, 128^3 CT phantom at 3 mm, dose-rate map included",
            "parity": "unpinned against the reference (its Monte Carlo cannot run); energy grids bit-identical to "
                      "this package's C restatement of the same transport"}


def measure_fit(device, shape=(256, 256, 256), reps=2):
    """Per-voxel FP64 mono-exponential fit (+ AUC) throughput, 4 timepoints of bi-exponential washout."""
    import torch
    from pyvoxeldosimetry_gb300.time_integration import TimeCurveFitting
    times = [1.0, 4.0, 24.0, 96.0]
    g = torch.Generator(device=device).manual_seed(3)
    a0 = torch.rand(shape, generator=g, device=device) * 1e4 + 1e2
    l1 = 0.6931 / (6.0 * (160.0 / 6.0) ** torch.rand(shape, generator=g, device=device))
    l2 = 0.6931 / (6.0 * (160.0 / 6.0) ** torch.rand(shape, generator=g, device=device))
    w = 0.2 + 0.6 * torch.rand(shape, generator=g, device=device)
    acts = torch.stack([a0 * (w * torch.exp(-l1 * t) + (1 - w) * torch.exp(-l2 * t)) for t in times]).contiguous()
    tf = TimeCurveFitting(64.1)
    tf.fit_time_activity_curve(times, acts[:, :8, :, :].contiguous())
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        tf.fit_time_activity_curve(times, acts)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = float(np.median(ms))
    nv = int(np.prod(shape))
    return {"value": nv / (t / 1e3) / 1e9, "unit": "Gvoxel/s", "ms_per_run": t, "voxels": nv,
            "workload": "mono-exponential FP64 fit + AUC per voxel, 4 timepoints, 256^3"}


def measure_vp_fit(device, shape=(256, 256, 256), reps=2):
    """Per-voxel two-exponential fit by variable projection (FP32 iterations finished in
    FP64) + analytic AUC, 4 timepoints of bi-exponential washout, half-lives 6..160 h."""
    import ctypes as C
    import torch
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    times = [1.0, 4.0, 24.0, 96.0]
    g = torch.Generator(device=device).manual_seed(3)
    u = lambda: torch.rand(shape, generator=g, device=device)
    a0 = u() ** 2 * 1e4 + 10.0
    l1 = 0.6931471805599453 / (6.0 * (160.0 / 6.0) ** u())
    l2 = 0.6931471805599453 / (6.0 * (160.0 / 6.0) ** u())
    w = 0.2 + 0.6 * u()
    acts = torch.stack([a0 * (w * torch.exp(-l1 * t) + (1 - w) * torch.exp(-l2 * t)) for t in times]).contiguous()
    del a0, l1, l2, w
    nv = int(np.prod(shape))
    params = torch.empty((4, nv), dtype=torch.float64, device=device)
    auc = torch.empty(nv, dtype=torch.float64, device=device)
    ok = torch.empty(nv, dtype=torch.uint8, device=device)
    t = (C.c_double * 4)(*times)
    p0 = (C.c_double * 5)(1.0, 0.1, 0.5, 0.01, 0.0)
    flags = N.PVD_FIT_P0_FROM_DATA | N.PVD_FIT_AUC_INF | N.PVD_FIT_VARPRO | N.PVD_FIT_MIXED
    ms = []
    for _ in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        N.check(lib.pvd_tac_fit(N.PVD_FIT_F4A, t, None, 4, p0, 0.0, 0.0, 2000, flags, acts.data_ptr(), nv,
                                params.data_ptr(), auc.data_ptr(), ok.data_ptr(), None, 1.0,
                                torch.cuda.current_stream(device).cuda_stream))
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    tm = float(np.median(ms[1:]))
    return {"value": nv / (tm / 1e3) / 1e9, "unit": "Gvoxel/s", "ms_per_run": tm, "voxels": nv,
            "converged_fraction": float(ok.float().mean()),
            "workload": f"two-exponential fit by variable projection (FP32 then FP64) + analytic AUC, "
                        f"4 timepoints, {shape[0]}x{shape[1]}x{shape[2]}"}


def measure_dvh(device, shape=(256, 256, 256), bins=1000, reps=5):
    """Dose-volume histogram (calculate_dvh): ROI statistics, numpy's edges and the
    histogram on the GPU, cumulative sum on the host; 10 algorithmic bytes per voxel
    (two passes over a float32 dose and a uint8 mask)."""
    import torch
    from pyvoxeldosimetry_gb300.core.utils import calculate_dvh
    g = torch.Generator(device=device).manual_seed(9)
    dose = torch.rand(shape, generator=g, device=device) * 60.0
    mask = (torch.rand(shape, generator=g, device=device) > 0.3).to(torch.uint8)
    calculate_dvh(dose, mask, bins)
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        calculate_dvh(dose, mask, bins)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    t = float(np.median(ms))
    nv = int(np.prod(shape))
    peak, _ = load_peaks()
    return {"value": nv / (t / 1e3) / 1e9, "unit": "Gvoxel/s", "ms_per_call": t, "voxels": nv, "bins": bins,
            "hbm_frac": 10.0 * nv / (t / 1e3) / 1e9 / peak,
            "workload": f"calculate_dvh, {shape[0]}x{shape[1]}x{shape[2]} float32 dose, uint8 ROI of 70 %, "
                        "whole call (statistics, edges and histogram on the device, one copy back)"}


def measure_resample(device, shape=(256, 256, 256), reps=5):
    """Cubic B-spline resampling 1.5 mm -> 2.0 mm and 2.0 mm -> 1.5 mm of a 256^3
    float32 volume (resample_volume: copy, 3 prefilter passes, evaluation)."""
    import torch
    from pyvoxeldosimetry_gb300.core.utils import resample_volume, resampled_shape
    g = torch.Generator(device=device).manual_seed(5)
    vol = torch.rand(shape, generator=g, device=device)
    res = {}
    for name, a, b in (("down_1.5_to_2.0", 1.5, 2.0), ("up_2.0_to_1.5", 2.0, 1.5)):
        resample_volume(vol, (a,) * 3, (b,) * 3)
        ms = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            resample_volume(vol, (a,) * 3, (b,) * 3)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        t = float(np.median(ms))
        m = int(np.prod(resampled_shape(shape, (a,) * 3, (b,) * 3)))
        n = int(np.prod(shape))
        # clone 8 B, prefilter 3 x 8 B per input voxel; evaluation reads the coefficients
        # (4 B per input voxel at best) and writes 4 B per output voxel
        peak, _ = load_peaks()
        bytes_ = 36 * n + 4 * m
        res[name] = {"ms": t, "out_gvox_s": m / (t / 1e3) / 1e9, "hbm_frac": bytes_ / (t / 1e3) / 1e9 / peak}
    return {"value": res["down_1.5_to_2.0"]["out_gvox_s"], "unit": "Gvoxel/s (output)", "cases": res,
            "workload": "resample_volume order 3, 256^3 float32, whole call"}


def measure_unet(device, small=False, train_steps=1000, reps=3):
    """Learned correction: one training step (forward, both gradients, Adam) on a
    64^3 crop, NN-corrected dose (plain density-scaled convolution + U-Net +
    apply) of a 128^3 CT-like phantom at 3 mm, and the GPU Monte Carlo run to 1 %
    statistical uncertainty on the same phantom (median relative standard error
    over voxels above 10 % of the maximum, from 10 independent batches)."""
    import torch
    from pyvoxeldosimetry_gb300 import phantoms
    from pyvoxeldosimetry_gb300.core import learned_correction as lc
    from pyvoxeldosimetry_gb300.core.kernel_convolution import KernelConvolutionCalculator
    from pyvoxeldosimetry_gb300.core.monte_carlo import McPlan, physics_tables
    pf = ROOT / "MEASURED_PEAKS.json"
    tc_peak, tc_src = 1900.0, "fallback (1.9 PFLOP/s bf16 burst)"
    if pf.exists():
        tc_peak, tc_src = float(json.loads(pf.read_text())["bf16_tflops"]), "measured (MEASURED_PEAKS.json bf16_tflops)"

    shape = (64, 64, 64) if small else (128, 128, 128)
    crop = (32, 32, 32) if small else (64, 64, 64)
    vox = (3.0, 3.0, 3.0)
    act, rho = phantoms.ct_phantom(shape, 3.0, seed=7)
    a = torch.from_numpy(act).to(device)
    r = torch.from_numpy(rho).to(device)
    conv = KernelConvolutionCalculator("Y90")
    dc = conv.calculate_dose_rate(a, vox, density=r)
    dcn = dc.cpu().numpy()
    pair = lc.make_pair(act, rho, dcn, dcn * 1.1, device=device)
    net = lc.UNet3D(seed=1, device=device)
    # inference first (so a launch list of this run starts with it): plain conv +
    # network + apply on the whole phantom
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = torch.empty_like(dc)
    lc.predict(net, a, r, dc, out=out)
    inf_ms, conv_ms = [], []
    for _ in range(reps):
        e0.record()
        d = conv.calculate_dose_rate(a, vox, density=r)
        e1.record()
        e1.synchronize()
        conv_ms.append(e0.elapsed_time(e1))
        e0.record()
        lc.predict(net, a, r, d, out=out)
        e1.record()
        e1.synchronize()
        inf_ms.append(e0.elapsed_time(e1))
    # the calculator's default: the prediction averaged over the 8 grid flips
    lc.predict(net, a, r, dc, out=out, symmetries=8)
    inf8_ms = []
    for _ in range(reps):
        e0.record()
        lc.predict(net, a, r, dc, out=out, symmetries=8)
        e1.record()
        e1.synchronize()
        inf8_ms.append(e0.elapsed_time(e1))
    conv_t, inf_t, inf8_t = float(np.median(conv_ms)), float(np.median(inf_ms)), float(np.median(inf8_ms))
    # whole training steps through the library's loop (focused crop, forward, loss, both
    # gradients, clipping, Adam), host clock around the loop with a device sync at its end:
    # forward and layer backward replayed as CUDA graphs (the default), and eager
    lc.train(net, [pair], 3, crop=crop)
    step_ms = lc.train(net, [pair], train_steps, crop=crop, lr=1e-4).seconds / train_steps * 1e3
    eager_ms = lc.train(net, [pair], train_steps // 4, crop=crop, lr=1e-4, graphs=False).seconds / (
        train_steps // 4) * 1e3
    # forward + data gradient (all but the first layer) + weight gradient
    fwd = lc.conv_flops(crop)
    first = 2.0 * 27 * 16 * 16 * crop[0] * crop[1] * crop[2]
    step_flops = 3 * fwd - first
    infer_crop = tuple(-(-n // 8) * 8 for n in shape)
    nvox = float(np.prod(shape))
    # Monte Carlo to 1 %: 10 batches, relative standard error of the mean per voxel
    plan = McPlan(shape, vox, physics_tables("Y90"), device)
    hb = 2_000_000 if small else 10_000_000
    batches = []
    e0.record()
    for b in range(10):
        _, dr, _ = plan.run(a, r, hb, 1000 + b, dose=True)
        batches.append(dr.cpu().numpy().astype(np.float64))
    e1.record()
    e1.synchronize()
    mc_ms = e0.elapsed_time(e1)
    plan.close()
    conv.close()
    net.status()
    large = None if small else measure_unet_large(device, net)
    st = np.stack(batches)
    mean = st.mean(0)
    sel = mean > 0.1 * mean.max()
    rse = st.std(0, ddof=1)[sel] / np.sqrt(10) / mean[sel]
    rse_med = float(np.median(rse))
    mc_1pct_ms = mc_ms * (rse_med / 0.01) ** 2
    nn_ms = conv_t + inf8_t
    return {
        "value": nvox / (nn_ms / 1e3) / 1e9, "unit": "Gvoxel/s (NN-corrected dose)",
        "workload": f"Y-90, {list(shape)} CT-like phantom at 3 mm: density-scaled conv + U-Net "
                    f"(4 levels, 16-128 ch) averaged over the 8 grid flips + apply; training step on a "
                    f"{list(crop)} crop",
        "plain_conv_ms": conv_t, "unet_inference_ms": inf_t, "unet_inference_8_flips_ms": inf8_t,
        "nn_corrected_ms": nn_ms, "nn_corrected_single_pass_ms": conv_t + inf_t,
        "plain_conv_gvox_s": nvox / (conv_t / 1e3) / 1e9,
        "unet_inference_tflops": lc.conv_flops(infer_crop) / (inf_t / 1e3) / 1e12,
        "train_step_ms": step_ms, "train_step_eager_ms": eager_ms,
        "train_step_tflops": step_flops / (step_ms / 1e3) / 1e12,
        "train_tensor_frac": step_flops / (step_ms / 1e3) / 1e12 / tc_peak,
        "tensor_peak_tflops": tc_peak, "tensor_peak_source": tc_src,
        "mc_histories_per_batch": hb, "mc_ms_10_batches": mc_ms, "mc_median_rel_se": rse_med,
        "mc_to_1pct_ms": mc_1pct_ms, "nn_vs_mc_1pct_speedup": mc_1pct_ms / nn_ms,
        "whole_body_512x512x400": large,
        "parity": "U-Net layers checked against a float64 restatement of this package's own network (the "
                  "reference has none: unpinned against the reference); MC unpinned as in 'mc'",
    }


def measure_unet_large(device, net, reps=2):
    """NN-corrected dose of one whole-body 512x512x400 volume at 1.5 mm (the whole-body
    inference size): plain density-scaled Y-90 convolution + U-Net (single pass, and
    averaged over the 8 grid flips) + apply, CUDA events around each call, inputs
    resident."""
    import torch
    from pyvoxeldosimetry_gb300 import phantoms
    from pyvoxeldosimetry_gb300.core import learned_correction as lc
    from pyvoxeldosimetry_gb300.core.kernel_convolution import KernelConvolutionCalculator
    shape, vox = (400, 512, 512), (1.5, 1.5, 1.5)
    act, rho = phantoms.ct_phantom(shape, 1.5, seed=11)
    a = torch.from_numpy(act).to(device)
    r = torch.from_numpy(rho).to(device)
    del act, rho
    conv = KernelConvolutionCalculator("Y90")
    out = torch.empty(shape, dtype=torch.float32, device=device)
    d = conv.calculate_dose_rate(a, vox, density=r)
    lc.predict(net, a, r, d, out=out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    conv_ms, inf_ms = [], []
    for _ in range(reps):
        e0.record()
        d = conv.calculate_dose_rate(a, vox, density=r)
        e1.record()
        e1.synchronize()
        conv_ms.append(e0.elapsed_time(e1))
        e0.record()
        lc.predict(net, a, r, d, out=out)
        e1.record()
        e1.synchronize()
        inf_ms.append(e0.elapsed_time(e1))
    e0.record()
    lc.predict(net, a, r, d, out=out, symmetries=8)
    e1.record()
    e1.synchronize()
    inf8 = e0.elapsed_time(e1)
    net.status()
    kshape = conv._kernel_specs(vox)[0][0].shape
    conv.close()
    c, i = float(np.median(conv_ms)), float(np.median(inf_ms))
    nvox = float(np.prod(shape))
    res = {"shape": list(shape), "plain_conv_ms": c, "unet_inference_ms": i, "nn_corrected_ms": c + i,
           "nn_corrected_gvox_s": nvox / ((c + i) / 1e3) / 1e9, "unet_inference_8_flips_ms": inf8,
           "nn_corrected_8_flips_ms": c + inf8,
           "unet_inference_tflops": lc.conv_flops(shape) / (i / 1e3) / 1e12,
           "device_memory_peak_gb": torch.cuda.max_memory_allocated(device) / 1e9}
    # plain convolution against the FP64 oracle on a slab of 16 z planes through the middle:
    # the linear convolution of the input planes within the kernel's reach of the slab
    # gives the exact dose of the slab's planes (checker, outside the timed region)
    from oracle import conv as oc
    from pyvoxeldosimetry_gb300.data import nuclides as nd
    z0, nz, hz = shape[0] // 2 - 8, 16, kshape[0] // 2
    act_s = a[z0 - hz:z0 + nz + hz].cpu().numpy()
    rho_s = r[z0 - hz:z0 + nz + hz].cpu().numpy()
    kk = nd.analytic_profile("Y90", vox, kshape)
    ref = oc.linear_conv_same_multi(act_s, [kk / kk.sum() * nd.gy_per_bq_s_scale("Y90", vox)], density=rho_s)[0]
    res["plain_conv_error_vs_fp64_oracle"] = dict(oc.error_stats(d[z0:z0 + nz].cpu().numpy(), ref[hz:hz + nz],
                                                                 density=rho_s[hz:hz + nz]),
                                                  slab=f"z {z0}..{z0 + nz - 1} of {shape[0]}")
    net._ws.clear()
    del a, r, d, out
    torch.cuda.empty_cache()
    return res


UNET_ACCURACY_STEPS = {"Y90": 120000, "Lu177": 40000}


def measure_unet_accuracy(device, small=False, n_train=128, steps=None, nuclides=("Y90", "Lu177")):
    """What the learned correction gains, measured in the same run, per nuclide: the U-Net
    trained on this package's own pairs (seeded 128^3 CT-like phantoms at 3 mm — the kind
    the MC-to-1 % time is measured on — density-scaled convolution at the Monte Carlo's
    energy per decay vs GPU Monte Carlo with 1e8 histories; Y-90 betas, Lu-177 betas and
    gammas; crops centred on weighted voxels; UNET_ACCURACY_STEPS Adam steps unless
    ``steps`` says otherwise), judged on 10 held-out phantoms against Monte Carlo with
    4e8 histories (about 0.4 % statistical uncertainty in the judged voxels), tissue
    voxels above 10 % of the tissue maximum: relative error of the plain dose, of the
    corrected dose averaged over the 8 grid flips (the calculator's default) and of the
    single-pass corrected dose."""
    from pyvoxeldosimetry_gb300.core import learned_correction as lc
    shape, vox = ((48, 48, 48), 4.0) if small else ((128, 128, 128), 3.0)
    n_held, hist_held = (2, 200_000_000) if small else (10, 400_000_000)
    if small:
        n_train, steps = 4, 300
    hist = 20_000_000 if small else 100_000_000
    crop = shape if small else (64, 64, 64)
    out = {}
    for nuc in nuclides:
        t0 = time.perf_counter()
        n_steps = steps or UNET_ACCURACY_STEPS.get(nuc, 40000)
        pairs = lc.generate_training_pairs(n_train, shape, vox, nuc, histories=hist, seed=100, device=device)
        held = lc.generate_training_pairs(n_held, shape, vox, nuc, histories=hist_held, seed=900, device=device)
        net = lc.UNet3D(seed=0, device=device)
        st = lc.train(net, pairs, n_steps, crop=crop, lr=5e-4)
        res = {"plain": [], "corrected": [], "corrected_single_pass": []}
        for p in held:
            corr = lc.predict(net, p.activity, p.density, p.dose_conv, sigma_max=float("inf"), symmetries=8)
            single = lc.predict(net, p.activity, p.density, p.dose_conv, sigma_max=float("inf"))
            mc, rho = p.dose_mc.cpu().numpy(), p.density.cpu().numpy()
            res["plain"].append(lc.dose_errors(p.dose_conv.cpu().numpy(), mc, density=rho))
            res["corrected"].append(lc.dose_errors(corr.cpu().numpy(), mc, density=rho))
            res["corrected_single_pass"].append(lc.dose_errors(single.cpu().numpy(), mc, density=rho))
        net.status()
        # the reference Monte Carlo's own noise: a second, independent run on the first held-out
        # phantoms against the first (their difference carries sqrt(2) x one run's noise;
        # within 3 sqrt(2) % is where an exact prediction would land within 3 % of one run)
        from pyvoxeldosimetry_gb300.core.monte_carlo import MonteCarloCalculator
        mc2 = MonteCarloCalculator(nuc, n_particles=hist_held)
        floor = []
        for k, p in enumerate(held[:2]):
            d2 = mc2.calculate_dose_rate(p.activity, (vox,) * 3, density=p.density, seed=5000 + k).cpu().numpy()
            rho = p.density.cpu().numpy()
            e = lc.dose_errors(d2, p.dose_mc.cpu().numpy(), density=rho)
            sel_err = np.abs(d2.astype(np.float64) - p.dose_mc.cpu().numpy()) / np.maximum(p.dose_mc.cpu().numpy(), 1e-30)
            tissue = (rho >= lc.TISSUE_DENSITY)
            ref = p.dose_mc.cpu().numpy()
            m = tissue & (ref > 0.1 * ref[tissue].max())
            floor.append((e["within_3pct"], float((sel_err[m] <= 0.03 * np.sqrt(2)).mean())))
        mc2.close()
        agg = {k: {m: float(np.mean([e[m] for e in v])) for m in ("mean", "median", "p95", "within_3pct")}
               for k, v in res.items()}
        out[nuc] = {"train_steps": n_steps, "train_phantoms": n_train, "train_seconds": st.seconds,
                    "skipped_steps": st.skipped, "total_seconds": time.perf_counter() - t0,
                    "held_out_phantoms": len(held), "plain_vs_mc": agg["plain"], "corrected_vs_mc": agg["corrected"],
                    "corrected_single_pass_vs_mc": agg["corrected_single_pass"], "symmetries": 8,
                    "worst_phantom_within_3pct": float(min(e["within_3pct"] for e in res["corrected"])),
                    "mc_vs_mc_within_3pct": float(np.mean([f[0] for f in floor])),
                    "exact_prediction_within_3pct_estimate": float(np.mean([f[1] for f in floor])),
                    "histories_per_training_phantom": hist, "histories_per_judging_phantom": hist_held}
        del pairs, held, net
    out["workload"] = (f"{list(shape)} CT-like phantoms at {vox} mm; judged: tissue voxels (density >= 0.2) above "
                       "10 % of the tissue maximum, relative error to Monte Carlo")
    return out


def run_only(args, device):
    """One sub-measurement alone (a bounded case to profile), printed as its own JSON line."""
    small = args.small
    if args.only == "mc":
        r = measure_mc(device, n_hist=1_000_000 if small else 10_000_000)
    elif args.only == "fit":
        r = measure_fit(device, shape=(128, 128, 128) if small else (256, 256, 256))
    elif args.only == "resample":
        r = measure_resample(device, shape=(128, 128, 128) if small else (256, 256, 256))
    elif args.only == "dvh":
        r = measure_dvh(device, shape=(128, 128, 128) if small else (256, 256, 256))
    elif args.only == "vpfit":
        r = measure_vp_fit(device, shape=(64, 128, 128) if small else (256, 256, 256))
    elif args.only == "unet":
        r = measure_unet(device, small=small)
        r["accuracy"] = measure_unet_accuracy(device, small=small, n_train=args.unet_train_phantoms)
    else:
        r = measure_batch(device, 2 if small else args.batch_volumes)
    print(json.dumps({"only": args.only, "small": small, **r}), flush=True)


def batch_volumes(device, n_volumes=64, seed=3, times=(1.0, 4.0, 24.0, 96.0), n_draw=64):
    """Uneven batch: n0, n1 ~ U{96..320}, n2 ~ U{96..256} (seeded), 4 timepoints of
    per-voxel bi-exponential washout A0 (w e^{-l1 t} + (1-w) e^{-l2 t}), half-lives
    log-uniform in [6, 160] h, w ~ U(0.2, 0.8), generated on the device."""
    import torch
    rng = np.random.default_rng(seed)
    shapes = [(int(rng.integers(96, 321)), int(rng.integers(96, 321)), int(rng.integers(96, 257)))
              for _ in range(max(n_draw, n_volumes))]
    vols = []
    for i in range(n_volumes):
        shape = shapes[i]
        g = torch.Generator(device=device).manual_seed(seed * 1000 + i)
        u = lambda: torch.rand(shape, generator=g, device=device)
        a0 = u() ** 2 * 1e4 + 10.0
        l1 = 0.6931471805599453 / (6.0 * (160.0 / 6.0) ** u())
        l2 = 0.6931471805599453 / (6.0 * (160.0 / 6.0) ** u())
        w = 0.2 + 0.6 * u()
        acts = torch.stack([a0 * (w * torch.exp(-l1 * t) + (1 - w) * torch.exp(-l2 * t)) for t in times])
        vols.append({"activity": acts.contiguous(), "times": list(times), "voxel_size": (1.5, 1.5, 1.5)})
        del a0, l1, l2, w
    return vols


def measure_batch(device, n_volumes=64, reps=2):
    """Batched time-integrated dose of the seeded uneven workload: per-voxel two-exponential
    fit (variable projection: FP32 iterations, FP64 Gauss-Newton polish, FP64 trust region
    for what the polish leaves) + analytic AUC + Y-90 convolution at autotuned FFT lengths
    of every volume, recorded once as a CUDA graph and launched as one.  The stages are
    also timed apart (every fit, then every convolution) for the fit's Mvoxel/s and the
    convolution stage's HBM fraction."""
    import torch
    from pyvoxeldosimetry_gb300 import _native as N
    from pyvoxeldosimetry_gb300.batch import BatchDoseCalculator
    from pyvoxeldosimetry_gb300.data import nuclides as nd
    t0 = time.perf_counter()
    vols = batch_volumes(device, n_volumes)
    nvox = sum(int(np.prod(v["activity"].shape[1:])) for v in vols)
    bc = BatchDoseCalculator("Y90", use_graph=True, autotune=True, device=device)
    bc.prepare(vols)
    setup_s = time.perf_counter() - t0
    lib = N.load()
    ms = []
    for _ in range(reps + 1):
        lib.pvd_launch_count(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        bc.run()
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    launches = int(lib.pvd_launch_count(1))
    fit_ms, conv_ms = bc.run_stages()
    ok = float(sum(float(bc.fit_results(i)[2].float().mean()) * np.prod(v["activity"].shape[1:])
                   for i, v in enumerate(vols)) / nvox)
    peak, _ = load_peaks()
    ks = nd.default_kernel_size("Y90", (1.5, 1.5, 1.5))
    conv_bytes = sum(byte_model(tuple(v["activity"].shape[1:]), ks, 1, False)["_per_step"] for v in vols)
    lengths = sorted({tuple(p.fft_shape) for p in bc.plans()})
    bc.close()
    del vols
    torch.cuda.empty_cache()
    t = float(np.median(ms[1:]))
    return {"value": nvox / (t / 1e3) / 1e9, "unit": "Gvoxel/s", "ms_per_batch": t, "volumes": n_volumes,
            "voxels": nvox, "gpu_launches_per_batch": launches, "fit_converged_fraction": ok,
            "fit_ms": fit_ms, "fit_mvoxel_s": nvox / (fit_ms / 1e3) / 1e6,
            "conv_ms": conv_ms, "conv_gvoxel_s": nvox / (conv_ms / 1e3) / 1e9,
            "conv_hbm_frac": conv_bytes / (conv_ms / 1e3) / 1e9 / peak, "conv_algorithmic_bytes": conv_bytes,
            "distinct_fft_shapes": len(lengths), "setup_s": setup_s,
            "workload": f"{n_volumes} seeded volumes 96..320 x 96..320 x 96..256 at 1.5 mm, 4 timepoints (1, 4, 24, "
                        "96 h), Y-90 21^3, autotuned FFT lengths per volume shape, one graph launch"}


def config_dict(name, wl):
    return {"workload": name, "shape": list(wl["shape"]), "voxel_mm": wl["voxel_mm"],
            "kernels": {n: [wl["ksize"][n]] * 3 for n in wl["nuclides"]}, "density_scaled": wl["density"],
            "voxels_per_step": int(np.prod(wl["shape"])) * len(wl["nuclides"]),
            "l2": "flushed between timed steps (256 MiB write, outside the events)",
            "parallelism": "replicas (one volume per GPU)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ct256_y90_lu177_i131", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-check", action="store_true", help="skip the error check against the FP64 oracle")
    ap.add_argument("--pads", help="explicit FFT lengths P0,P1,P2 (default: the autotuner's choice)")
    ap.add_argument("--unet-train-phantoms", type=int, default=128,
                    help="seeded 128^3 phantoms (x 1e8 MC histories) the learned correction trains on per nuclide")
    ap.add_argument("--no-extras", action="store_true", help="skip the MC, fit and batch sub-measurements")
    ap.add_argument("--batch-volumes", type=int, default=64,
                    help="volumes of the 64-volume seeded uneven batch to run in the batch sub-measurement")
    ap.add_argument("--only", choices=["mc", "fit", "vpfit", "batch", "dvh", "resample", "unet"],
                    help="run one sub-measurement alone and print it (no contract line)")
    ap.add_argument("--small", action="store_true", help="with --only: a bounded case for profiling")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    wl = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, wl, rank)
        return

    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local_rank)
    device = torch.device("cuda", local_rank)
    if world > 1:
        dist.init_process_group("nccl", device_id=device)

    if args.only:
        run_only(args, device)
        return

    from pyvoxeldosimetry_gb300 import _native as N
    from pyvoxeldosimetry_gb300.core.kernel_convolution import KernelConvolutionCalculator

    lib = N.load()
    act, rho = make_inputs(wl)
    shape = wl["shape"]
    vox = int(np.prod(shape))
    nk = len(wl["nuclides"])
    vs = (wl["voxel_mm"],) * 3
    cfg = {"kernel_size": wl["ksize"], "device": device}
    if args.pads:  # explicit FFT lengths instead of the autotuner's
        cfg["autotune"] = False
        cfg["pads"] = tuple(int(x) for x in args.pads.split(","))
    calc = KernelConvolutionCalculator(wl["nuclides"], config=cfg)
    plan = calc._plan_for(shape, vs, device)
    act_d = torch.from_numpy(act).to(device)
    rho_d = torch.from_numpy(rho).to(device) if rho is not None else None
    out_d = torch.empty((nk, *shape), dtype=torch.float32, device=device)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=device)  # 256 MiB > 129 MB L2

    def barrier():
        if world > 1:
            dist.barrier()

    for i in range(args.warmup):
        flush.fill_(float(i))
        plan.execute(act_d, density=rho_d, out=out_d)
    torch.cuda.synchronize()

    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    N.check(lib.pvd_plan_profile(plan._h, 1))
    lib.pvd_launch_count(1)
    gpu_id = str(local_rank)
    try:
        uuid = str(torch.cuda.get_device_properties(device).uuid)
        gpu_id = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
    except Exception:
        pass
    with ClockSampler(gpu_id) as clk:
        barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.fill_(float(i))
            evs[i][0].record(stream)
            plan.execute(act_d, density=rho_d, out=out_d)
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        barrier()
    launches = int(lib.pvd_launch_count(0))
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = max_over_ranks(float(np.sum(step_ms)), device)
    ms_arr = (ctypes.c_double * 5)()
    cnt_arr = (ctypes.c_int * 5)()
    N.check(lib.pvd_plan_pass_times(plan._h, ms_arr, cnt_arr))
    N.check(lib.pvd_plan_profile(plan._h, 0))
    pass_ms = {PASS_NAMES[i]: float(ms_arr[i]) for i in range(5)}
    pass_n = {PASS_NAMES[i]: int(cnt_arr[i]) for i in range(5)}
    value = job_throughput(world, nk * vox, args.steps, total_ms)

    # roofline of the dominant pass
    kmax = [max(wl["ksize"][n] for n in wl["nuclides"])] * 3
    bm = byte_model(shape, kmax, nk, wl["density"])
    peak, peak_src = load_peaks()
    dom = max(PASS_NAMES, key=lambda k: pass_ms[k])
    avg_s = pass_ms[dom] / max(pass_n[dom], 1) / 1e3
    launch_bytes = bm[dom] * args.steps / max(pass_n[dom], 1)  # the pass's bytes per step over its launches
    achieved = launch_bytes / avg_s / 1e9
    traffic = NCU_DRAM_BYTES_PER_LAUNCH.get((args.workload, PASS_KERNELS[PASS_NAMES.index(dom)],
                                             tuple(plan.fft_shape)))
    step_s = total_ms / args.steps / 1e3
    roofline = {"bound": "hbm", "kernel": PASS_KERNELS[PASS_NAMES.index(dom)], "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "algorithmic_bytes_per_launch": launch_bytes, "launches_per_step": pass_n[dom] / args.steps,
                "peak_source": peak_src,
                "pass_ms_per_step": {k: pass_ms[k] / args.steps for k in PASS_NAMES},
                "pipeline_achieved": bm["_per_step"] / step_s / 1e9,
                "pipeline_frac": bm["_per_step"] / step_s / 1e9 / peak,
                "compulsory_frac": bm["_compulsory_per_step"] / step_s / 1e9 / peak,
                "fft_shape": list(plan.fft_shape), "p_min": bm["_p_min"]}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantom)",
            "config": config_dict(args.workload, wl), "roofline": roofline, "gpu_launches": launches,
            "clocks": clk.summary()}

    # errors of one step's output against the FP64 oracle (checker, outside the timed region)
    refs = None
    if rank == 0 and not args.no_check:
        errs, refs = oracle_errors(act, rho, wl, out_d.cpu().numpy())
        line["error_vs_fp64_oracle"] = errs

    # end to end through the public API from pinned host memory
    if not args.no_e2e:
        act_h = torch.from_numpy(act).pin_memory()
        rho_h = torch.from_numpy(rho).pin_memory() if rho is not None else None
        out_h = torch.empty((nk, *shape), dtype=torch.float32, pin_memory=True)
        for i in range(args.warmup):
            calc.calculate_dose_rate(act_h, vs, density=rho_h, out=out_h)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        barrier()
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for i in range(args.steps):
            ev[i][0].record(stream)
            calc.calculate_dose_rate(act_h, vs, density=rho_h, out=out_h)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        barrier()
        e2e_ms = max_over_ranks(float(np.sum([a.elapsed_time(b) for a, b in ev])), device)
        line["e2e"] = {"value": job_throughput(world, nk * vox, args.steps, e2e_ms), "unit": UNIT,
                       "h2d_bytes_per_step": 4 * vox * (2 if rho is not None else 1),
                       "d2h_bytes_per_step": 4 * vox * nk, "ms_per_step": e2e_ms / args.steps,
                       "wall_ms_per_step": 1e3 * wall / args.steps,
                       "api": "KernelConvolutionCalculator.calculate_dose_rate(pinned CPU tensors)"}
        line["e2e"]["link"] = link_bound(act_h, out_h, e2e_ms / args.steps, roofline["pass_ms_per_step"],
                                         total_ms / args.steps)
        if rank == 0 and not args.no_check:
            line["e2e"]["error_vs_fp64_oracle"] = oracle_errors(act, rho, wl, out_h.numpy(), refs)[0]
        # the drop-in user's call: pageable numpy in, new numpy arrays out, through the
        # reference's facade (DoseCalculator.calculate_dose, single timepoint), host wall clock
        from pyvoxeldosimetry_gb300.core.dose_calculator import DoseCalculator
        dc = DoseCalculator(wl["nuclides"], method="kernel",
                            config={"kernel_size": wl["ksize"], "device": device})
        act_np = np.ascontiguousarray(act)
        rho_np = np.ascontiguousarray(rho) if rho is not None else None
        for i in range(args.warmup):
            res = dc.calculate_dose(activity_maps=[act_np], time_points=[0.0], voxel_size=vs,
                                    tissue_densities=rho_np)
        barrier()
        np_ms = []
        for i in range(args.steps):
            t0 = time.perf_counter()
            res = dc.calculate_dose(activity_maps=[act_np], time_points=[0.0], voxel_size=vs,
                                    tissue_densities=rho_np)
            np_ms.append(1e3 * (time.perf_counter() - t0))
        barrier()
        np_total = max_over_ranks(float(np.sum(np_ms)), device)
        d_np = res.dose_rate_maps[0]
        line["e2e_numpy"] = {"value": job_throughput(world, nk * vox, args.steps, np_total), "unit": UNIT,
                             "h2d_bytes_per_step": 4 * vox * (2 if rho is not None else 1),
                             "d2h_bytes_per_step": 4 * vox * nk, "ms_per_step": np_total / args.steps,
                             "api": "DoseCalculator(method='kernel').calculate_dose(activity_maps=[numpy], "
                                    "tissue_densities=numpy) -> new numpy arrays (pageable host memory, host "
                                    "wall clock per call)",
                             "output": f"{type(d_np).__name__} {getattr(d_np, 'dtype', '')} {list(d_np.shape)}"}
        if rank == 0 and not args.no_check:
            line["e2e_numpy"]["error_vs_fp64_oracle"] = oracle_errors(act, rho, wl, d_np, refs)[0]
        dc.calculator.close()

    if not args.no_extras and rank == 0:  # sub-measurements of one GPU; only rank 0 prints
        line["mc"] = measure_mc(device)
        line["tac_fit"] = measure_fit(device)
        line["tac_fit_vp"] = measure_vp_fit(device)
        line["batch"] = measure_batch(device, args.batch_volumes)
        line["dvh"] = measure_dvh(device)
        line["resample"] = measure_resample(device)
        line["unet"] = measure_unet(device)
        line["unet"]["accuracy"] = measure_unet_accuracy(device, n_train=args.unet_train_phantoms)

    if rank == 0 and not args.no_cpu_baseline:
        ks = reference_kernels(wl)
        t0 = time.perf_counter()
        cpu_reference_stock(act, ks[0])
        dt = time.perf_counter() - t0
        t0 = time.perf_counter()
        cpu_reference_conv(act, rho, ks[0])
        dt_pad = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": vox / dt / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"one full {list(shape)} {wl['nuclides'][0]} convolution: the reference "
                                          "operator exactly as kernel_convolution.py:71-74 runs it (numpy float64, "
                                          "unpadded circular, one thread)",
                                "seconds": dt,
                                "padded_linear": {"value": vox / dt_pad / 1e9, "seconds": dt_pad,
                                                  "sample": "the same operator on zero-padded inputs + density "
                                                            "divide (the linear convolution computed here)"}}
        line["vs_cpu_baseline_1core"] = {
            "device_resident_vs_stock": value / line["cpu_baseline"]["value"],
            "device_resident_vs_padded": value / line["cpu_baseline"]["padded_linear"]["value"]}
        if "e2e" in line:
            line["vs_cpu_baseline_1core"]["e2e_vs_stock"] = line["e2e"]["value"] / line["cpu_baseline"]["value"]
            line["vs_cpu_baseline_1core"]["e2e_vs_padded"] = \
                line["e2e"]["value"] / line["cpu_baseline"]["padded_linear"]["value"]
        if "e2e_numpy" in line:
            line["vs_cpu_baseline_1core"]["e2e_numpy_vs_stock"] = \
                line["e2e_numpy"]["value"] / line["cpu_baseline"]["value"]
    if world > 1:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

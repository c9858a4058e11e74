"""Time-integrated dose of a batch of volumes of uneven sizes in one graph launch.

For every volume (T timepoint activity maps, their times in hours, voxel size,
optional density): a per-voxel two-exponential least-squares fit
(``pvd_tac_fit``, f4a model by variable projection from an exponential-peeling
start; by default FP32 trust-region iterations finished by FP64 ones, whose
convergence tests decide success), its analytic integral to infinity as
cumulated activity, and the dose-point-kernel convolution of that
cumulated activity (``pvd_conv_execute``; density-scaled when a density map is
given), giving absorbed dose in Gy.  ``prepare`` builds one convolution plan per
distinct (shape, voxel size), allocates every buffer, and has the native batch
runtime (``pvd_batch_create``) record all the volumes' kernel launches in one
CUDA graph; ``run`` launches it (``pvd_batch_run``), so the whole batch is one
launch from the host.  Without the graph, ``run`` enqueues the same work
directly (``pvd_batch_execute``).

This is the batched workload the dose calculator serves many patients,
timepoints and grid sizes with; the reference processes one volume at a time
on the CPU (pyvoxeldosimetry/core/dose_calculator.py:85-164,
time_integration/curve_fitting.py:112-219).
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Sequence

import numpy as np
import torch

from . import _native as N
from .conv import ConvPlan, _require_cuda
from .data import nuclides as nd

SECONDS_PER_HOUR = 3600.0


def partition_volumes(shapes: Sequence[Sequence[int]], world: int) -> List[List[int]]:
    """Volumes of a batch shared out over ``world`` replicas (one GPU each): largest
    first, each to the replica with the fewest voxels so far (ties to the lower rank),
    so every rank computes the same assignment without communicating.  Returns, per
    rank, the indices of its volumes in ascending order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    sizes = [int(np.prod(s)) for s in shapes]
    load = [0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(sizes)), key=lambda k: (-sizes[k], k)):
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += sizes[i]
    return [sorted(x) for x in parts]


class BatchDoseCalculator:
    def __init__(self, radionuclide: str = "Y90", kernel_size=None, use_graph: bool = True, mixed_fit: bool = True,
                 autotune: bool = False, max_fev: int = 2000, device=None):
        nd.get_nuclide(radionuclide)
        self.radionuclide = radionuclide
        self.kernel_size = kernel_size
        self.use_graph = use_graph
        self.mixed_fit = mixed_fit
        self.autotune = autotune
        self.max_fev = int(max_fev)
        self.device = _require_cuda(device)
        self._lib = N.load()
        self._plans: Dict[tuple, ConvPlan] = {}
        self._items: List[dict] = []
        self._desc = None          # pvd_batch_item array
        self._batch = None         # pvd_batch handle (recorded graph)

    # -- setup ------------------------------------------------------------------
    def _plan(self, shape, vs) -> ConvPlan:
        key = (tuple(shape), tuple(vs))
        p = self._plans.get(key)
        if p is None:
            ks = self.kernel_size or nd.default_kernel_size(self.radionuclide, vs)
            ks = (ks,) * 3 if np.isscalar(ks) else tuple(ks)
            pads = None
            if self.autotune:
                from .autotune import tune
                pads = tune(shape, ks, 1, device=self.device)
            p = ConvPlan(shape, kmax=ks, n_kernels=1, pad=pads, device=self.device)
            p.set_kernel(0, nd.analytic_profile(self.radionuclide, vs, ks),
                         scale=nd.gy_per_bq_s_scale(self.radionuclide, vs), normalize=True)
            self._plans[key] = p
        return p

    def prepare(self, volumes: Sequence[dict]) -> None:
        """``volumes``: dicts with ``activity`` (CUDA float32 [T, n0, n1, n2]), ``times``
        (T hours), ``voxel_size`` (mm, 3) and optional ``density`` (CUDA float32)."""
        self._release_batch()
        self._items = []
        for v in volumes:
            act = v["activity"]
            if not (isinstance(act, torch.Tensor) and act.is_cuda and act.dtype == torch.float32 and act.dim() == 4):
                raise TypeError("activity must be a CUDA float32 tensor [T, n0, n1, n2]")
            act = act.contiguous()
            times = [float(t) for t in v["times"]]
            if len(times) != act.shape[0] or len(times) < 4:
                raise ValueError("one map per time point, at least 4 time points for the two-exponential fit")
            vs = tuple(float(x) for x in v["voxel_size"])
            shape = tuple(act.shape[1:])
            rho = v.get("density")
            if rho is not None and (tuple(rho.shape) != shape or not rho.is_cuda):
                raise ValueError("density must be a CUDA tensor of the volume's shape")
            nvox = int(np.prod(shape))
            item = {
                "act": act, "times": times, "rho": None if rho is None else rho.float().contiguous(),
                "plan": self._plan(shape, vs), "nvox": nvox,
                "params": torch.empty((4, nvox), dtype=torch.float64, device=self.device),
                "auc": torch.empty(nvox, dtype=torch.float64, device=self.device),
                "ok": torch.empty(nvox, dtype=torch.uint8, device=self.device),
                "cum": torch.empty(shape, dtype=torch.float32, device=self.device),
                "dose": torch.empty((1, *shape), dtype=torch.float32, device=self.device),
            }
            self._items.append(item)
        desc = (N.BatchItem * len(self._items))()
        for d, it in zip(desc, self._items):
            it["times_c"] = (C.c_double * len(it["times"]))(*it["times"])
            d.plan = it["plan"]._h
            d.activity_d = it["act"].data_ptr()
            d.times = C.cast(it["times_c"], C.c_void_p)
            d.n_times = len(it["times"])
            d.density_d = it["rho"].data_ptr() if it["rho"] is not None else None
            d.params_d = it["params"].data_ptr()
            d.auc_d = it["auc"].data_ptr()
            d.ok_d = it["ok"].data_ptr()
            d.cum_d = it["cum"].data_ptr()
            d.dose_d = it["dose"].data_ptr()
        self._desc = desc
        if self.use_graph and self._items:
            h = C.c_void_p()
            with torch.cuda.device(self.device):
                torch.cuda.current_stream(self.device).synchronize()  # inputs written on torch's stream
                N.check(self._lib.pvd_batch_create(desc, len(self._items), self._fit_flags(), self.max_fev,
                                                   SECONDS_PER_HOUR, C.byref(h)))
            self._batch = h

    def _fit_flags(self) -> int:
        return N.PVD_FIT_VARPRO | (N.PVD_FIT_MIXED if self.mixed_fit else 0)

    def _release_batch(self) -> None:
        if self._batch is not None:
            self._lib.pvd_batch_destroy(self._batch)
            self._batch = None
        self._desc = None

    # -- execution --------------------------------------------------------------
    def run(self) -> List[torch.Tensor]:
        """Absorbed dose (Gy) per volume (device tensors, owned by this calculator)."""
        if not self._items:
            return []
        with torch.cuda.device(self.device):
            sh = torch.cuda.current_stream(self.device).cuda_stream
            if self._batch is not None:
                N.check(self._lib.pvd_batch_run(self._batch, sh))
            else:
                N.check(self._lib.pvd_batch_execute(self._desc, len(self._items), self._fit_flags(),
                                                    self.max_fev, SECONDS_PER_HOUR, sh))
        return [it["dose"][0] for it in self._items]

    def run_stages(self):
        """The batch's work as two directly enqueued stages, every volume's fit and then
        every volume's convolution, with CUDA events around each stage (instrumentation
        for measuring the stages apart; ``run`` is the production call).  Returns
        (fit_ms, conv_ms)."""
        if not self._items:
            return 0.0, 0.0
        p0 = (C.c_double * 5)(1.0, 0.1, 0.5, 0.01, 0.0)
        flags = self._fit_flags() | N.PVD_FIT_P0_FROM_DATA | N.PVD_FIT_AUC_INF
        with torch.cuda.device(self.device):
            st = torch.cuda.current_stream(self.device)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ev[0].record(st)
            for it in self._items:
                N.check(self._lib.pvd_tac_fit(N.PVD_FIT_F4A, it["times_c"], None, len(it["times"]), p0, 0.0, 0.0,
                                              self.max_fev, flags, it["act"].data_ptr(), it["nvox"],
                                              it["params"].data_ptr(), it["auc"].data_ptr(), it["ok"].data_ptr(),
                                              it["cum"].data_ptr(), SECONDS_PER_HOUR, st.cuda_stream))
            ev[1].record(st)
            for it in self._items:
                it["plan"].execute(it["cum"], density=it["rho"], out=it["dose"], stream=st)
            ev[2].record(st)
            ev[2].synchronize()
        return ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])

    def plans(self):
        """The convolution plan of each volume, in order."""
        return [it["plan"] for it in self._items]

    def calculate(self, volumes: Sequence[dict]) -> List[torch.Tensor]:
        self.prepare(volumes)
        return self.run()

    def fit_results(self, i: int):
        """(params [4, *shape] FP64, cumulated activity Bq h FP64, ok mask) of volume i."""
        it = self._items[i]
        shape = tuple(it["cum"].shape)
        return it["params"].view(4, *shape), it["auc"].view(shape), it["ok"].view(shape).bool()

    def cumulated(self, i: int) -> torch.Tensor:
        """Cumulated activity (Bq s, float32) of volume i: the convolution's input."""
        return self._items[i]["cum"]

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def close(self) -> None:
        self._release_batch()
        self._items = []
        for p in self._plans.values():
            p.close()
        self._plans = {}

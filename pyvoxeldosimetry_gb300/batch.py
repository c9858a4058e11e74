"""Time-integrated dose of a batch of volumes of uneven sizes in one graph launch.

For every volume (T timepoint activity maps, their times in hours, voxel size,
optional density): a per-voxel two-exponential least-squares fit
(``pvd_tac_fit``, f4a model by variable projection from an exponential-peeling
start; by default FP32 trust-region iterations finished by FP64 ones, whose
convergence tests decide success), its analytic integral to infinity as
cumulated activity, and the dose-point-kernel convolution of that
cumulated activity (``pvd_conv_execute``; density-scaled when a density map is
given), giving absorbed dose in Gy.  ``prepare`` builds one convolution plan per
distinct (shape, voxel size), allocates every buffer, and captures all the
volumes' kernel launches in a single CUDA graph; ``run`` replays it, so the
whole batch is one launch from the host.

This is the batched workload the dose calculator serves many patients,
timepoints and grid sizes with; the reference processes one volume at a time
on the CPU (pyvoxeldosimetry/core/dose_calculator.py:85-164,
time_integration/curve_fitting.py:112-219).
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _native as N
from .conv import ConvPlan, _require_cuda
from .data import nuclides as nd

SECONDS_PER_HOUR = 3600.0
F4A = 4


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
        self._graph: Optional[torch.cuda.CUDAGraph] = None

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
        self._items = []
        self._graph = None
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
        if self.use_graph:
            side = torch.cuda.Stream(self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(side):
                self._launch_all()  # one eager pass before capture
            torch.cuda.current_stream(self.device).wait_stream(side)
            torch.cuda.synchronize(self.device)
            self._graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self._graph):
                self._launch_all()

    def _launch_all(self) -> None:
        flags = (N.PVD_FIT_P0_FROM_DATA | N.PVD_FIT_AUC_INF | N.PVD_FIT_VARPRO
                 | (N.PVD_FIT_MIXED if self.mixed_fit else 0))
        p0 = (C.c_double * 5)(1.0, 0.1, 0.5, 0.01, 0.0)
        sh = torch.cuda.current_stream(self.device).cuda_stream
        for it in self._items:
            t = (C.c_double * len(it["times"]))(*it["times"])
            N.check(self._lib.pvd_tac_fit(F4A, t, None, len(it["times"]), p0, 0.0, 0.0, self.max_fev, flags,
                                          it["act"].data_ptr(), it["nvox"], it["params"].data_ptr(),
                                          it["auc"].data_ptr(), it["ok"].data_ptr(), it["cum"].data_ptr(),
                                          SECONDS_PER_HOUR, sh))
            it["plan"].execute(it["cum"], density=it["rho"], out=it["dose"])

    # -- execution --------------------------------------------------------------
    def run(self) -> List[torch.Tensor]:
        """Absorbed dose (Gy) per volume (device tensors, owned by this calculator)."""
        if not self._items:
            return []
        with torch.cuda.device(self.device):
            if self._graph is not None:
                self._graph.replay()
            else:
                self._launch_all()
        return [it["dose"][0] for it in self._items]

    def calculate(self, volumes: Sequence[dict]) -> List[torch.Tensor]:
        self.prepare(volumes)
        return self.run()

    def fit_results(self, i: int):
        """(params [4, *shape] FP64, cumulated activity Bq h FP64, ok mask) of volume i."""
        it = self._items[i]
        shape = tuple(it["cum"].shape)
        return it["params"].view(4, *shape), it["auc"].view(shape), it["ok"].view(shape).bool()

    def close(self) -> None:
        self._graph = None
        self._items = []
        for p in self._plans.values():
            p.close()
        self._plans = {}

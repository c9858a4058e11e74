"""Trapezoidal time integration of activity maps on the GPU.

Mirrors ActivitySampler (pyvoxeldosimetry/core/activity_sampler.py:8-78):
same constructor validation (half-life > 0, units in hours/minutes/seconds),
``sample_timepoints`` and ``integrate_activity(..., method='trapezoid')``.
The weighted sum runs in ``pvd_weighted_sum``; ``integrate_dose_rates`` is the
method the reference's façade calls but never defines
(core/dose_calculator.py:138).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import List, Optional

import numpy as np
import torch

from .. import _io
from .. import _native as N
from ..conv import _require_cuda, _stream_handle
from .kernel_convolution import trapezoid_weights

SECONDS_PER = {"hours": 3600.0, "minutes": 60.0, "seconds": 1.0}


def weighted_sum(maps, weights, out=None):
    """sum_t weights[t] * maps[t] on the GPU; maps in any array kind."""
    kind = _io.kind_of(maps[0])
    device = _require_cuda(maps[0].device if kind == _io.CUDA_TENSOR else None)
    lib = N.load()
    with torch.cuda.device(device):
        shape = tuple(maps[0].shape)
        if any(tuple(m.shape) != shape for m in maps):
            raise ValueError("All activity maps must have the same dimensions")
        dev = [_io.to_device(m, device, "map") for m in maps]
        res = torch.empty(shape, dtype=torch.float32, device=device)
        ptrs = (C.c_void_p * len(dev))(*[d.data_ptr() for d in dev])
        w = (C.c_float * len(dev))(*[float(x) for x in weights])
        N.check(lib.pvd_weighted_sum(ptrs, w, len(dev), res.numel(), res.data_ptr(), _stream_handle(None)))
        return _io.from_device(res, kind, out)


class ActivitySampler:
    def __init__(self, half_life: float, units: str = "hours"):
        self.half_life = half_life
        self.units = units
        self._validate_inputs()

    def _validate_inputs(self):
        if self.half_life <= 0:
            raise ValueError("Half-life must be positive")
        if self.units not in ["hours", "minutes", "seconds"]:
            raise ValueError("Invalid time units")

    def sample_timepoints(self, start_time: float, end_time: float, n_points: int = 10) -> np.ndarray:
        return np.linspace(start_time, end_time, n_points)

    def integrate_activity(self, activity_maps, time_points: List[float], method: str = "trapezoid"):
        """Cumulated activity sum_i (A_i + A_{i+1})/2 (t_{i+1} - t_i), time in ``units``."""
        if method != "trapezoid":
            raise ValueError(f"Unknown integration method: {method}")
        return weighted_sum(list(activity_maps), trapezoid_weights(time_points))

    def physical_decay_tail(self, t_from: float, t_to: Optional[float]) -> float:
        """Integral of exp(-lambda (t - t_from)) dt from t_from to t_to (inf when None), in ``units``."""
        lam = math.log(2.0) / self.half_life
        if t_to is None:
            return 1.0 / lam
        return (1.0 - math.exp(-lam * max(t_to - t_from, 0.0))) / lam

    def integrate_dose_rates(self, dose_rates, time_points: List[float], integration_limit: Optional[float] = None):
        """Absorbed dose (Gy) from dose rates (Gy/s) at ``time_points``: trapezoid over
        the sampled interval, plus, when ``integration_limit`` (same unit as the
        time points) lies past the last sample, the physical-decay tail of the
        last dose rate up to that limit."""
        sec = SECONDS_PER[self.units]
        w = trapezoid_weights(time_points, sec)
        if integration_limit is not None and integration_limit > time_points[-1]:
            w[-1] += self.physical_decay_tail(time_points[-1], integration_limit) * sec
        return weighted_sum(list(dose_rates), w)

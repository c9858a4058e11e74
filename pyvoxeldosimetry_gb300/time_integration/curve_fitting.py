"""Per-voxel time-activity-curve fitting on the GPU (FP64, one thread per voxel).

Mirrors TimeCurveFitting (pyvoxeldosimetry/time_integration/curve_fitting.py):
``fit_time_activity_curve`` (:19-65) with ``_calculate_accumulated_dose``
(:74-84), and ``fit_time_activity_curve_advanced`` (:112-219) with its NUKFIT
(f2, f3, f3a, f4a, f4b, f4c) and "lmfit" (mono/bi/tri-exponential) tables,
initial guesses, sigma = 1/weight, failure fallbacks and AUC rules.  The fits
run in ``pvd_tac_fit``; image loading (``load_timepoint_images``, DICOM/NIfTI)
is outside this package.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Tuple

import numpy as np
import torch

from .. import _io
from .. import _native as N
from ..conv import _require_cuda, _stream_handle

MODEL_IDS = {"f2": 1, "f3": 2, "f3a": 3, "f4a": 4, "f4b": 5, "f4c": 6,
             "mono-exponential": 7, "bi-exponential": 8, "tri-exponential": 9}
NUKFIT = ["f2", "f3", "f3a", "f4a", "f4b", "f4c"]
LMFIT = ["mono-exponential", "bi-exponential", "tri-exponential"]
MONO_MAXFEV = 200 * (2 + 1)  # curve_fit's default maxfev for lmdif with n = 2 parameters
ADVANCED_MAXFEV = 10000      # curve_fitting.py:206


def _p0_table(half_life: float) -> dict:
    """Initial guesses of curve_fitting.py:150-168."""
    return {"f2": [1.0, 0.1], "f3": [1.0, 0.1, 0.01], "f3a": [1.0, 0.5, 0.1], "f4a": [1.0, 0.1, 0.5, 0.01],
            "f4b": [1.0, 0.1, 0.5, 0.01, 0.693], "f4c": [1.0, 0.1, 0.5, 0.01, 0.693],
            "mono-exponential": [1.0, half_life], "bi-exponential": [1.0, half_life, half_life / 2],
            "tri-exponential": [1.0, half_life, 0.5, half_life / 2, half_life]}


def _run_fit(model_id, n_par, times, weights, p0, lam_phys, auc_limit, max_fev, flags, activities):
    acts = activities if not isinstance(activities, (list, tuple)) else None
    if acts is None:
        kinds = {_io.kind_of(a) for a in activities}
        kind = kinds.pop() if len(kinds) == 1 else _io.NUMPY
        shape = tuple(activities[0].shape)
        if kind == _io.CUDA_TENSOR:
            stack = torch.stack([a.float() for a in activities])
        else:
            stack = np.stack([np.asarray(a, dtype=np.float32) for a in activities])
    else:
        kind = _io.kind_of(acts)
        shape = tuple(acts.shape[1:])
        stack = acts
    n_t = len(times)
    if len(stack) != n_t:
        raise ValueError("one activity map per time point is required")
    device = _require_cuda(stack.device if kind == _io.CUDA_TENSOR else None)
    lib = N.load()
    with torch.cuda.device(device):
        a = _io.to_device(stack, device, "activities").reshape(n_t, -1)
        nvox = a.shape[1]
        params = torch.empty((n_par, nvox), dtype=torch.float64, device=device)
        auc = torch.empty(nvox, dtype=torch.float64, device=device)
        ok = torch.empty(nvox, dtype=torch.uint8, device=device)
        t = (C.c_double * n_t)(*[float(x) for x in times])
        w = (C.c_double * n_t)(*[float(x) for x in weights]) if weights is not None else None
        p = (C.c_double * 5)(*(list(p0) + [0.0] * (5 - len(p0)))) if p0 is not None else None
        N.check(lib.pvd_tac_fit(model_id, t, w, n_t, p, float(lam_phys), float(auc_limit), int(max_fev), flags,
                                a.data_ptr(), nvox, params.data_ptr(), auc.data_ptr(), ok.data_ptr(), None, 1.0,
                                _stream_handle(None)))
        params = params.reshape((n_par, *shape))
        auc = auc.reshape(shape)
        ok = ok.reshape(shape)
        if kind == _io.CUDA_TENSOR:
            return params, auc, ok
        return params.cpu().numpy(), auc.cpu().numpy(), ok.cpu().numpy().astype(bool)


class TimeCurveFitting:
    def __init__(self, half_life: float):
        self.half_life = half_life
        self.decay_constant = np.log(2) / half_life

    def fit_time_activity_curve(self, times: List[float], activities, weight_factors: Optional[List[float]] = None,
                                integration_limit: Optional[float] = None, return_success: bool = False):
        """Mono-exponential A0 exp(-lam t) fit per voxel with p0 = [A(t0), ln2/T1/2] and
        sigma = 1/weight; failures give [0, ln2/T1/2].  Returns (params (2, *shape),
        accumulated = A0/lam (1 - exp(-lam * limit)), limit = 100 T1/2 by default)."""
        limit = 100 * self.half_life if integration_limit is None else integration_limit
        params, auc, ok = _run_fit(0, 2, times, weight_factors, None, self.decay_constant, limit,
                                   MONO_MAXFEV, 0, activities)
        return (params, auc, ok) if return_success else (params, auc)

    def _calculate_accumulated_dose(self, fitted_params, integration_limit: float = None):
        if integration_limit is None:
            integration_limit = 100 * self.half_life
        a0, lam = fitted_params[0], fitted_params[1]
        return a0 / lam * (1 - np.exp(-lam * integration_limit))

    def fit_time_activity_curve_advanced(self, times: List[float], activities, model: str = "nukfit",
                                         model_name: str = None, weight_factors: Optional[List[float]] = None,
                                         force_zero_at_t0: bool = False, integration_limit: float = None,
                                         phys_half_life: float = None, return_fit_params: bool = False):
        """NUKFIT / lmfit model fit per voxel; AUC = trapezoid of the fitted curve over
        the sampled times (curve_fitting.py:215).  Returns (params, aucs) or, with
        ``return_fit_params``, (params, aucs, info) where info carries the model and a
        per-voxel success map."""
        if model.lower() == "nukfit":
            names = NUKFIT
        elif model.lower() == "lmfit":
            names = LMFIT
        else:
            raise ValueError(f"Unknown model type: {model}")
        if model_name is None:
            model_name = names[0]
        if model_name not in names:
            raise KeyError(model_name)
        p0 = _p0_table(self.half_life)[model_name]
        lam_phys = self.decay_constant if phys_half_life is None else np.log(2) / phys_half_life
        n_par = len(p0)
        flags = 2 | (1 if force_zero_at_t0 else 0)
        params, auc, ok = _run_fit(MODEL_IDS[model_name], n_par, times, weight_factors, p0, lam_phys, 0.0,
                                   ADVANCED_MAXFEV, flags, activities)
        if return_fit_params:
            return params, auc, {"model": model, "model_name": model_name, "success": ok}
        return params, auc

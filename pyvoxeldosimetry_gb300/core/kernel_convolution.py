"""Dose-point-kernel convolution calculator on the GPU.

Drop-in for KernelConvolutionCalculator
(pyvoxeldosimetry/core/kernel_convolution.py:26-114): same constructor
(radionuclide, tissue_name, kernel_resolution, config), same
``calculate_dose_rate(activity_map, voxel_size)`` and
``calculate_absorbed_dose(activity_maps, time_points, voxel_size)``, plus
``calculate_absorbed_dose_from_accumulated`` that the reference's façade calls
but never defines (core/dose_calculator.py:104,123).

Differences from the reference, each deliberate:
  * the convolution is zero-padded and linear by default (``config['mode'] =
    'linear'``); ``'reference_circular'`` reproduces the reference's unpadded
    circular operator with its K//2 shift exactly (kernel_convolution.py:71-74);
  * the default kernel is the analytic exp(-r/lambda)/r^2 profile evaluated at
    the activity's own voxel size and normalised to the mean beta energy, so no
    resampling is needed (the reference's ``_resample_activity`` is a stub that
    returns None, kernel_convolution.py:108-114).  An explicit kernel
    (``config['kernel']`` or assigning ``calculator.kernel``) or
    ``kernel_profile='reference'`` is defined at ``kernel_resolution``: an
    activity at another voxel size is resampled to that grid on the GPU
    (cubic B-spline, total activity conserved; ``config['resample_order']`` 1
    for trilinear), convolved there, and the dose resampled back to the
    activity's grid (``config['resample_output'] = 'kernel'`` returns the
    kernel-grid dose, which is what the reference's stub was meant to feed);
  * an optional density map gives the density-scaled dose D/rho;
  * ``config['energy_per_decay_mev']`` (a number or {nuclide: number}) replaces the
    stated mean beta energy the analytic kernel is normalised to (the learned
    correction uses the mean of the spectrum its Monte Carlo samples);
  * the multi-timepoint trapezoid runs as ONE convolution of the trapezoid-
    weighted activity (identical by linearity) with the weighting fused into
    the first FFT pass;
  * results are float32 and come back in the caller's array kind (numpy in ->
    numpy out, CUDA tensor in -> CUDA tensor out);
  * the FFT lengths of a new (shape, kernel size) are chosen by timing the
    candidates once (``pyvoxeldosimetry_gb300.autotune``, cached on disk);
    ``config['autotune'] = False`` takes the smallest fast length instead, and
    ``config['pads'] = (P0, P1, P2)`` gives the lengths explicitly.
"""
from __future__ import annotations

from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from .. import _io
from ..conv import ConvPlan, _require_cuda
from ..data import nuclides as nd
from .dosimetry_base import DosimetryCalculator

SECONDS_PER_HOUR = 3600.0


def trapezoid_weights(time_points: Sequence[float], seconds_per_unit: float = 1.0) -> List[float]:
    """w_t such that sum_t w_t A_t == sum_i (A_i + A_{i+1})/2 (t_{i+1} - t_i) * seconds_per_unit
    (core/activity_sampler.py:69-78, core/kernel_convolution.py:99-104)."""
    t = [float(x) for x in time_points]
    w = [0.0] * len(t)
    for i in range(len(t) - 1):
        dt = (t[i + 1] - t[i]) * seconds_per_unit
        w[i] += dt / 2
        w[i + 1] += dt / 2
    return w


class KernelConvolutionCalculator(DosimetryCalculator):
    def __init__(self, radionuclide, tissue_name: str = "water", kernel_resolution: float = 1.0,
                 config: Optional[Dict[str, Any]] = None):
        super().__init__(radionuclide, tissue_name, config)
        self.kernel_resolution = kernel_resolution
        self.tissue_name = tissue_name
        self.mode = self.config.get("mode", "linear")
        if self.mode not in ("linear", "reference_circular"):
            raise ValueError(f"mode must be 'linear' or 'reference_circular', got {self.mode!r}")
        self.kernel_profile = self.config.get("kernel_profile", "analytic")
        if self.kernel_profile not in ("analytic", "reference"):
            raise ValueError(f"kernel_profile must be 'analytic' or 'reference', got {self.kernel_profile!r}")
        for n in self.nuclides:
            nd.get_nuclide(n)  # ValueError for unknown nuclides, like KernelFactory.get_kernel
        self.kernel = self.config.get("kernel")
        self.kernel_size = self.config.get("kernel_size")
        self.device = self.config.get("device")
        self._plan: Optional[ConvPlan] = None
        self._plan_key = None

    # -- kernels ----------------------------------------------------------------
    def _size_for(self, nuc: str, voxel_size) -> Tuple[int, int, int]:
        ks = self.kernel_size
        if isinstance(ks, dict):
            ks = ks.get(nuc)
        if ks is None:
            return nd.default_kernel_size(nuc, voxel_size)
        if np.isscalar(ks):
            return (int(ks),) * 3
        return tuple(int(x) for x in ks)

    def _kernel_specs(self, voxel_size) -> List[Tuple[np.ndarray, float, bool]]:
        """(kernel FP64, scale, normalise-on-GPU) per nuclide."""
        vs = tuple(float(v) for v in voxel_size)
        if self._fixed_grid() and vs != (float(self.kernel_resolution),) * 3:
            raise ValueError(f"voxel_size {vs} differs from kernel_resolution {self.kernel_resolution}")
        if self.kernel is not None:
            ks = self.kernel if isinstance(self.kernel, (list, tuple)) else [self.kernel] * len(self.nuclides)
            if len(ks) != len(self.nuclides):
                raise ValueError("one explicit kernel per nuclide is required")
            return [(np.asarray(k, dtype=np.float64), 1.0, False) for k in ks]
        specs = []
        for nuc in self.nuclides:
            shape = self._size_for(nuc, vs if self.kernel_profile == "analytic" else self.kernel_resolution)
            if self.kernel_profile == "analytic":
                e = self.config.get("energy_per_decay_mev")
                e = e.get(nuc) if isinstance(e, dict) else e
                specs.append((nd.analytic_profile(nuc, vs, shape), nd.gy_per_bq_s_scale(nuc, vs, energy_mev=e), True))
            else:
                specs.append((nd.reference_profile(nuc, self.tissue_name, float(self.kernel_resolution), shape),
                              1.0, False))
        return specs

    def _plan_for(self, shape, voxel_size, device) -> ConvPlan:
        vs = tuple(float(v) for v in voxel_size)
        spec_key = (vs, id(self.kernel), self.kernel_profile, repr(self.kernel_size), self.tissue_name,
                    float(self.kernel_resolution), repr(self.config.get("energy_per_decay_mev")))
        key = (tuple(shape), self.mode, str(device), spec_key)
        if self._plan is not None and self._plan_key == key:
            return self._plan
        specs = self._kernel_specs(vs)
        if self._plan is not None:
            self._plan.close()
            self._plan = None
        kmax = tuple(max(k.shape[i] for k, _, _ in specs) for i in range(3))
        pads = self.config.get("pads")
        if pads is None and self.mode == "linear" and self.config.get("autotune", True):
            from ..autotune import tune
            pads = tune(shape, kmax, len(specs), device=device)
        plan = ConvPlan(shape, kmax=kmax, n_kernels=len(specs), mode=self.mode, pad=pads, device=device)
        for slot, (k, s, nm) in enumerate(specs):
            plan.set_kernel(slot, k, scale=s, normalize=nm)
        self._plan, self._plan_key = plan, key
        return plan

    def _fixed_grid(self) -> bool:
        """Kernels defined at kernel_resolution (explicit or the reference generators)."""
        return self.kernel is not None or self.kernel_profile == "reference"

    def _run_resampled(self, activity, voxel_size, density, weights, out_scale, out):
        """Activity (and density) resampled to the kernel grid, convolved there, the
        dose resampled back to the activity's grid (or returned on the kernel grid)."""
        from .utils import resample_volume
        kr = (float(self.kernel_resolution),) * 3
        vs = tuple(float(v) for v in voxel_size)
        order = int(self.config.get("resample_order", 3))
        acts = activity if weights is not None else [activity]
        kind = _io.kind_of(acts[0])
        device = _require_cuda(self.device if self.device is not None else
                               (acts[0].device if kind == _io.CUDA_TENSOR else None))
        shape = tuple(acts[0].shape)
        with torch.cuda.device(device):
            dev_acts = [resample_volume(_io.to_device(a, device, "activity"), vs, kr, order=order,
                                        conserve_total=True) for a in acts]
            rho = None
            if density is not None:
                if tuple(density.shape) != shape:
                    raise ValueError("density map must have the activity map's shape")
                rho = resample_volume(_io.to_device(density, device, "density"), vs, kr, order=1)
            res = self._run(dev_acts if weights is not None else dev_acts[0], kr, rho, weights, out_scale, None)
            if self.config.get("resample_output", "input") != "kernel":
                maps = res if not isinstance(self.radionuclide, str) else res[None]
                back = torch.stack([resample_volume(mp, kr, vs, order=order, output_shape=shape) for mp in maps])
                res = back if not isinstance(self.radionuclide, str) else back[0]
            return _io.from_device(res, kind, out)

    # -- public API -------------------------------------------------------------
    def _run(self, activity, voxel_size, density, weights, out_scale, out):
        if len(voxel_size) != 3:
            raise ValueError("voxel_size must be a tuple of length 3.")
        if self._fixed_grid() and tuple(float(v) for v in voxel_size) != (float(self.kernel_resolution),) * 3:
            return self._run_resampled(activity, voxel_size, density, weights, out_scale, out)
        acts = activity if weights is not None else [activity]
        kind = _io.kind_of(acts[0])
        device = _require_cuda(self.device if self.device is not None else
                               (acts[0].device if kind == _io.CUDA_TENSOR else None))
        with torch.cuda.device(device):
            shape = tuple(acts[0].shape)
            if len(shape) != 3:
                raise ValueError("activity map must be 3-D")
            if any(tuple(a.shape) != shape for a in acts):
                raise ValueError("All activity maps must have the same dimensions")
            plan = self._plan_for(shape, voxel_size, device)
            if weights is None and kind != _io.CUDA_TENSOR and _io.kind_of(density) != _io.CUDA_TENSOR:
                return self._run_host(plan, acts[0], density, out_scale, out, kind, shape)
            dev_acts = [_io.to_device(a, device, "activity") for a in acts]
            rho = None
            if density is not None:
                if tuple(density.shape) != shape:
                    raise ValueError("density map must have the activity map's shape")
                rho = _io.to_device(density, device, "density")
            res = plan.execute(dev_acts[0] if weights is None else dev_acts, density=rho, out_scale=out_scale,
                               weights=weights)
            if isinstance(self.radionuclide, str):
                res = res[0]
            return _io.from_device(res, kind, out)

    def _run_host(self, plan, activity, density, out_scale, out, kind, shape):
        """Host arrays in and out: the plan's pipelined copy/compute path."""
        if density is not None and tuple(density.shape) != shape:
            raise ValueError("density map must have the activity map's shape")
        single = isinstance(self.radionuclide, str)
        dst = None
        if out is not None:
            t = torch.from_numpy(out) if isinstance(out, np.ndarray) else out
            dst = t.view(1, *shape) if single else t
        res = plan.execute_host(activity, density, out=dst, out_scale=out_scale)
        if out is not None:
            return out
        if single:
            res = res[0]
        return res.numpy() if kind == _io.NUMPY else res

    def calculate_dose_rate(self, activity_map, voxel_size: Tuple[float, float, float], density=None, out=None):
        """Dose rate (Gy/s) of an activity map (Bq per voxel).

        With ``density`` (g/cc, same shape) the dose is scaled to local mass
        (D / rho, 0 where rho <= 0).  With a list of nuclides the result has a
        leading nuclide axis; all nuclides share one forward transform.
        """
        return self._run(activity_map, voxel_size, density, None, 1.0, out)

    def calculate_absorbed_dose(self, activity_maps, time_points: List[float], voxel_size, density=None, out=None):
        """Absorbed dose (Gy): trapezoid over the dose rates at ``time_points`` (hours),
        evaluated as one convolution of the trapezoid-weighted activity."""
        if len(activity_maps) != len(time_points):
            raise ValueError("Number of activity maps must match number of time points")
        w = trapezoid_weights(time_points, SECONDS_PER_HOUR)
        return self._run(list(activity_maps), voxel_size, density, w, 1.0, out)

    def calculate_absorbed_dose_from_accumulated(self, accumulated_activity, voxel_size, density=None,
                                                 seconds_per_unit: float = SECONDS_PER_HOUR, out=None):
        """Absorbed dose (Gy) from cumulated activity (Bq x time unit, hours by default)."""
        return self._run(accumulated_activity, voxel_size, density, None, float(seconds_per_unit), out)

    def close(self):
        if self._plan is not None:
            self._plan.close()
            self._plan = None

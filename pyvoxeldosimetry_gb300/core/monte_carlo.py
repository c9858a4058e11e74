"""GPU Monte Carlo dose calculator.

Mirrors MonteCarloCalculator (pyvoxeldosimetry/core/monte_carlo.py:10-172):
constructor (radionuclide, tissue_composition, n_particles, random_seed,
config), ``calculate_dose_rate(activity_map, voxel_size)`` in Gy/s and
``calculate_absorbed_dose`` as the trapezoid of per-timepoint dose rates
(:139-167).  The transport runs in ``pvd_mc_run`` (one thread per history);
the physics model is the builder's (pyvoxeldosimetry_gb300/data/mc_physics.py)
because the reference's never runs (:38-40).  Results are bit-reproducible for a
given ``random_seed`` (default 0; the reference's default None meant an
unseeded generator).
"""
from __future__ import annotations

import ctypes as C
from typing import Any, Dict, List, Optional, Tuple

import numpy as np
import torch

from .. import _io
from .. import _native as N
from ..conv import _require_cuda, _stream_handle
from ..data import mc_physics as mp
from ..data import nuclides as nd
from .dosimetry_base import DosimetryCalculator
from .kernel_convolution import SECONDS_PER_HOUR, trapezoid_weights

FIX_UNIT_MEV = 2.0 ** -32


def physics_tables(radionuclide: str, e_cut: float = mp.E_CUT) -> Dict[str, Any]:
    """Host tables and emission data of one nuclide, as pvd_mc_desc takes them."""
    nuc = nd.get_nuclide(radionuclide)
    beta = mp.beta_inverse_cdf(radionuclide) if len(nuc.spectrum_e) >= 2 else np.zeros(2, np.float32)
    lines = mp.emission_lines(radionuclide)
    e_beta_max = float(beta[-1]) if len(nuc.spectrum_e) >= 2 else 0.0
    rde, rng = mp.electron_range_table(max(e_beta_max, max([e for e, _ in lines], default=0.0), 0.05) * 1.001)
    pde, mu, cf = mp.photon_tables(max(max([e for e, _ in lines], default=0.1), 0.1) * 1.001)
    return {"beta_icdf": beta, "range": rng, "range_de": float(rde), "mu_rho": mu, "compton_frac": cf,
            "photon_de": float(pde), "gamma_e": np.array([e for e, _ in lines], np.float32),
            "gamma_yield": np.array([p for _, p in lines], np.float32),
            "beta_yield": 1.0 if len(nuc.spectrum_e) >= 2 else 0.0, "e_cut": float(e_cut)}


class McPlan:
    """Owner of a ``pvd_mc_plan*`` for one grid and nuclide."""

    def __init__(self, shape, voxel_mm, tables: Dict[str, Any], device=None):
        self.device = _require_cuda(device)
        self._lib = N.load()
        self.shape = tuple(int(s) for s in shape)
        self.tables = tables
        d = N.McDesc()
        for i in range(3):
            d.n[i] = self.shape[i]
            d.voxel_mm[i] = float(voxel_mm[i])
        self._keep = [np.ascontiguousarray(tables[k], np.float32) for k in ("beta_icdf", "range", "mu_rho",
                                                                              "compton_frac")]
        d.beta_icdf, d.n_beta = self._keep[0].ctypes.data, len(self._keep[0])
        d.range, d.n_range, d.range_de = self._keep[1].ctypes.data, len(self._keep[1]), tables["range_de"]
        d.mu_rho, d.compton_frac = self._keep[2].ctypes.data, self._keep[3].ctypes.data
        d.n_photon, d.photon_de = len(self._keep[2]), tables["photon_de"]
        ng = len(tables["gamma_e"])
        if ng > 8:
            raise ValueError("at most 8 gamma lines")
        d.n_gamma = ng
        for i in range(ng):
            d.gamma_e[i] = float(tables["gamma_e"][i])
            d.gamma_yield[i] = float(tables["gamma_yield"][i])
        d.beta_yield = float(tables["beta_yield"])
        d.e_cut = float(tables["e_cut"])
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check(self._lib.pvd_mc_plan_create(C.byref(d), C.byref(h)))
        self._h = h

    def run(self, activity: torch.Tensor, density: Optional[torch.Tensor], n_histories: int, seed: int,
            dose: bool = True, stats: bool = False):
        """Returns (edep uint64 tensor as int64 bits, dose-rate float32 tensor or None, stats dict or None)."""
        edep = torch.empty(self.shape, dtype=torch.int64, device=self.device)
        dr = torch.empty(self.shape, dtype=torch.float32, device=self.device) if dose else None
        st = N.McStats() if stats else None
        with torch.cuda.device(self.device):
            N.check(self._lib.pvd_mc_run(self._h, activity.data_ptr(),
                                         density.data_ptr() if density is not None else None,
                                         int(n_histories), int(seed), edep.data_ptr(),
                                         dr.data_ptr() if dr is not None else None,
                                         C.byref(st) if st is not None else None, _stream_handle(None)))
        sd = None
        if st is not None:
            sd = {"total_weight": st.total_weight, "emitted": st.emitted, "escaped": st.escaped, "steps": st.steps,
                  "activity_bq": st.activity_bq}
        return edep, dr, sd

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.pvd_mc_plan_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MonteCarloCalculator(DosimetryCalculator):
    def __init__(self, radionuclide: str, tissue_composition: Any = None, n_particles: int = 1000000,
                 random_seed: Optional[int] = None, config: Optional[Dict[str, Any]] = None):
        super().__init__(radionuclide, tissue_composition, config)
        if not isinstance(radionuclide, str):
            raise TypeError("MonteCarloCalculator takes one radionuclide")
        self.n_particles = int(n_particles)
        self.random_seed = 0 if random_seed is None else int(random_seed)
        self.decay_data = physics_tables(radionuclide, self.config.get("e_cut", mp.E_CUT))
        self.device = self.config.get("device")
        self._plan: Optional[McPlan] = None
        self._key = None
        self.last_stats: Optional[Dict[str, Any]] = None

    def _plan_for(self, shape, voxel_size, device) -> McPlan:
        key = (tuple(shape), tuple(float(v) for v in voxel_size), str(device))
        if self._plan is None or self._key != key:
            if self._plan is not None:
                self._plan.close()
            self._plan = McPlan(shape, voxel_size, self.decay_data, device)
            self._key = key
        return self._plan

    def calculate_dose_rate(self, activity_map, voxel_size: Tuple[float, float, float], density=None,
                            n_particles: Optional[int] = None, seed: Optional[int] = None):
        """Dose rate (Gy/s): deposited energy per history x activity (Bq) / voxel mass."""
        if len(voxel_size) != 3:
            raise ValueError("voxel_size must be a tuple of length 3.")
        kind = _io.kind_of(activity_map)
        device = _require_cuda(self.device if self.device is not None else
                               (activity_map.device if kind == _io.CUDA_TENSOR else None))
        with torch.cuda.device(device):
            shape = tuple(activity_map.shape)
            if len(shape) != 3:
                raise ValueError("activity map must be 3-D")
            a = _io.to_device(activity_map, device, "activity")
            rho = None
            if density is not None:
                if tuple(density.shape) != shape:
                    raise ValueError("density map must have the activity map's shape")
                rho = _io.to_device(density, device, "density")
            plan = self._plan_for(shape, voxel_size, device)
            _, dr, st = plan.run(a, rho, self.n_particles if n_particles is None else n_particles,
                                 self.random_seed if seed is None else seed, dose=True, stats=True)
            self.last_stats = st
            return _io.from_device(dr, kind)

    def calculate_absorbed_dose(self, activity_maps, time_points: List[float], voxel_size, density=None):
        """Trapezoid of the per-timepoint dose rates, time in hours (monte_carlo.py:139-167)."""
        if len(activity_maps) != len(time_points):
            raise ValueError("Number of activity maps must match number of time points")
        rates = [self.calculate_dose_rate(a, voxel_size, density=density, seed=self.random_seed + i)
                 for i, a in enumerate(activity_maps)]
        from .activity_sampler import weighted_sum
        return weighted_sum(rates, trapezoid_weights(time_points, SECONDS_PER_HOUR))

    def calculate_absorbed_dose_from_accumulated(self, accumulated_activity, voxel_size, density=None,
                                                 seconds_per_unit: float = SECONDS_PER_HOUR):
        """Cumulated activity (Bq x time unit) -> Gy: the dose-rate shape scaled by the unit."""
        d = self.calculate_dose_rate(accumulated_activity, voxel_size, density=density)
        return d * seconds_per_unit

    def close(self):
        if self._plan is not None:
            self._plan.close()
            self._plan = None

"""Dose-calculation façade.

Mirrors DoseCalculator / DoseCalculationResult
(pyvoxeldosimetry/core/dose_calculator.py:24-164): same constructor
(radionuclide, method, config), same ``calculate_dose`` keywords and routing
(accumulated activity / several timepoints / one timepoint) and the same
ValueErrors.  Changes:
  * method aliases: 'kernel' == 'kernel_convolution'; 'gpu_monte_carlo' ==
    'monte_carlo' (the in-repo GPU transport); 'gate_monte_carlo' (an external
    Geant4 application) is not provided and raises NotImplementedError;
  * ``tissue_densities`` is used: dose is scaled to local mass (the reference
    accepts and ignores it, :90);
  * the half-life defaults to the nuclide's (the reference's default 0.0 makes
    ActivitySampler raise, :76-79, activity_sampler.py:25-26);
  * the two methods the reference calls but never defines
    (``calculate_absorbed_dose_from_accumulated``, ``integrate_dose_rates``)
    exist, so both multi-timepoint modes work;
  * timepoint maps are used as given: image registration (SimpleITK in the
    reference, core/image_registration.py) is outside this package, so maps must
    already be aligned;
  * ``ct_image`` (Hounsfield units) may replace ``tissue_densities``: the density
    comes from the GPU HU calibration of ``tissue.TissueComposition``;
  * ``config['single_timepoint_dose'] = 'physical_decay'`` also returns the
    absorbed dose of one timepoint under physical decay to infinity,
    D = dose_rate * T1/2 * 3600 / ln 2.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Tuple

from ..data import nuclides as nd
from .activity_sampler import SECONDS_PER, ActivitySampler
from .kernel_convolution import KernelConvolutionCalculator

METHODS = {"kernel": "kernel", "kernel_convolution": "kernel", "gpu_monte_carlo": "monte_carlo",
           "monte_carlo": "monte_carlo", "gate_monte_carlo": "gate", "nn_corrected": "nn_corrected"}


@dataclass
class DoseCalculationResult:
    """Container for dose calculation results."""
    absorbed_dose: Optional[Any]
    dose_rate_maps: List[Any]
    time_points: List[float]
    metadata: Dict[str, Any]


class DoseCalculator:
    """Main class for performing dose calculations."""

    def __init__(self, radionuclide, method: str = "kernel", config: Optional[Dict[str, Any]] = None):
        self.radionuclide = radionuclide
        self.method = method.lower()
        self.config = config or {}
        kind = METHODS.get(self.method)
        if kind == "kernel":
            self.calculator = KernelConvolutionCalculator(
                radionuclide=radionuclide,
                tissue_name=self.config.get("tissue_name", "water"),
                kernel_resolution=self.config.get("kernel_resolution", 1.0),
                config=self.config)
        elif kind == "monte_carlo":
            from .monte_carlo import MonteCarloCalculator
            self.calculator = MonteCarloCalculator(
                radionuclide=radionuclide,
                tissue_composition=self.config.get("tissue_composition", None),
                n_particles=self.config.get("n_particles", 1000000),
                random_seed=self.config.get("random_seed", None),
                config=self.config)
        elif kind == "nn_corrected":
            from .learned_correction import NNCorrectedDoseCalculator
            self.calculator = NNCorrectedDoseCalculator(radionuclide, self.config.get("tissue_composition", None),
                                                        self.config)
        elif kind == "gate":
            raise NotImplementedError("gate_monte_carlo drives the external GATE/Geant4 application, which this "
                                      "package does not provide; use method='monte_carlo'")
        else:
            raise ValueError(f"Unsupported calculation method: {method}")
        nuc = radionuclide if isinstance(radionuclide, str) else radionuclide[0]
        half_life = self.config.get("half_life")
        units = self.config.get("time_units", "hours")
        if half_life is None:
            half_life = nd.get_nuclide(nuc).half_life_h * 3600.0 / SECONDS_PER.get(units, 3600.0)
        self.activity_sampler = ActivitySampler(half_life=half_life, units=units)

    def calculate_dose(self, activity_maps=None, time_points: Optional[List[float]] = None,
                       voxel_size: Tuple[float, float, float] = (1.0, 1.0, 1.0), tissue_densities=None,
                       accumulated_activity=None, integration_mode: str = "activity",
                       integration_limit: Optional[float] = None, ct_image=None) -> DoseCalculationResult:
        """Absorbed dose or dose rate depending on the input (routing of
        core/dose_calculator.py:85-164).  ``ct_image`` (HU, same shape as the activity),
        used when ``tissue_densities`` is not given, supplies the density through
        TissueComposition's HU calibration (``config['hu_density_calibration']``,
        metal-artefact step unless ``config['handle_artifacts']`` is False)."""
        if len(voxel_size) != 3:
            raise ValueError("voxel_size must be a tuple of length 3.")
        calc = self.calculator
        if tissue_densities is None and ct_image is not None:
            from ..tissue import TissueComposition
            tissue_densities = TissueComposition(self.config).calculate_density(
                ct_image, handle_artifacts=self.config.get("handle_artifacts", True))

        if accumulated_activity is not None:
            sec = SECONDS_PER[self.activity_sampler.units]
            dose = calc.calculate_absorbed_dose_from_accumulated(accumulated_activity, voxel_size,
                                                                 density=tissue_densities, seconds_per_unit=sec)
            return DoseCalculationResult(dose, [], [], {"mode": "accumulated_activity"})

        if activity_maps is not None and time_points is not None and len(activity_maps) > 1:
            self._validate_inputs(activity_maps, time_points, voxel_size)
            if integration_mode == "activity":
                # trapezoid of activity then dose == one convolution of the trapezoid-weighted
                # activity; calculate_absorbed_dose fuses the weighting into the first FFT pass
                sec = SECONDS_PER[self.activity_sampler.units]
                dose = calc.calculate_absorbed_dose(activity_maps, [t * sec / 3600.0 for t in time_points],
                                                    voxel_size, density=tissue_densities)
                return DoseCalculationResult(dose, [], list(time_points), {"mode": "multi_timepoint_activity"})
            elif integration_mode == "dose_rate":
                rates = [calc.calculate_dose_rate(a, voxel_size, density=tissue_densities) for a in activity_maps]
                dose = self.activity_sampler.integrate_dose_rates(rates, list(time_points), integration_limit)
                return DoseCalculationResult(dose, rates, list(time_points), {"mode": "multi_timepoint_doserate"})
            else:
                raise ValueError(f"Unknown integration_mode: {integration_mode}")

        if activity_maps is not None and len(activity_maps) == 1:
            self._validate_inputs(activity_maps, time_points or [0], voxel_size)
            rate = calc.calculate_dose_rate(activity_maps[0], voxel_size, density=tissue_densities)
            absorbed = None
            if self.config.get("single_timepoint_dose") == "physical_decay":
                tau = self.activity_sampler.half_life * SECONDS_PER[self.activity_sampler.units] / math.log(2.0)
                absorbed = rate * tau
            return DoseCalculationResult(absorbed, [rate], list(time_points or []), {"mode": "single_timepoint"})

        raise ValueError("Invalid input for dose calculation.")

    def _validate_inputs(self, activity_maps, time_points, voxel_size):
        if not activity_maps:
            raise ValueError("No activity maps provided")
        if len(activity_maps) != len(time_points):
            raise ValueError("Number of activity maps must match number of time points")
        if len(voxel_size) != 3:
            raise ValueError("Voxel size must be 3D")
        shape = tuple(activity_maps[0].shape)
        if not all(tuple(m.shape) == shape for m in activity_maps):
            raise ValueError("All activity maps must have the same dimensions")

"""Plugin interface every dose method implements.

Mirrors DosimetryCalculator (pyvoxeldosimetry/core/dosimetry_base.py:8-70):
same constructor, same abstract methods, same TypeError for a non-string
radionuclide.  One extension: ``radionuclide`` may also be a list/tuple of
strings, in which case results carry a leading nuclide axis.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Any, Dict, List, Optional, Tuple


class DosimetryCalculator(ABC):
    """Abstract base class for all dosimetry calculation methods."""

    def __init__(self, radionuclide, tissue_composition: Any, config: Optional[Dict[str, Any]] = None):
        self.radionuclide = radionuclide
        self.tissue_composition = tissue_composition
        self.config = config or {}
        self._validate_inputs()

    def _validate_inputs(self):
        r = self.radionuclide
        if isinstance(r, str):
            return
        if isinstance(r, (list, tuple)) and r and all(isinstance(x, str) for x in r):
            return
        raise TypeError("Radionuclide must be a string")

    @property
    def nuclides(self) -> List[str]:
        return [self.radionuclide] if isinstance(self.radionuclide, str) else list(self.radionuclide)

    @abstractmethod
    def calculate_dose_rate(self, activity_map, voxel_size: Tuple[float, float, float]):
        """Dose rate (Gy/s) from an activity map (Bq per voxel); voxel size in mm."""

    @abstractmethod
    def calculate_absorbed_dose(self, activity_maps, time_points: List[float],
                                voxel_size: Tuple[float, float, float]):
        """Absorbed dose (Gy) from activity maps at ``time_points`` (hours)."""

    def get_config(self) -> Dict[str, Any]:
        return self.config.copy()

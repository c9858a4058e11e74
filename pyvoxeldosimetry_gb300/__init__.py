"""GB300-native (sm_103a) voxel dosimetry: a drop-in for the dose-calculation
hot path of devhliu/PyVoxelDosimetry.

Public names mirror the reference package (pyvoxeldosimetry/__init__.py:8-21,
pyvoxeldosimetry/core/__init__.py:7-24).  All dose arithmetic runs in the CUDA
library ``libpvd_gb300.so`` behind the C ABI in ``include/pvd.h``; importing
this package does not need a GPU, using it does.
"""
__version__ = "0.1.0"

from .core.dosimetry_base import DosimetryCalculator
from .core.kernel_convolution import KernelConvolutionCalculator
from .core.activity_sampler import ActivitySampler
from .core.dose_calculator import DoseCalculator, DoseCalculationResult
from .core.monte_carlo import MonteCarloCalculator
from .time_integration.curve_fitting import TimeCurveFitting
from .core.utils import calculate_dvh, load_dose_map, resample_dose_map, resample_volume, save_dose_map
from .data.dose_kernels import KernelFactory
from .batch import BatchDoseCalculator
from .core.learned_correction import NNCorrectedDoseCalculator, UNet3D
from .tissue import TissueComposition
from .data.mc_decay import load_decay_data

__all__ = [
    "TissueComposition", "load_decay_data",
    "NNCorrectedDoseCalculator",
    "UNet3D",
    "DosimetryCalculator",
    "KernelConvolutionCalculator",
    "ActivitySampler",
    "DoseCalculator",
    "DoseCalculationResult",
    "MonteCarloCalculator",
    "TimeCurveFitting",
    "calculate_dvh",
    "save_dose_map",
    "load_dose_map",
    "resample_dose_map",
    "resample_volume",
    "KernelFactory",
    "BatchDoseCalculator",
]

"""CT-derived tissue composition and mass density on the GPU."""
from .composition import DEFAULT_HU_DENSITY, TissueComposition

__all__ = ["TissueComposition", "DEFAULT_HU_DENSITY"]

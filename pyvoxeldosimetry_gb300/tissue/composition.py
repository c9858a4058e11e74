"""Tissue composition (and mass density) from a CT image in Hounsfield units.

Mirrors TissueComposition (pyvoxeldosimetry/tissue/composition.py:36-93): same
constructor, the same ``tissue_types`` HU ranges, and ``calculate_composition(
ct_image, handle_artifacts=True)`` returning the same dict of masks (air, lung,
soft_tissue, bone, water; closed ranges that overlap and leave gaps exactly as the
reference's do) after the same metal-artefact step (voxels above 2000 HU take the
value of the Gaussian-smoothed image, sigma 1 voxel).  Everything runs in one pass
on the GPU (``pvd_hu_composition``).  numpy in -> float64 numpy masks out, as in the
reference; CUDA tensor in -> float32 CUDA masks.

Added, because the reference has no step from HU to the density its dose
calculator's ``tissue_densities`` expects (core/dose_calculator.py:90):
``calculate_density`` (and ``calculate_composition_and_density``) give the mass
density by linear interpolation through (HU, g/cc) calibration points, by default
``DEFAULT_HU_DENSITY``: air 0.0012 g/cc at -1000 HU, water 1.0 at 0 HU (lung of
0.26 g/cc falls at about -740 HU on that line), the reference's cortical bone
1.85 g/cc at +1000 HU (data/dose_kernels/tissue_properties.py:20-26) and the same
slope up to 3000 HU; clamped beyond the end points.
"""
from __future__ import annotations

import ctypes as C
from typing import Any, Dict, Optional, Sequence, Tuple

import numpy as np
import torch

from .. import _io
from .. import _native as N
from ..conv import _require_cuda

TISSUE_ORDER = ("air", "lung", "soft_tissue", "bone", "water")
DEFAULT_HU_DENSITY: Tuple[Tuple[float, float], ...] = ((-1000.0, 0.0012), (0.0, 1.0), (1000.0, 1.85), (3000.0, 2.85))


class TissueComposition:
    def __init__(self, config: Optional[Dict[str, Any]] = None):
        self.config = config or {}
        self.tissue_types = {
            "air": {"hu_range": (-1000, -900)},
            "lung": {"hu_range": (-900, -500)},
            "soft_tissue": {"hu_range": (-100, 100)},
            "bone": {"hu_range": (300, 3000)},
            "water": {"hu_range": (-10, 10)},
        }
        self.calibration = tuple(tuple(map(float, p)) for p in
                                 self.config.get("hu_density_calibration", DEFAULT_HU_DENSITY))
        self.device = self.config.get("device")

    def _run(self, ct_image, handle_artifacts: bool, masks: bool, density: bool):
        kind = _io.kind_of(ct_image)
        device = _require_cuda(self.device if self.device is not None else
                               (ct_image.device if kind == _io.CUDA_TENSOR else None))
        lib = N.load()
        with torch.cuda.device(device):
            ct = _io.to_device(ct_image, device, "ct_image")
            if ct.dim() != 3:
                raise ValueError("ct_image must be 3-D")
            n = ct.numel()
            m = torch.empty((5, *ct.shape), dtype=torch.uint8, device=device) if masks else None
            rho = torch.empty(ct.shape, dtype=torch.float32, device=device) if density else None
            hu = (C.c_float * len(self.calibration))(*[p[0] for p in self.calibration])
            rv = (C.c_float * len(self.calibration))(*[p[1] for p in self.calibration])
            N.check(lib.pvd_hu_composition(ct.data_ptr(), *ct.shape, N.PVD_HU_ARTIFACTS if handle_artifacts else 0,
                                           hu, rv, len(self.calibration), m.data_ptr() if m is not None else None,
                                           rho.data_ptr() if rho is not None else None, None,
                                           torch.cuda.current_stream(device).cuda_stream))
            del n
        out_m = None
        if masks:
            if kind == _io.CUDA_TENSOR:
                mf = m.to(torch.float32)
                out_m = {t: mf[i] for i, t in enumerate(TISSUE_ORDER)}
            else:
                mh = m.cpu().numpy()
                out_m = {t: mh[i].astype(float) for i, t in enumerate(TISSUE_ORDER)}
                if kind == _io.CPU_TENSOR:
                    out_m = {t: torch.from_numpy(v) for t, v in out_m.items()}
        out_r = None
        if density:
            out_r = rho if kind == _io.CUDA_TENSOR else _io.from_device(rho, kind)
        return out_m, out_r

    def calculate_composition(self, ct_image, handle_artifacts: bool = True) -> Dict[str, Any]:
        """Masks of the tissue classes (1.0 inside the class's HU range, else 0.0)."""
        return self._run(ct_image, handle_artifacts, True, False)[0]

    def calculate_density(self, ct_image, handle_artifacts: bool = True):
        """Mass density (g/cc, float32) from the HU calibration; 0 where the CT is NaN."""
        return self._run(ct_image, handle_artifacts, False, True)[1]

    def calculate_composition_and_density(self, ct_image, handle_artifacts: bool = True):
        """Both in one pass over the volume: (masks dict, density)."""
        return self._run(ct_image, handle_artifacts, True, True)

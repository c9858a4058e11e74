"""Dose-point-kernel library: the reference's kernel factory and generators
(pyvoxeldosimetry/data/dose_kernels/kernel_factory.py:12-75, *_kernel.py),
evaluated on the GPU in FP64 (``pvd_radial_kernel``).

Each generator is a list of radial terms (see include/pvd.h) built from the
nuclide's data and the tissue tables of the reference's generators:

  Y90    Cole beta, range 11 Emax^1.5 / (rho SPR), weight rho SPR; bremsstrahlung
         photons 0.015 (Z/7.42)^2 rho, mu = 0.096 rho; times the tissue factor
         (y90_kernel.py:20-161)
  Lu177  per branch Cole beta, range 5 Emax^1.5 / (rho SPR), weight abundance rho SPR;
         gamma lines, mu = rho (mu/rho) (0.2/E)^3.2 (lu177_kernel.py:52-184)
  Ga68   positron Cole term, range 9 Emax^1.5 x tissue factor; 511 keV annihilation
         and gamma-line photons with the tissue's mu x (0.511/E)^3.2; times the tissue
         factor (ga68_kernel.py:19-106)
  Ac225  parent and daughter alphas (1 - (r/R)^1.7) exp(-4.5 r/R) E/5, R = 0.0006 E^1.7
         x the tissue's alpha range factor; gamma lines with
         mu = 0.096 (0.5/E)^3.2 (Z/7.42)^0.5 rho (ac225_kernel.py:37-191)
  F18    the reference's generator is a stub (f18_kernel.py:33-45 return None): the
         Ga-68 form with F-18's data (Emax 0.634 MeV, no gamma lines)
  Tb161  the reference's class is abstract (tb161_kernel.py): the Lu-177 form with
         Tb-161's branches and gamma lines (Tb161.json)

Differences from the reference, each deliberate: the JSON data files the
reference cannot parse (they carry // comments) are restated as tables here;
r = 0 uses the radius of the sphere of the voxel's volume for photon terms
(``reference_r0=True`` gives the reference's NaN / 0); the Ac-225 kernel has no
overall tissue factor (the reference calls a method it does not define,
ac225_kernel.py:95); the cache is keyed by nuclide, tissue, voxel size, grid
and the r = 0 rule (the reference keys it by nuclide and tissue only, so a
second voxel size returns the first one's kernel), kept in memory and, with
``cache_dir``, on disk; no plots are written.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path
from typing import Dict, List, Optional, Tuple

import numpy as np

# density, effective Z, stopping-power ratio, mu/rho (lu177_kernel.py:88-127, tb161_kernel.py:21-59,
# y90_kernel.py:57-91, ac225_kernel.py:99-138 share these values)
TISSUES = {
    "water": (1.0, 7.42, 1.0, 0.096),
    "lung": (0.26, 7.41, 1.04, 0.095),
    "soft_tissue": (1.04, 7.46, 1.04, 0.097),
    "bone": (1.85, 13.8, 1.15, 0.110),
    "iodine_contrast": (1.30, 53.0, 1.12, 0.245),
}
Y90_TISSUE_FACTOR = {"water": 1.0, "lung": 1.04, "soft_tissue": 1.04, "bone": 1.15, "iodine_contrast": 1.12}
GA_TISSUE_FACTOR = {"water": 1.0, "lung": 0.3, "soft_tissue": 1.04, "bone": 1.6, "iodine_contrast": 1.3}
GA_MU = {"water": 0.096, "lung": 0.029, "soft_tissue": 0.099, "bone": 0.172, "iodine_contrast": 0.158}
AC_ALPHA_RANGE_FACTOR = {"water": 1.0, "lung": 3.85, "soft_tissue": 0.96, "bone": 0.54, "iodine_contrast": 0.77}

# nuclide data (data/dose_kernels/*/*.json)
Y90_EMAX = 2.280
LU177_BRANCHES = ((0.498, 0.795), (0.385, 0.089), (0.177, 0.116))
LU177_GAMMAS = ((0.208, 0.111), (0.113, 0.062))
TB161_BRANCHES = ((0.593, 0.504), (0.453, 0.222), (0.419, 0.274))
TB161_GAMMAS = ((0.0487, 0.171), (0.0574, 0.103), (0.0749, 0.136))
GA68_EMAX, GA68_GAMMAS = 1.899, ((1.077, 0.03),)
F18_EMAX = 0.634
AC225_ALPHAS = ((5.830, 0.506), (5.792, 0.494), (6.341, 1.0), (7.067, 1.0), (5.875, 1.0), (8.375, 1.0))
AC225_GAMMAS = ((0.100, 0.012), (0.150, 0.036), (0.440, 0.026))

# kernel_factory.py:24-31
DEFAULT_GRID_SIZES = {
    "F18": (101, 101, 101), "Ga68": (151, 151, 151), "Y90": (201, 201, 201),
    "Lu177": (81, 81, 81), "Tb161": (71, 71, 71), "Ac225": (251, 251, 251),
}
SUPPORTED = list(DEFAULT_GRID_SIZES)


def _tissue(tissue: str):
    return TISSUES.get(tissue, TISSUES["water"])


def kernel_terms(nuclide: str, tissue: str, reference_r0: bool = False) -> Tuple[List[tuple], float]:
    """(terms, scale): terms as (type, center, weight, p1, p2, p3) tuples (see include/pvd.h)."""
    from .. import _native as N
    rho, z, spr, mur = _tissue(tissue)
    center_nan = N.PVD_CENTER_NAN if reference_r0 else N.PVD_CENTER_R0
    center_zero = N.PVD_CENTER_ZERO if reference_r0 else N.PVD_CENTER_R0
    cole, photon, alpha = N.PVD_TERM_COLE, N.PVD_TERM_PHOTON, N.PVD_TERM_ALPHA
    if nuclide == "Y90":
        terms = [(cole, 0, rho * spr, 11.0 * Y90_EMAX ** 1.5 / rho / spr, 0.0, 0.0),
                 (photon, center_nan, 0.015 * (z / 7.42) ** 2 * rho, 0.096 * rho, 0.0, 0.0)]
        return terms, Y90_TISSUE_FACTOR.get(tissue, 1.0)
    if nuclide in ("Lu177", "Tb161"):
        branches, gammas = (LU177_BRANCHES, LU177_GAMMAS) if nuclide == "Lu177" else (TB161_BRANCHES, TB161_GAMMAS)
        terms = [(cole, 0, ab * rho * spr, 5.0 * e ** 1.5 / rho / spr, 0.0, 0.0) for e, ab in branches]
        terms += [(photon, center_zero, inten, rho * mur * (0.2 / e) ** 3.2, 0.0, 0.0) for e, inten in gammas]
        return terms, 1.0
    if nuclide in ("Ga68", "F18"):
        e_max, gammas = (GA68_EMAX, GA68_GAMMAS) if nuclide == "Ga68" else (F18_EMAX, ())
        f = GA_TISSUE_FACTOR.get(tissue, 1.0)
        mu0 = GA_MU.get(tissue, 0.096)
        terms = [(cole, 0, 1.0, 9.0 * e_max ** 1.5 * f, 0.0, 0.0),
                 (photon, center_nan, 1.0, mu0 * (0.511 / 0.511) ** 3.2, 0.0, 0.0)]
        terms += [(photon, center_nan, inten, mu0 * (0.511 / e) ** 3.2, 0.0, 0.0) for e, inten in gammas]
        return terms, f
    if nuclide == "Ac225":
        arf = AC_ALPHA_RANGE_FACTOR.get(tissue, 1.0)
        terms = [(alpha, 0, inten * (e / 5.0), 0.0006 * e ** 1.7 * arf, 1.7, 4.5) for e, inten in AC225_ALPHAS]
        terms += [(photon, center_zero, inten, 0.096 * (0.5 / e) ** 3.2 * (z / 7.42) ** 0.5 * rho, 0.0, 0.0)
                  for e, inten in AC225_GAMMAS]
        return terms, 1.0
    raise ValueError(f"Unsupported nuclide: {nuclide}. Supported: {SUPPORTED}")


def generate_kernel(nuclide: str, tissue: str, voxel_size: float, grid_size, reference_r0: bool = False,
                    device=None, as_tensor: bool = False):
    """The nuclide's kernel on a grid centred on voxel grid//2, FP64, computed on the GPU.
    Returns numpy (default) or the CUDA tensor."""
    import torch
    from .. import _native as N
    from ..conv import _require_cuda
    dev = _require_cuda(device)
    terms, scale = kernel_terms(nuclide, tissue, reference_r0)
    grid = tuple(int(g) for g in grid_size)
    if len(grid) != 3 or min(grid) < 1:
        raise ValueError("grid_size must be three positive integers")
    vs = (float(voxel_size),) * 3 if np.isscalar(voxel_size) else tuple(float(v) for v in voxel_size)
    arr = (N.RadialTerm * len(terms))(*[N.RadialTerm(*t) for t in terms])
    lib = N.load()
    with torch.cuda.device(dev):
        out = torch.empty(grid, dtype=torch.float64, device=dev)
        N.check(lib.pvd_radial_kernel(arr, len(terms), float(scale), *grid, (C.c_double * 3)(*vs), out.data_ptr(),
                                      torch.cuda.current_stream(dev).cuda_stream))
        return out if as_tensor else out.cpu().numpy()


class KernelFactory:
    """Drop-in for the reference's KernelFactory (kernel_factory.py:12-75)."""

    _default_grid_sizes: Dict[str, Tuple[int, int, int]] = dict(DEFAULT_GRID_SIZES)

    def __init__(self, cache_dir: Optional[str] = None, reference_r0: bool = False, device=None):
        self.cache_dir = Path(cache_dir) if cache_dir else None
        if self.cache_dir is not None:
            self.cache_dir.mkdir(parents=True, exist_ok=True)
        self.reference_r0 = reference_r0
        self.device = device
        self._cache: Dict[tuple, np.ndarray] = {}
        self._lock = threading.Lock()

    @classmethod
    def supported_nuclides(cls) -> List[str]:
        return list(cls._default_grid_sizes)

    def get_kernel(self, nuclide: str, tissue_type: str, voxel_size: float = 1.0,
                   grid_size: Optional[Tuple[int, int, int]] = None, force_regenerate: bool = False) -> np.ndarray:
        """The kernel of ``nuclide`` in ``tissue_type`` at ``voxel_size`` mm on ``grid_size``
        (the reference's default grid per nuclide when None); ValueError for an
        unsupported nuclide, as the reference."""
        if nuclide not in self._default_grid_sizes:
            raise ValueError(f"Unsupported nuclide: {nuclide}. Supported: {list(self._default_grid_sizes)}")
        grid = tuple(int(g) for g in (grid_size or self._default_grid_sizes[nuclide]))
        key = (nuclide, tissue_type, float(voxel_size), grid, bool(self.reference_r0))
        with self._lock:
            if not force_regenerate and key in self._cache:
                return self._cache[key].copy()
            path = None
            if self.cache_dir is not None:
                r0 = "ref_r0" if self.reference_r0 else "r0"
                path = self.cache_dir / (f"{nuclide}_{tissue_type}_{float(voxel_size):g}mm_"
                                         f"{grid[0]}x{grid[1]}x{grid[2]}_{r0}.npy")
                if not force_regenerate and path.exists():
                    k = np.load(path)
                    self._cache[key] = k
                    return k.copy()
            k = generate_kernel(nuclide, tissue_type, voxel_size, grid, self.reference_r0, self.device)
            self._cache[key] = k
            if path is not None:
                np.save(path, k)
            return k.copy()

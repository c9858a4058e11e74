"""Radionuclide data and dose-point-kernel builders (host, FP64).

Nuclide constants restate the reference's data files (paths within
devhliu/PyVoxelDosimetry):
  Y90  : data/dose_kernels/Y90/Y90.json:16-23 (T1/2 64.1 h, Emax 2.280, Emean 0.934 MeV);
         data/mc_decay/Y90.json:5-19 (beta spectrum points)
  Lu177: data/mc_decay/Lu177.json:5-32 (T1/2 6.647 d, Emean 0.149, Emax 0.498 MeV, gammas);
         data/dose_kernels/Lu177/Lu177.json:21-26 (beta branches, used by the reference generator)
  I131 : data/mc_decay/I131.json:5-38 (T1/2 8.0207 d, Emean 0.182, Emax 0.807 MeV, gammas)
  F18, Ga68, Tb161: data/dose_kernels/*/ *.json "half_life" and mean/max energies.

Kernel profiles:
  "analytic"  : k(r) = exp(-r/lambda)/r^2, lambda = 1.8 mm for Y-90 and scaled by the
                nuclide's beta CSDA range (data/mc_decay/*.json "beta_csda_range") for
                the others; the centre voxel uses the radius of the sphere of equal
                volume r0 = (3 dV / 4 pi)^(1/3).  Normalised (on the GPU, FP64) so the
                kernel sums to 1, then scaled to Gy/(Bq s) by the mean beta energy.
  "reference" : the reference generators' kernels (data.dose_kernels, GPU FP64) with the
                r = 0 singularity of the photon terms replaced by r0 (the reference
                produces NaN there, y90_kernel.py:134-138).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import mc_decay

JOULE_PER_MEV = 1.602176634e-13


@dataclass(frozen=True)
class Nuclide:
    symbol: str
    half_life_h: float
    beta_mean_mev: float
    beta_max_mev: float
    beta_csda_range_mm: float
    kernel_reach_mm: float                     # half-width of the default kernel grid
    spectrum_e: tuple = ()                     # beta spectrum sample energies (MeV)
    spectrum_p: tuple = ()                     # relative probability density at spectrum_e
    gammas: tuple = ()                         # ((energy MeV, photons per decay), ...)
    beta_branches: tuple = ()                  # ((Emax MeV, abundance), ...) for the reference generator
    extra: dict = field(default_factory=dict)


NUCLIDES = {
    # Y-90's kernel half-life is data/dose_kernels/Y90/Y90.json's 64.1 h (the Monte Carlo
    # data file says 64.053 h); spectra and gamma lines come from the Monte Carlo data
    "Y90": Nuclide("Y90", 64.1, 0.934, 2.280, 11.3, 15.0,
                   spectrum_e=mc_decay.beta_spectrum("Y90")[0], spectrum_p=mc_decay.beta_spectrum("Y90")[1],
                   beta_branches=((2.280, 1.0),)),
    "Lu177": Nuclide("Lu177", mc_decay.half_life_hours("Lu177"), 0.149, 0.498, 1.7, 6.0,
                     spectrum_e=mc_decay.beta_spectrum("Lu177")[0], spectrum_p=mc_decay.beta_spectrum("Lu177")[1],
                     gammas=mc_decay.gamma_lines("Lu177"),
                     beta_branches=((0.498, 0.795), (0.385, 0.089), (0.177, 0.116))),
    "I131": Nuclide("I131", mc_decay.half_life_hours("I131"), 0.182, 0.807, 3.2, 7.5,
                    spectrum_e=mc_decay.beta_spectrum("I131")[0], spectrum_p=mc_decay.beta_spectrum("I131")[1],
                    gammas=mc_decay.gamma_lines("I131")),
    "F18": Nuclide("F18", 1.8295, 0.250, 0.634, 2.4, 6.0),
    "Ga68": Nuclide("Ga68", 1.128, 0.836, 1.899, 9.0, 12.0),
    "Tb161": Nuclide("Tb161", 165.432, 0.154, 0.593, 1.8, 6.0),
    # alpha emitter (data/dose_kernels/Ac225/Ac225.json): kernels only from the reference
    # generator's form (kernel_profile='reference'); no beta terms
    "Ac225": Nuclide("Ac225", 240.0, 0.0, 0.0, 0.0, 5.0, extra={"alpha": True}),
}

Y90_LAMBDA_MM = 1.8


def get_nuclide(symbol: str) -> Nuclide:
    try:
        return NUCLIDES[symbol]
    except KeyError:
        raise ValueError(f"Unsupported nuclide: {symbol}. Supported: {sorted(NUCLIDES)}") from None


def _vox3(voxel_size):
    if np.isscalar(voxel_size):
        return (float(voxel_size),) * 3
    v = tuple(float(x) for x in voxel_size)
    if len(v) != 3:
        raise ValueError("voxel_size must be a scalar or a 3-tuple")
    return v


def default_kernel_size(symbol: str, voxel_size, density: float = 1.0) -> tuple:
    """Odd kernel dims covering +/- the nuclide's kernel reach (15 mm Y-90, 6 mm Lu-177,
    7.5 mm I-131) in a medium of the given density (reach / density): 15^3 at 2 mm and
    21^3 at 1.5 mm for Y-90 in water, 9^3 / 11^3 at 1.5 mm."""
    nuc = get_nuclide(symbol)
    reach = nuc.kernel_reach_mm / float(density)
    return tuple(2 * int(math.floor(reach / d + 1e-9)) + 1 for d in _vox3(voxel_size))


def radius_grid(shape, voxel_size) -> np.ndarray:
    """Distance (mm) of each kernel voxel centre from the centre voxel shape//2."""
    v = _vox3(voxel_size)
    idx = np.indices(shape, dtype=np.float64)
    return np.sqrt(sum(((idx[i] - shape[i] // 2) * v[i]) ** 2 for i in range(3)))


def equal_volume_radius(voxel_size) -> float:
    v = _vox3(voxel_size)
    return (3.0 * v[0] * v[1] * v[2] / (4.0 * math.pi)) ** (1.0 / 3.0)


def analytic_lambda_mm(symbol: str) -> float:
    nuc = get_nuclide(symbol)
    if nuc.extra.get("alpha"):
        raise ValueError(f"{symbol} is an alpha emitter: no analytic beta profile; use kernel_profile='reference'")
    return Y90_LAMBDA_MM * nuc.beta_csda_range_mm / NUCLIDES["Y90"].beta_csda_range_mm


def analytic_profile(symbol: str, voxel_size, shape=None, density: float = 1.0) -> np.ndarray:
    """Un-normalised exp(-r/lambda)/r^2 kernel (FP64), centre voxel at r0.  ``density``
    gives the kernel of a homogeneous medium of that density relative to water: the decay
    length becomes lambda / density (ranges scale inversely with density)."""
    shape = tuple(shape) if shape is not None else default_kernel_size(symbol, voxel_size, density)
    r = radius_grid(shape, voxel_size)
    r = np.where(r == 0.0, equal_volume_radius(voxel_size), r)
    lam = analytic_lambda_mm(symbol) / float(density)
    return np.exp(-r / lam) / (r * r)


def gy_per_bq_s_scale(symbol: str, voxel_size, water_density: float = 1.0, energy_mev=None) -> float:
    """Mean beta energy per decay deposited in one voxel of water, in Gy per (Bq s):
    E_mean [MeV] * 1.602176634e-13 [J/MeV] / (rho * dV [mm^3] * 1e-6 [kg / (g/cc mm^3)]).
    ``energy_mev`` replaces the nuclide's stated mean beta energy (e.g. the mean of the
    spectrum the Monte Carlo samples, ``mc_physics.spectrum_mean``)."""
    v = _vox3(voxel_size)
    nuc = get_nuclide(symbol)
    if nuc.extra.get("alpha"):
        raise ValueError(f"{symbol} is an alpha emitter: no analytic beta profile; use kernel_profile='reference'")
    e = nuc.beta_mean_mev if energy_mev is None else float(energy_mev)
    return e * JOULE_PER_MEV / (water_density * v[0] * v[1] * v[2] * 1e-6)


def reference_profile(symbol: str, tissue: str, voxel_size: float, shape, fix_r0: bool = True) -> np.ndarray:
    """The reference generator's kernel for ``symbol`` (Y90, Lu177, Ga68, F18, Tb161,
    Ac225), computed on the GPU by the kernel library (``data.dose_kernels``).  With
    ``fix_r0`` the photon terms use the radius of the sphere of the voxel's volume at
    the centre voxel instead of the reference's NaN (0 * inf) or 0."""
    from .dose_kernels import generate_kernel
    if symbol not in ("Y90", "Lu177", "Ga68", "F18", "Tb161", "Ac225"):
        raise ValueError(f"no reference generator for {symbol}")
    return generate_kernel(symbol, tissue, voxel_size, tuple(shape), reference_r0=not fix_r0)

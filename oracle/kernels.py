"""ORACLE — test infrastructure only, never the product path.

FP64 numpy restatement of the reference's dose-point-kernel generators
(pyvoxeldosimetry/data/dose_kernels/*_kernel.py), term by term, and of the
two that the reference leaves unfinished (F-18: stub methods returning None,
f18_kernel.py:33-45; Tb-161: abstract, no generate_kernel, tb161_kernel.py),
which the GPU library defines with the reference's own Ga-68 and Lu-177 forms
and the nuclides' data files.  ``reference_r0=True`` keeps the reference's value
at r = 0 for the photon terms (NaN for Y-90 and Ga-68, 0 for Lu-177 and
Ac-225); otherwise r = 0 is replaced by the radius of the sphere of the voxel's
volume.  Checked against vectors produced by the reference itself
(tests/golden/make_golden.py).
"""
from __future__ import annotations

import numpy as np

# tissue tables of the generators (y90_kernel.py:57-91, lu177_kernel.py:88-127,
# tb161_kernel.py:21-59, ac225_kernel.py:99-138, ga68_kernel.py:86-106)
LU_TISSUE = {
    "water": (1.0, 7.42, 1.0, 0.096), "lung": (0.26, 7.41, 1.04, 0.095), "soft_tissue": (1.04, 7.46, 1.04, 0.097),
    "bone": (1.85, 13.8, 1.15, 0.110), "iodine_contrast": (1.30, 53.0, 1.12, 0.245),
}  # density, effective Z, stopping-power ratio, mu/rho
AC_RANGE = {"water": 1.0, "lung": 3.85, "soft_tissue": 0.96, "bone": 0.54, "iodine_contrast": 0.77}
GA_SCALE = {"water": 1.0, "lung": 0.3, "soft_tissue": 1.04, "bone": 1.6, "iodine_contrast": 1.3}
GA_MU = {"water": 0.096, "lung": 0.029, "soft_tissue": 0.099, "bone": 0.172, "iodine_contrast": 0.158}
Y90_SCALE = {"water": 1.0, "lung": 1.04, "soft_tissue": 1.04, "bone": 1.15, "iodine_contrast": 1.12}


def radius(grid, voxel):
    c = [s // 2 for s in grid]
    x, y, z = np.meshgrid(*(np.arange(g) - cc for g, cc in zip(grid, c)), indexing="ij")
    return np.sqrt((x * voxel) ** 2 + (y * voxel) ** 2 + (z * voxel) ** 2)


def r0_of(voxel):
    return (3.0 * voxel ** 3 / (4.0 * np.pi)) ** (1.0 / 3.0)


def cole(r, rng, weight):
    """weight (1 - r/R)^2 exp(-2 r/R) for r <= R, else 0."""
    out = np.zeros_like(r)
    m = r <= rng
    out[m] = (1 - r[m] / rng) ** 2 * np.exp(-2 * r[m] / rng) * weight
    return out


def photon(r, mu, weight, reference_r0, voxel, nan_at_zero):
    rc = r if reference_r0 else np.where(r == 0.0, r0_of(voxel), r)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = weight * np.exp(-mu * rc / 10) / (4 * np.pi * rc ** 2)
    if reference_r0:
        v = np.where(r > 0, v, np.nan if nan_at_zero else 0.0)
    return v


def alpha(r, rng, weight):
    """weight (1 - (r/R)^1.7) exp(-4.5 r/R) for r <= R (ac225_kernel.py:140-166)."""
    out = np.zeros_like(r)
    m = r <= rng
    out[m] = (1 - (r[m] / rng) ** 1.7) * np.exp(-4.5 * r[m] / rng) * weight
    return out


def y90(tissue, voxel, grid, reference_r0=False):
    """y90_kernel.py:20-55, 93-161."""
    rho, z, spr, _ = LU_TISSUE.get(tissue, LU_TISSUE["water"])
    r = radius(grid, voxel)
    k = cole(r, 11.0 * 2.280 ** 1.5 / rho / spr, rho * spr)
    k = k + photon(r, 0.096 * rho, 0.015 * (z / 7.42) ** 2 * rho, reference_r0, voxel, True)
    return k * Y90_SCALE.get(tissue, 1.0)


def lu177(tissue, voxel, grid, reference_r0=False,
          branches=((0.498, 0.795), (0.385, 0.089), (0.177, 0.116)),
          gammas=((0.208, 0.111), (0.113, 0.062))):
    """lu177_kernel.py:52-86, 129-184 (Tb-161 uses the same form with its own data)."""
    rho, _, spr, mur = LU_TISSUE.get(tissue, LU_TISSUE["water"])
    r = radius(grid, voxel)
    k = np.zeros_like(r)
    for e, ab in branches:
        k += ab * cole(r, 5.0 * e ** 1.5 / rho / spr, rho * spr)
    for e, inten in gammas:
        k += photon(r, rho * mur * (0.2 / e) ** 3.2, inten, reference_r0, voxel, False)
    return k


def tb161(tissue, voxel, grid, reference_r0=False):
    """Tb-161 with the Lu-177 generator's form and Tb161.json's branches and gamma lines."""
    return lu177(tissue, voxel, grid, reference_r0,
                 branches=((0.593, 0.504), (0.453, 0.222), (0.419, 0.274)),
                 gammas=((0.0487, 0.171), (0.0574, 0.103), (0.0749, 0.136)))


def ga68(tissue, voxel, grid, reference_r0=False, e_max=1.899, gammas=((1.077, 0.03),)):
    """ga68_kernel.py:19-106: positron Cole term (range 9 Emax^1.5 x tissue factor),
    511 keV annihilation photons, gamma lines, all times the tissue factor."""
    f = GA_SCALE.get(tissue, 1.0)
    mu0 = GA_MU.get(tissue, 0.096)
    r = radius(grid, voxel)
    k = cole(r, 9.0 * e_max ** 1.5 * f, 1.0)
    k = k + photon(r, mu0 * (0.511 / 0.511) ** 3.2, 1.0, reference_r0, voxel, True)
    for e, inten in gammas:
        k = k + photon(r, mu0 * (0.511 / e) ** 3.2, inten, reference_r0, voxel, True)
    return k * f


def f18(tissue, voxel, grid, reference_r0=False):
    """F-18 with the Ga-68 generator's form and F18.json's data (Emax 0.634 MeV, no gammas)."""
    return ga68(tissue, voxel, grid, reference_r0, e_max=0.634, gammas=())


AC_ALPHAS = ((5.830, 0.506), (5.792, 0.494), (6.341, 1.0), (7.067, 1.0), (5.875, 1.0), (8.375, 1.0))
AC_GAMMAS = ((0.100, 0.012), (0.150, 0.036), (0.440, 0.026))


def ac225_alpha(r, energy, tissue):
    """Ac225KernelGenerator._calculate_alpha_contribution (ac225_kernel.py:140-166)."""
    rng = 0.0006 * energy ** 1.7 * AC_RANGE.get(tissue, 1.0)
    return alpha(r, rng, energy / 5.0)


def ac225_gamma(r, energy, intensity, tissue, reference_r0=True, voxel=1.0):
    """Ac225KernelGenerator._calculate_gamma_contribution (ac225_kernel.py:168-184)."""
    rho, z, _, _ = LU_TISSUE.get(tissue, LU_TISSUE["water"])
    mu = 0.096 * (0.5 / energy) ** 3.2 * (z / 7.42) ** 0.5
    return photon(r, mu * rho, intensity, reference_r0, voxel, False)


def ac225(tissue, voxel, grid, reference_r0=False):
    """ac225_kernel.py:67-97: parent and daughter alphas plus gamma lines.  The
    reference multiplies by a tissue scaling factor it never defines (the call
    raises AttributeError, ac225_kernel.py:95); tissue enters through the
    alpha range factor and the photon attenuation only."""
    r = radius(grid, voxel)
    k = np.zeros_like(r)
    for e, inten in AC_ALPHAS:
        k += inten * ac225_alpha(r, e, tissue)
    for e, inten in AC_GAMMAS:
        k += ac225_gamma(r, e, inten, tissue, reference_r0, voxel)
    return k


GENERATORS = {"Y90": y90, "Lu177": lu177, "Ga68": ga68, "F18": f18, "Tb161": tb161, "Ac225": ac225}

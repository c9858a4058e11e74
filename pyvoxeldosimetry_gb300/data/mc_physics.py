"""Physics tables for the in-repo Monte Carlo (host, numpy), passed to the GPU.

The reference's Monte Carlo (pyvoxeldosimetry/core/monte_carlo.py) never runs (its
constructor calls undefined table builders, :38-40) and its decay data stop at
0.1 MeV for photons (data/mc_decay/*.json "gamma_mass_attenuation").  The model
here is the builder's, stated in full:

* beta energies: inverse CDF of the nuclide's piecewise-linear spectrum
  (data/mc_decay/<nuclide>.json "spectrum_points"), on a uniform probability grid;
* electron transport: continuous slowing down along straight steps, CSDA range in
  water from the Katz-Penfold empirical relation R[g/cm^2] = 0.412 E^(1.265 - 0.0954 ln E)
  (E in MeV, 0.01-2.5 MeV), scaled by the local density; multiple scattering by the
  Highland formula with X0(water) = 36.08 g/cm^2; electrons below 10 keV stop;
* photons: total mass attenuation of water from the NIST XCOM table (values below),
  Compton part from the Klein-Nishina cross section times water's electron density
  (3.343e23 e/g), the remainder treated as absorption (photoelectric); Woodcock
  tracking through the density map; photons below 10 keV are absorbed.

Tables are uniform in energy so the device (and the oracle) interpolate with basic
arithmetic only.
"""
from __future__ import annotations

import numpy as np

from .nuclides import get_nuclide

ELECTRON_MASS_MEV = 0.51099895
X0_WATER = 36.08                 # g/cm^2
WATER_ELECTRONS_PER_G = 3.343e23
R_E_CM = 2.8179403262e-13        # classical electron radius
E_CUT = 0.01                     # MeV

# NIST XCOM, water, total attenuation with coherent scattering (cm^2/g)
XCOM_E = np.array([0.01, 0.015, 0.02, 0.03, 0.04, 0.05, 0.06, 0.08, 0.10, 0.15, 0.20, 0.30, 0.40, 0.50, 0.60,
                   0.80, 1.00, 1.25, 1.50, 2.00, 3.00])
XCOM_MU = np.array([5.329, 1.673, 0.8096, 0.3756, 0.2683, 0.2269, 0.2059, 0.1837, 0.1707, 0.1505, 0.1370,
                    0.1186, 0.1061, 0.09687, 0.08956, 0.07865, 0.07072, 0.06323, 0.05754, 0.04942, 0.03969])

N_TABLE = 2048


def katz_penfold_range(e_mev):
    """CSDA range (g/cm^2) of electrons of kinetic energy E (MeV) in water."""
    e = np.asarray(e_mev, dtype=np.float64)
    return 0.412 * np.power(e, 1.265 - 0.0954 * np.log(e))


def beta_inverse_cdf(symbol: str, n: int = 1025) -> np.ndarray:
    """Energies E(u) at u = i/(n-1) of the piecewise-linear beta spectrum (float32)."""
    nuc = get_nuclide(symbol)
    e = np.asarray(nuc.spectrum_e, dtype=np.float64)
    p = np.asarray(nuc.spectrum_p, dtype=np.float64)
    if e.size < 2:
        raise ValueError(f"{symbol} has no beta spectrum")
    seg = 0.5 * (p[1:] + p[:-1]) * np.diff(e)   # probability mass of each linear segment
    total = seg.sum()
    cdf = np.concatenate([[0.0], np.cumsum(seg)]) / total
    out = np.empty(n)
    for i, ui in enumerate(np.linspace(0.0, 1.0, n)):
        j = int(np.clip(np.searchsorted(cdf, ui, side="right") - 1, 0, len(seg) - 1))
        target = (ui - cdf[j]) * total          # mass to cover inside segment j
        p0, p1, e0, e1 = p[j], p[j + 1], e[j], e[j + 1]
        s = (p1 - p0) / (e1 - e0)               # pdf(x) = p0 + s x on [0, e1 - e0]
        if abs(s) < 1e-15:
            x = target / p0 if p0 > 0 else 0.0
        else:
            x = (-p0 + np.sqrt(max(p0 * p0 + 2 * s * target, 0.0))) / s
        out[i] = min(max(e0 + x, e0), e1)
    out[0], out[-1] = e[0], e[-1]
    return out.astype(np.float32)


def spectrum_mean(symbol: str) -> float:
    """Mean energy of the piecewise-linear spectrum (MeV)."""
    nuc = get_nuclide(symbol)
    e = np.asarray(nuc.spectrum_e, dtype=np.float64)
    p = np.asarray(nuc.spectrum_p, dtype=np.float64)
    x = np.linspace(e[0], e[-1], 200001)
    px = np.interp(x, e, p)
    return float(np.trapezoid(px * x, x) / np.trapezoid(px, x))


def electron_range_table(e_max: float, n: int = N_TABLE):
    """Uniform grid E_i = i * dE (i < n) up to e_max and the CSDA range R(E_i) (g/cm^2).
    R(0) = 0; below 10 keV the range is taken proportional to E^1.75 (continuous at 10 keV)."""
    e = np.linspace(0.0, e_max, n)
    r = np.zeros(n)
    hi = e >= E_CUT
    r[hi] = katz_penfold_range(e[hi])
    lo = (e > 0) & ~hi
    r[lo] = katz_penfold_range(E_CUT) * (e[lo] / E_CUT) ** 1.75
    return np.float32(e_max / (n - 1)), r.astype(np.float32)


def klein_nishina_sigma(e_mev):
    """Klein-Nishina total cross section per electron (cm^2)."""
    k = np.asarray(e_mev, dtype=np.float64) / ELECTRON_MASS_MEV
    a = (1 + k) / k ** 2 * (2 * (1 + k) / (1 + 2 * k) - np.log(1 + 2 * k) / k)
    b = np.log(1 + 2 * k) / (2 * k) - (1 + 3 * k) / (1 + 2 * k) ** 2
    return 2 * np.pi * R_E_CM ** 2 * (a + b)


def photon_tables(e_max: float, n: int = N_TABLE):
    """Uniform grid up to e_max: total mu/rho (cm^2/g) and the Compton fraction."""
    e = np.linspace(0.0, e_max, n)
    ee = np.maximum(e, XCOM_E[0])
    mu = np.exp(np.interp(np.log(ee), np.log(XCOM_E), np.log(XCOM_MU)))
    comp = klein_nishina_sigma(ee) * WATER_ELECTRONS_PER_G
    frac = np.clip(comp / mu, 0.0, 1.0)
    return np.float32(e_max / (n - 1)), mu.astype(np.float32), frac.astype(np.float32)


def emission_lines(symbol: str):
    """Gamma lines (energy MeV, photons per decay) of the nuclide."""
    return [(float(e), float(p)) for e, p in get_nuclide(symbol).gammas]

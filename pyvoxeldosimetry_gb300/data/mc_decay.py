"""Monte Carlo decay data: ``load_decay_data`` of the reference.

Mirrors ``load_decay_data`` (pyvoxeldosimetry/data/mc_decay/__init__.py:10-24),
which reads ``data/mc_decay/<nuclide>.json``: same name, same argument, same
ValueError for a nuclide without data, and a dict with the same keys and values
for the nuclides whose decays the GPU Monte Carlo transports (Y-90, Lu-177,
I-131).  The values are the reference's data files (half-life, beta spectrum
points, gamma lines, conversion electrons, the low-energy photon attenuation
table), restated as physical data; ``tests/test_decay_data_cpu.py`` checks them
value for value against the files as the reference loads them.

The Monte Carlo's own tables (``data.mc_physics``) and the kernel constants
(``data.nuclides``) are built from this data: beta spectrum points, gamma lines
and yields.  The MC does not transport conversion electrons, and takes photon
attenuation from NIST XCOM over the full energy range instead of the files'
0.01-0.1 MeV table.
"""
from __future__ import annotations

import copy
from typing import Any, Dict

_ATTEN_E = [0.01, 0.015, 0.02, 0.03, 0.04, 0.05, 0.06, 0.08, 0.1]

DECAY_DATA: Dict[str, Dict[str, Any]] = {
    "Y90": {
        "name": "Y90", "atomic_number": 39, "mass_number": 90,
        "half_life": 64.053, "half_life_unit": "hours",
        "decay_modes": [{
            "type": "beta-", "branching_ratio": 0.99983,
            "spectrum": {
                "mean_energy": 0.934, "max_energy": 2.280,
                "spectrum_points": {
                    "energy": [0.0, 0.2, 0.4, 0.6, 0.8, 1.0, 1.2, 1.4, 1.6, 1.8, 2.0, 2.2, 2.280],
                    "probability": [0.0, 0.12, 0.22, 0.30, 0.36, 0.40, 0.42, 0.38, 0.32, 0.24, 0.15, 0.06, 0.0],
                },
            },
        }],
        "physics_parameters": {
            "beta_csda_range": 11.3,
            "gamma_mass_attenuation": {
                "energies": _ATTEN_E,
                "coefficients": [4.098, 1.285, 0.5548, 0.1568, 0.0692, 0.0408, 0.0306, 0.0244, 0.0235],
            },
        },
    },
    "Lu177": {
        "name": "Lu177", "atomic_number": 71, "mass_number": 177,
        "half_life": 6.647, "half_life_unit": "days",
        "decay_modes": [{
            "type": "beta-", "branching_ratio": 1.0,
            "spectrum": {
                "mean_energy": 0.149, "max_energy": 0.498,
                "spectrum_points": {
                    "energy": [0.0, 0.1, 0.2, 0.3, 0.4, 0.498],
                    "probability": [0.0, 0.35, 0.48, 0.42, 0.22, 0.0],
                },
            },
        }],
        "gamma_emissions": [{"energy": 0.208, "intensity": 0.1094}, {"energy": 0.113, "intensity": 0.0641}],
        "conversion_electrons": [{"energy": 0.1819, "intensity": 0.0047}],
        "physics_parameters": {
            "beta_csda_range": 1.7,
            "gamma_mass_attenuation": {
                "energies": _ATTEN_E,
                "coefficients": [4.312, 1.348, 0.5798, 0.1638, 0.0723, 0.0426, 0.0319, 0.0253, 0.0244],
            },
        },
    },
    "I131": {
        "name": "I131", "atomic_number": 53, "mass_number": 131,
        "half_life": 8.0207, "half_life_unit": "days",
        "decay_modes": [{
            "type": "beta-", "branching_ratio": 1.0,
            "spectrum": {
                "mean_energy": 0.182, "max_energy": 0.807,
                "spectrum_points": {
                    "energy": [0.0, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.807],
                    "probability": [0.0, 0.25, 0.42, 0.48, 0.42, 0.32, 0.20, 0.08, 0.0],
                },
            },
        }],
        "gamma_emissions": [{"energy": 0.364, "intensity": 0.812}, {"energy": 0.637, "intensity": 0.0717},
                            {"energy": 0.284, "intensity": 0.0606}],
        "conversion_electrons": [{"energy": 0.334, "intensity": 0.0402}],
        "physics_parameters": {
            "beta_csda_range": 3.2,
            "gamma_mass_attenuation": {
                "energies": _ATTEN_E,
                "coefficients": [4.235, 1.324, 0.5702, 0.1611, 0.0711, 0.0419, 0.0314, 0.0249, 0.0240],
            },
        },
    },
}

_HOURS_PER_UNIT = {"seconds": 1.0 / 3600.0, "minutes": 1.0 / 60.0, "hours": 1.0, "days": 24.0}


def load_decay_data(radionuclide: str) -> Dict[str, Any]:
    """Decay properties of ``radionuclide`` for the Monte Carlo (a fresh copy)."""
    if radionuclide not in DECAY_DATA:
        raise ValueError(f"Decay data not found for {radionuclide}")
    return copy.deepcopy(DECAY_DATA[radionuclide])


def half_life_hours(radionuclide: str) -> float:
    d = DECAY_DATA[radionuclide]
    return d["half_life"] * _HOURS_PER_UNIT[d["half_life_unit"]]


def beta_spectrum(radionuclide: str):
    """(energies, probability densities) of the first beta decay mode's spectrum points."""
    sp = DECAY_DATA[radionuclide]["decay_modes"][0]["spectrum"]["spectrum_points"]
    return tuple(sp["energy"]), tuple(sp["probability"])


def gamma_lines(radionuclide: str):
    """((energy MeV, photons per decay), ...)."""
    return tuple((g["energy"], g["intensity"]) for g in DECAY_DATA[radionuclide].get("gamma_emissions", []))

"""ORACLE — test infrastructure only, never the product path.

TissueComposition.calculate_composition with its artefact handling
(pyvoxeldosimetry/tissue/composition.py:48-93) restated in numpy/scipy, and the
package's HU -> density calibration (linear through anchor points, clamped, NaN -> 0).
Pinned against the reference's own output (tests/golden/make_golden.py, ``tissue_*``).
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import gaussian_filter

RANGES = (("air", -1000, -900), ("lung", -900, -500), ("soft_tissue", -100, 100), ("bone", 300, 3000),
          ("water", -10, 10))


def handle_artifacts(ct):
    """composition.py:72-93: metal (> 2000 HU) replaced by the sigma-1 Gaussian smoothing of
    the image with metal (and NaN) set to 0."""
    ct = np.asarray(ct)
    metal = ct > 2000
    corrected = ct.copy()
    corrected[metal] = np.nan
    smoothed = gaussian_filter(np.nan_to_num(corrected), sigma=1)
    corrected[metal] = smoothed[metal]
    return corrected


def composition(ct, artifacts=True):
    """composition.py:48-70: closed HU ranges -> float masks."""
    img = handle_artifacts(ct) if artifacts else np.asarray(ct)
    return {name: ((img >= lo) & (img <= hi)).astype(float) for name, lo, hi in RANGES}


def density(ct, anchors, artifacts=True):
    img = handle_artifacts(ct) if artifacts else np.asarray(ct, dtype=np.float64)
    hu = np.array([a[0] for a in anchors], dtype=np.float64)
    rho = np.array([a[1] for a in anchors], dtype=np.float64)
    out = np.interp(np.asarray(img, dtype=np.float64), hu, rho)
    return np.where(np.isnan(img), 0.0, out)

"""ORACLE — test infrastructure only, never the product path.

Dose-volume histogram as the reference computes it, and numpy's uniform-bin
arithmetic restated step by step (the GPU histogram follows the latter, so a CPU
test can check that restatement against ``np.histogram`` itself).
"""
from __future__ import annotations

import numpy as np


def calculate_dvh(dose_map: np.ndarray, roi_mask: np.ndarray, bins: int = 1000):
    """pyvoxeldosimetry/core/utils.py:233-262: histogram of the ROI doses, then
    1 - cumsum / n; returns (upper bin edges, cumulative volume fraction)."""
    if dose_map.shape != roi_mask.shape:
        raise ValueError("Dose map and ROI mask must have same dimensions")
    roi_doses = dose_map[roi_mask > 0]
    if len(roi_doses) == 0:
        raise ValueError("ROI mask is empty")
    hist, edges = np.histogram(roi_doses, bins=bins)
    cum_dvh = 1.0 - np.cumsum(hist) / len(roi_doses)
    return edges[1:], cum_dvh


def numpy_uniform_bins(a: np.ndarray, bins: int):
    """numpy's histogram for an integer bin count and no range
    (numpy/lib/_histograms_impl.py: _get_outer_edges, then the uniform-bin
    branch of histogram), restated: outer edges from min/max (widened by 0.5 on
    each side when equal), linspace edges in the data's type, index
    ((x - first) / (last - first)) * bins truncated, last index folded into the
    last bin, one correction down (x < edge[i]) and one up (x >= edge[i + 1],
    not in the last bin).  Returns (counts, edges)."""
    a = np.asarray(a).ravel()
    t = a.dtype.type
    first, last = a.min(), a.max()
    if not (np.isfinite(first) and np.isfinite(last)):
        raise ValueError(f"autodetected range of [{first}, {last}] is not finite")
    if first == last:
        first, last = first - 0.5, last + 0.5
    edges = np.linspace(first, last, bins + 1, endpoint=True, dtype=t)
    denom = t(last - first)
    f = ((a - t(first)) / denom) * t(bins)
    assert f.dtype == a.dtype
    idx = f.astype(np.intp)
    idx[idx == bins] -= 1
    idx[a < edges[idx]] -= 1
    up = (a >= edges[idx + 1]) & (idx != bins - 1)
    idx[up] += 1
    return np.bincount(idx, minlength=bins).astype(np.intp), edges


def numpy_linspace_edges(first, last, bins):
    """np.linspace(first, last, bins + 1) for scalar endpoints of one floating type,
    restated (numpy/_core/function_base.py `linspace`): step = (last - first) / bins,
    edge i = i * step + first (each operation rounded in the type), the last edge =
    last; when the step underflows to 0, (i / bins) * (last - first) + first.  The GPU
    computes the histogram edges this way."""
    t = type(first)
    delta = t(last - first)
    step = t(delta / t(bins))
    i = np.arange(bins + 1).astype(t)
    if step == 0:
        y = (i / t(bins)).astype(t) * delta
    else:
        y = (i * step).astype(t)
    y = (y + first).astype(t)
    y[-1] = last
    return y

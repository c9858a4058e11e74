"""ORACLE — test infrastructure only, never the product path.

Spacing resampling with scipy.ndimage (the spline library nibabel's order-3
conform, which the reference's resample_dose_map calls, delegates to), on the
GPU path's geometry: both grids share the volume's outer corner, output voxel j
is sampled at input coordinate (j + 0.5) * out / in - 0.5; cubic B-spline
(order 3) or trilinear (order 1), mirror boundaries, FP64.
"""
from __future__ import annotations

import numpy as np


def resampled_shape(shape, input_spacing, output_spacing):
    return tuple(int(np.ceil(n * float(a) / float(b) - 1e-9)) for n, a, b in zip(shape, input_spacing, output_spacing))


def resample(volume, input_spacing, output_spacing, order=3, conserve_total=False, output_shape=None):
    from scipy import ndimage
    v = np.asarray(volume, dtype=np.float64)
    m = output_shape or resampled_shape(v.shape, input_spacing, output_spacing)
    axes = [(np.arange(mi) + 0.5) * (float(b) / float(a)) - 0.5
            for mi, a, b in zip(m, input_spacing, output_spacing)]
    coords = np.meshgrid(*axes, indexing="ij")
    out = ndimage.map_coordinates(v, coords, order=order, mode="mirror", prefilter=(order > 1))
    if conserve_total:
        out *= np.prod([float(b) for b in output_spacing]) / np.prod([float(a) for a in input_spacing])
    return out

"""ORACLE — test infrastructure only, never the product path.

FP64 numpy restatement of the reference's dose-convolution and time-integration
operators (devhliu/PyVoxelDosimetry).  Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg may import this module; the CUDA library is
checked against it.

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function here
against vectors produced by importing the reference itself
(``tests/golden/make_golden.py`` → ``tests/golden/reference_golden.npz``).
"""
from __future__ import annotations

import numpy as np

JOULE_PER_MEV = 1.602176634e-13


def reference_circular_conv(activity: np.ndarray, kernel: np.ndarray) -> np.ndarray:
    """The reference operator, verbatim semantics.

    pyvoxeldosimetry/core/kernel_convolution.py:71-74:
    ``np.fft.ifftn(np.fft.fftn(A) * np.fft.fftn(K, A.shape)).real`` — circular,
    unpadded, kernel zero-padded or truncated to A.shape at the high end.
    """
    a = np.asarray(activity)
    return np.fft.ifftn(np.fft.fftn(a) * np.fft.fftn(kernel, a.shape)).real


def linear_conv_same(activity: np.ndarray, kernel: np.ndarray, pad=None) -> np.ndarray:
    """Zero-padded linear convolution cropped to the input grid ("same").

    The reference operator (kernel_convolution.py:71-74) applied to arrays
    zero-padded to P >= N + K - 1 per axis, then cropped at offset K//2, which
    removes both the circular wrap-around and the K//2 shift of the reference.
    """
    a = np.asarray(activity, dtype=np.float64)
    k = np.asarray(kernel, dtype=np.float64)
    if pad is None:
        pad = tuple(n + kk - 1 for n, kk in zip(a.shape, k.shape))
    full = np.fft.ifftn(np.fft.fftn(a, pad) * np.fft.fftn(k, pad)).real
    c = [kk // 2 for kk in k.shape]
    return full[c[0]:c[0] + a.shape[0], c[1]:c[1] + a.shape[1], c[2]:c[2] + a.shape[2]]


def density_scale(dose_water: np.ndarray, density) -> np.ndarray:
    """Dose to local mass: D = D_water / rho, and 0 where rho <= 0 or NaN.

    The reference accepts ``tissue_densities`` and ignores it
    (pyvoxeldosimetry/core/dose_calculator.py:90); this is the builder-defined
    density-scaled convolution: energy per voxel from the water kernel,
    divided by the voxel's own mass.
    """
    if density is None:
        return dose_water
    rho = np.asarray(density, dtype=np.float64)
    out = np.zeros_like(dose_water, dtype=np.float64)
    ok = rho > 0
    out[ok] = dose_water[ok] / rho[ok]
    return out


def trapezoid_activity(activity_maps, time_points) -> np.ndarray:
    """ActivitySampler._trapezoid_integration (core/activity_sampler.py:69-78).

    sum_i (A_i + A_{i+1}) / 2 * (t_{i+1} - t_i), time in the caller's unit.
    """
    result = np.zeros_like(np.asarray(activity_maps[0], dtype=np.float64))
    for i in range(len(time_points) - 1):
        dt = time_points[i + 1] - time_points[i]
        result += (np.asarray(activity_maps[i], np.float64) + np.asarray(activity_maps[i + 1], np.float64)) / 2 * dt
    return result


def trapezoid_weights(time_points, seconds_per_unit: float = 1.0) -> np.ndarray:
    """Per-map weights w_t with sum_t w_t A_t == the trapezoid of the maps."""
    t = np.asarray(time_points, dtype=np.float64)
    w = np.zeros(len(t))
    for i in range(len(t) - 1):
        dt = (t[i + 1] - t[i]) * seconds_per_unit
        w[i] += dt / 2
        w[i + 1] += dt / 2
    return w


def absorbed_dose_from_rates(dose_rates, time_points) -> np.ndarray:
    """KernelConvolutionCalculator.calculate_absorbed_dose's trapezoid
    (core/kernel_convolution.py:99-104): time in hours, dt converted to s."""
    dose = np.zeros_like(np.asarray(dose_rates[0], dtype=np.float64))
    for i in range(len(time_points) - 1):
        dt = (time_points[i + 1] - time_points[i]) * 3600
        dose += (np.asarray(dose_rates[i], np.float64) + np.asarray(dose_rates[i + 1], np.float64)) / 2 * dt
    return dose

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


def linear_conv_same_multi(activity: np.ndarray, kernels, density=None, workers=None) -> list:
    """``density_scale(linear_conv_same(activity, k), density)`` for several kernels,
    in float64 with one shared forward transform of the activity (scipy.fft's real
    transforms on all host threads).  The same operator as ``linear_conv_same``, at
    the minimal padding P = N + K_max - 1 (every P >= N + K - 1 gives the same
    linear convolution), for volumes where the complex numpy path is too slow."""
    import os

    import scipy.fft as sf
    a = np.asarray(activity, dtype=np.float64)
    ks = [np.asarray(k, dtype=np.float64) for k in kernels]
    kmax = [max(k.shape[i] for k in ks) for i in range(3)]
    pad = tuple(n + kk - 1 for n, kk in zip(a.shape, kmax))
    w = workers or os.cpu_count() or 1
    fa = sf.rfftn(a, pad, workers=w)
    out = []
    for k in ks:
        full = sf.irfftn(fa * sf.rfftn(k, pad, workers=w), pad, workers=w)
        c = [kk // 2 for kk in k.shape]
        d = np.ascontiguousarray(full[c[0]:c[0] + a.shape[0], c[1]:c[1] + a.shape[1], c[2]:c[2] + a.shape[2]])
        del full
        out.append(density_scale(d, density))
    return out


def error_stats(dose, ref, density=None, tissue_rho: float = 0.2) -> dict:
    """Errors of a dose map against its FP64 oracle: normwise maximum
    max|D - D_ref| / max|D_ref| (the parity tolerance's measure), normwise mean
    mean|D - D_ref| / max|D_ref|, and the largest pointwise relative error over
    voxels above 10 % of max|D_ref|.

    With ``density`` (the map a density-scaled dose was divided by) also: the same
    normwise maximum of the energy per unit volume D * rho (the convolution's own
    output, whose FP32 rounding error 1/rho then amplifies: about 830x in air of
    0.0012 g/cc), and the normwise maximum over tissue voxels (rho >= tissue_rho)
    scaled by the largest tissue dose."""
    d = np.asarray(dose, dtype=np.float64)
    r = np.asarray(ref, dtype=np.float64)
    scale = float(np.abs(r).max())
    if scale == 0.0:
        out = {"max_normwise": float(np.abs(d).max()), "mean_normwise": float(np.abs(d).mean()),
               "max_rel_above_10pct": 0.0}
    else:
        diff = np.abs(d - r)
        hot = np.abs(r) > 0.1 * scale
        out = {"max_normwise": float(diff.max() / scale), "mean_normwise": float(diff.mean() / scale),
               "max_rel_above_10pct": float((diff[hot] / np.abs(r[hot])).max()) if hot.any() else 0.0}
    if density is not None:
        rho = np.nan_to_num(np.asarray(density, dtype=np.float64), nan=0.0)
        ok = rho > 0
        e_ref = np.abs(r * rho)[ok]
        e_diff = np.abs((d - r) * rho)[ok]
        out["energy_max_normwise"] = float(e_diff.max() / e_ref.max()) if ok.any() and e_ref.max() > 0 else 0.0
        t = rho >= tissue_rho
        t_scale = float(np.abs(r[t]).max()) if t.any() else 0.0
        out["tissue_max_normwise"] = float(np.abs(d - r)[t].max() / t_scale) if t_scale > 0 else 0.0
    return out


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

"""Seeded synthetic phantoms for the dose workloads (no patient data).

* ``sphere_phantom``: uniform sphere in water with a 1 % background and
  Poisson noise (the reference's single-timepoint Y-90 example shape,
  examples/single_timepoint_y90_physical_decay.py:8-23, scaled to 128^3 at
  2 mm and 1 GBq).
* ``ct_phantom``: CT-like density (body, lungs, spine, ribs, air) with an
  activity map of liver/body uptake plus 3-8 spherical lesions.
* ``biexp_timeseries``: activity at several timepoints from a per-voxel
  bi-exponential washout.

All arrays are float32, C order (axis 2 contiguous).
"""
from __future__ import annotations

import numpy as np


def _grid_mm(shape, voxel_mm):
    """Coordinates (mm) of voxel centres relative to the volume centre, broadcastable."""
    axes = []
    for i, (n, d) in enumerate(zip(shape, voxel_mm)):
        v = (np.arange(n, dtype=np.float32) - (n - 1) / 2.0) * np.float32(d)
        s = [1, 1, 1]
        s[i] = n
        axes.append(v.reshape(s))
    return axes


def sphere_phantom(shape=(128, 128, 128), voxel_mm=2.0, radius_mm=20.0, total_bq=1e9, background=0.01,
                   counts_per_voxel=1000.0, seed=1) -> np.ndarray:
    """Uniform sphere holding ``total_bq`` on a background of ``background`` x the
    sphere concentration, with Poisson noise of ``counts_per_voxel`` expected counts
    at sphere concentration.  Centre at voxel shape//2."""
    c = [n // 2 for n in shape]
    idx = np.indices(shape, dtype=np.float32)
    r2 = sum(((idx[i] - c[i]) * voxel_mm) ** 2 for i in range(3))
    inside = r2 <= radius_mm ** 2 + 1e-6
    c_sphere = total_bq / inside.sum()
    act = np.where(inside, c_sphere, background * c_sphere).astype(np.float64)
    rng = np.random.default_rng(seed)
    counts = rng.poisson(counts_per_voxel * act / c_sphere)
    return (counts * c_sphere / counts_per_voxel).astype(np.float32)


def ct_phantom(shape=(256, 256, 256), voxel_mm=1.5, seed=2, liver_bq_per_ml=1e4):
    """CT-like phantom: returns (activity Bq/voxel, density g/cc).

    Density: air 0.0012 outside an ellipsoidal body of 1.05, two lung
    ellipsoids of 0.3, a spine cylinder and rib shells of 1.85.  Activity:
    liver ellipsoid (uptake 1), rest of body 0.05, plus 3-8 spherical lesions of
    radius U[5,30] mm at U[5,50] x liver uptake, placed inside the body.
    """
    rng = np.random.default_rng(seed)
    vox = (voxel_mm,) * 3 if np.isscalar(voxel_mm) else tuple(voxel_mm)
    z, y, x = _grid_mm(shape, vox)
    ext = [n * d / 2 for n, d in zip(shape, vox)]
    # body ellipsoid semi-axes, clipped to the field of view
    bz, by, bx = min(185.0, 0.95 * ext[0]), min(115.0, 0.9 * ext[1]), min(170.0, 0.95 * ext[2])
    body = (z / bz) ** 2 + (y / by) ** 2 + (x / bx) ** 2 <= 1.0
    rho = np.full(shape, 0.0012, dtype=np.float32)
    rho[body] = 1.05
    lz, ly, lx = 0.35 * bz, 0.55 * by, 0.28 * bx
    for sx in (-1, 1):
        lung = ((z - 0.35 * bz) / lz) ** 2 + (y / ly) ** 2 + ((x - sx * 0.45 * bx) / lx) ** 2 <= 1.0
        rho[lung & body] = 0.3
    spine = ((y + 0.6 * by) ** 2 + x ** 2 <= (0.12 * by) ** 2) & (np.abs(z) <= 0.9 * bz) & body
    rho[spine] = 1.85
    rib_r2 = (y / (0.92 * by)) ** 2 + (x / (0.92 * bx)) ** 2
    ribs = (np.abs(rib_r2 - 1.0) < 0.04) & (np.mod(z + 1000.0, 25.0) < 8.0) & (z > 0) & body
    rho[ribs] = 1.85
    liver = ((z + 0.05 * bz) / (0.3 * bz)) ** 2 + ((y - 0.1 * by) / (0.5 * by)) ** 2 + \
        ((x + 0.4 * bx) / (0.35 * bx)) ** 2 <= 1.0
    liver &= body
    voxel_ml = np.prod(vox) / 1000.0
    conc = np.zeros(shape, dtype=np.float32)
    conc[body] = 0.05
    conc[liver] = 1.0
    n_les = int(rng.integers(3, 9))
    for _ in range(n_les):
        r = rng.uniform(5.0, 30.0)
        uptake = rng.uniform(5.0, 50.0)
        for _try in range(100):
            cz, cy, cx = (rng.uniform(-0.7, 0.7) * bz, rng.uniform(-0.6, 0.6) * by, rng.uniform(-0.7, 0.7) * bx)
            if (cz / bz) ** 2 + (cy / by) ** 2 + (cx / bx) ** 2 <= 0.5:
                break
        les = (z - cz) ** 2 + (y - cy) ** 2 + (x - cx) ** 2 <= r * r
        conc[les & body] = uptake
    act = (conc * np.float32(liver_bq_per_ml * voxel_ml)).astype(np.float32)
    return np.ascontiguousarray(act), np.ascontiguousarray(rho)


def biexp_timeseries(a0: np.ndarray, times_h, seed=3, t_range=(6.0, 160.0)):
    """Activity maps A(t) = A0 [w e^{-l1 t} + (1-w) e^{-l2 t}] with per-voxel half-lives
    log-uniform in ``t_range`` hours and w ~ U(0.2, 0.8).  Returns (T, *shape) float32
    and the per-voxel (w, T1, T2)."""
    rng = np.random.default_rng(seed)
    shape = a0.shape
    lo, hi = np.log(t_range[0]), np.log(t_range[1])
    t1 = np.exp(rng.uniform(lo, hi, shape)).astype(np.float32)
    t2 = np.exp(rng.uniform(lo, hi, shape)).astype(np.float32)
    w = rng.uniform(0.2, 0.8, shape).astype(np.float32)
    out = np.empty((len(times_h), *shape), dtype=np.float32)
    for i, t in enumerate(times_h):
        out[i] = a0 * (w * np.exp(-np.log(2) * t / t1) + (1 - w) * np.exp(-np.log(2) * t / t2))
    return out, (w, t1, t2)

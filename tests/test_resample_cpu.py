"""The GPU resampler's algorithm, restated in numpy (the cubic B-spline
prefilter as the 33-tap symmetric filter sqrt(3) z^|k| on the mirror-extended
line, 4-tap evaluation at mirrored indices), equals
scipy.ndimage.map_coordinates(order=3, mode='mirror') — the oracle the GPU
tests compare against."""
import numpy as np
import pytest

Z = np.sqrt(3.0) - 2.0


def prefilter(x, half=16):
    n = len(x)
    x = np.asarray(x, dtype=np.float64)
    return np.array([np.sqrt(3.0) * sum(Z ** abs(k) * x[mirror(i - k, n)] for k in range(-half, half + 1))
                     for i in range(n)])


def mirror(k, n):
    if n == 1:
        return 0
    period = 2 * n - 2
    k = abs(k) % period
    return period - k if k >= n else k


def evaluate(c, u):
    fl = np.floor(u)
    t, b, s = u - fl, int(fl), 1 - (u - fl)
    w = [s ** 3 / 6, (4 - 6 * t * t + 3 * t ** 3) / 6, (1 + 3 * t + 3 * t * t - 3 * t ** 3) / 6, t ** 3 / 6]
    return sum(w[k] * c[mirror(b - 1 + k, len(c))] for k in range(4))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 7, 40])
def test_restated_bspline_equals_scipy(n):
    from scipy import ndimage
    x = np.random.default_rng(n).random(n)
    c = prefilter(x)
    us = np.concatenate([np.linspace(-0.49, n - 0.51, 61), np.arange(n, dtype=float)])
    mine = np.array([evaluate(c, u) for u in us])
    ref = ndimage.map_coordinates(x, [us], order=3, mode="mirror")
    np.testing.assert_allclose(mine, ref, rtol=0, atol=1e-9 * np.abs(ref).max())


def test_oracle_geometry():
    from oracle import resample as ors
    v = np.random.default_rng(1).random((6, 7, 8))
    np.testing.assert_allclose(ors.resample(v, (2, 2, 2), (2, 2, 2)), v, atol=1e-12)
    assert ors.resampled_shape((10, 3, 7), (1.5, 0.1, 2.0), (1.5, 0.1, 3.0)) == (10, 3, 5)

"""Learned-correction network: CPU checks (no GPU needed).

* the oracle's hand-written backward equals torch autograd (float64, no rounding);
* the product's layer table equals the oracle's;
* the U-Net entry points reject bad geometry, channel counts and pointers
  before any CUDA call.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import unet as ou
from pyvoxeldosimetry_gb300 import _native as N
from pyvoxeldosimetry_gb300.core import learned_correction as lc


def _random_problem(dims=(16, 16, 16), seed=0):
    rng = np.random.default_rng(seed)
    flat = np.zeros(ou.n_params())
    o = 0
    for _, ci, co in ou.LAYERS:
        flat[o:o + co * ci * 27] = rng.normal(0, np.sqrt(2.0 / (27 * ci)), co * ci * 27)
        o += co * ci * 27
        flat[o:o + co] = rng.normal(0, 0.05, co)
        o += co
    flat[o:o + 34] = rng.normal(0, 0.3, 34)
    vols = [rng.random(dims).astype(np.float32) for _ in range(3)]
    x0 = ou.input_features(vols, [1.0, 1.0, 1.0], [1, 0, 1])
    target = torch.as_tensor(rng.normal(0, 0.3, dims))
    weight = torch.as_tensor((rng.random(dims) > 0.3).astype(np.float64))
    return ou.unpack(flat), x0, target, weight


def test_oracle_backward_equals_autograd():
    params, x0, target, weight = _random_problem()
    acts = ou.forward(params, x0, bf16=False)
    g, lm, ls = ou.backward(params, acts, target, weight, bf16=False)
    ga = ou.autograd_grads(params, x0, target, weight)
    a, b = ou.flat_grads(g), ou.flat_grads(ga)
    assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b)
    assert lm > 0 and ls > 0


def test_layer_tables_agree():
    assert lc.LAYERS == ou.LAYERS
    assert lc.HEAD_SIZE == ou.HEAD_SIZE
    assert lc.SLOPE == ou.SLOPE and lc.EPS == ou.EPS
    # parameter layout: per layer W [co][ci][27] then b [co], head last
    n = sum(co * ci * 27 + co for _, ci, co in lc.LAYERS) + lc.HEAD_SIZE
    assert n == ou.n_params()


def test_geometry():
    g = lc.geometry((16, 12, 10))
    assert tuple(g.dims) == (16, 12, 10)
    assert g.padded == 18 * 14 * 12
    assert g.padded_tiles % 128 == 0 and g.padded_tiles >= g.padded > g.padded_tiles - 128
    assert g.margin % 8 == 0 and g.margin >= 14 * 12 + 12 + 1
    assert g.rows == 2 * g.margin + g.padded_tiles
    lib = N.load()
    bad = N.UnetGeom()
    assert lib.pvd_unet_geometry(0, 4, 4, C.byref(bad)) == 1


def test_conv_flop_count():
    # 2 * 27 * sum(ci * co / 8^level) per voxel + the head
    per = sum(2 * 27 * ci * co / 8 ** lc.LEVEL[n] for n, ci, co in lc.LAYERS) + 64
    assert lc.conv_flops((8, 8, 8)) == pytest.approx(per * 512)


def test_validation_before_any_cuda_call():
    lib = N.load()
    g = lc.geometry((8, 8, 8))
    fake = 1 << 20  # never dereferenced: every case fails validation first
    # channels not a multiple of 16
    assert lib.pvd_unet_conv3d(C.byref(g), fake, 24, fake, None, fake, 16, None, 0, 0.01, None) == 1
    # misaligned tensor
    assert lib.pvd_unet_conv3d(C.byref(g), fake + 8, 16, fake, None, fake, 16, None, 0, 0.01, None) == 1
    # unknown flag
    assert lib.pvd_unet_conv3d(C.byref(g), fake, 16, fake, None, fake, 16, None, 64, 0.01, None) == 1
    # geometry not from pvd_unet_geometry
    g2 = lc.geometry((8, 8, 8))
    g2.rows += 8
    assert lib.pvd_unet_conv3d(C.byref(g2), fake, 16, fake, None, fake, 16, None, 0, 0.01, None) == 1
    # workspace too small for the weight gradient
    sz = C.c_size_t()
    assert lib.pvd_unet_wgrad_workspace(C.byref(g), 16, 32, C.byref(sz)) == 0 and sz.value > 0
    assert lib.pvd_unet_conv3d_wgrad(C.byref(g), fake, 16, fake, 32, fake, 0, fake, sz.value - 1, None) == 1
    # pooling pairs must halve every dim
    g4 = lc.geometry((4, 4, 2))
    assert lib.pvd_unet_pool(C.byref(g), fake, C.byref(g4), fake, 16, None) == 1
    # Adam needs step >= 1
    assert lib.pvd_adam_step(fake, fake, fake, fake, 10, 1e-3, 0.9, 0.999, 1e-8, 0.0, 0, None) == 1
    assert "pvd_adam_step" in N.last_error()


def test_nn_corrected_calculator_needs_a_model():
    from pyvoxeldosimetry_gb300 import DoseCalculator, NNCorrectedDoseCalculator
    with pytest.raises(ValueError):
        DoseCalculator("Y90", method="nn_corrected")
    with pytest.raises(TypeError):
        NNCorrectedDoseCalculator(["Y90", "Lu177"], config={"model_path": "x.npz"})


def test_dose_errors_restricts_to_tissue_above_threshold():
    d = np.array([1.0, 2.0, 3.0, 10.0, 0.5])
    ref = np.array([1.0, 2.2, 3.0, 10.0, 0.5])
    rho = np.array([1.0, 1.0, 0.01, 1.0, 1.0])  # voxel 2 is air
    e = lc.dose_errors(d, ref, rel_threshold=0.1, density=rho)
    assert e["voxels"] == 2  # 2.2 and 10.0: strictly above 10 % of the tissue max 10; 3.0 is air
    assert e["max"] == pytest.approx(0.2 / 2.2)


def test_log_ratio_target():
    dc = np.array([10.0, 5.0, 0.5, 8.0, 4.0, 100.0, 0.9, 0.3])
    dm = np.array([12.0, 5.0, 0.6, 0.0, 4.0 * np.e ** 5, 1.0, 600.0, 59.0])
    rho = np.array([1.0, 0.3, 1.0, 1.0, 1.85, 0.0012, 0.3, 0.3])  # voxel 5 is air
    t, w, dmax = lc.log_ratio_target(dc, dm, rho, rel_threshold=0.1)
    assert dmax == 10.0  # the air voxel's 100 is not a tissue maximum
    # weighted: tissue with conv dose > 1.0 or MC dose > 60.0 (10 % of 600), both doses positive
    assert w.tolist() == [1.0, 1.0, 0.0, 0.0, 1.0, 0.0, 1.0, 0.0]
    assert t[0] == pytest.approx(np.log(1.2)) and t[1] == 0.0
    assert t[4] == pytest.approx(3.0)  # clipped
    assert t[6] == pytest.approx(3.0)  # selected on the MC dose alone (lung), clipped
    assert t.dtype == np.float32 and w.dtype == np.float32


def test_focused_crops_hold_a_weighted_voxel_and_stay_in_range():
    rng = np.random.default_rng(0)
    for _ in range(3000):
        vd = tuple(int(x) for x in rng.integers(20, 140, 3))
        crop = tuple(int(x) for x in rng.choice([32, 48, 64], 3))
        w = rng.random(vd) > 0.999
        hot = np.flatnonzero(w.ravel())
        o = lc.crop_origin(rng, vd, crop, hot)
        assert all(min(0, vd[k] - crop[k]) <= o[k] <= max(0, vd[k] - crop[k]) for k in range(3))
        if hot.size:
            sub = w[max(o[0], 0):o[0] + crop[0], max(o[1], 0):o[1] + crop[1], max(o[2], 0):o[2] + crop[2]]
            assert sub.any()
        # in a flipped frame the crop holds a flipped weighted voxel
        fl = tuple(k for k in range(3) if rng.random() < 0.5)
        o3 = lc.crop_origin(rng, vd, crop, hot, fl)
        if hot.size:
            wf = np.flip(w, fl) if fl else w
            sub = wf[max(o3[0], 0):o3[0] + crop[0], max(o3[1], 0):o3[1] + crop[1], max(o3[2], 0):o3[2] + crop[2]]
            assert sub.any()
        o2 = lc.crop_origin(rng, vd, crop)          # unfocused: the same range
        assert all(min(0, vd[k] - crop[k]) <= o2[k] <= max(0, vd[k] - crop[k]) for k in range(3))


def test_every_bulk_copy_stays_inside_the_plane():
    """Row ranges read by the tensor-core kernels' bulk copies, restated from their
    tiling, against the plane size pvd_unet_geometry gives (random grids)."""
    rng = np.random.default_rng(4)
    for _ in range(300):
        d, h, w = (int(v) for v in rng.integers(1, 90, 3))
        g = lc.geometry((d, h, w))
        hp, wp = h + 2, w + 2
        reach = hp * wp + wp + 1  # largest |tap offset|
        # k_conv3: tiles of 128 rows over padded_tiles; slab rows [p0 + off(dz,dy) - 1, +130)
        last_p0 = g.padded_tiles - 128
        assert g.margin - reach >= 0
        assert g.margin + last_p0 + (hp * wp + wp) - 1 + 130 <= g.rows
        # k_conv3s: tiles of 126 output rows over padded; slab rows [p0 + off(dz,dy) - 1, +128)
        n_tiles = -(-g.padded // 126)
        last_p0s = (n_tiles - 1) * 126
        assert g.margin + last_p0s + (hp * wp + wp) - 1 + 128 <= g.rows
        # k_wgrad: stages of 64 rows over padded_tiles, A rows shifted by any tap offset
        assert g.margin + (g.padded_tiles - 64) + reach + 64 <= g.rows
        # outputs: every written row p < padded_tiles lies inside the plane
        assert g.margin + g.padded_tiles <= g.rows


def test_symmetry_codes_are_the_48_grid_symmetries():
    """symmetry(code): 48 distinct (permutation, flips) pairs, codes 0..7 the flips alone,
    and numpy's transform of a volume undone by the inverse mapping the library uses."""
    seen = {lc.symmetry(c) for c in range(48)}
    assert len(seen) == 48
    assert all(lc.symmetry(c)[0] == (0, 1, 2) for c in range(8))
    rng = np.random.default_rng(2)
    v = rng.random((3, 4, 5))
    for c in range(48):
        perm, flips = lc.symmetry(c)
        u = np.transpose(v, perm)
        u = np.flip(u, flips) if flips else u
        assert u.shape == tuple(v.shape[a] for a in perm)
        # the library's map: U[u] = V[v] with v[perm[k]] = flip_k ? dim - 1 - u_k : u_k
        for _ in range(5):
            uu = [int(rng.integers(n)) for n in u.shape]
            vv = [0, 0, 0]
            for k in range(3):
                vv[perm[k]] = v.shape[perm[k]] - 1 - uu[k] if k in flips else uu[k]
            assert u[tuple(uu)] == v[tuple(vv)]
    with pytest.raises(ValueError):
        lc.symmetry(48)

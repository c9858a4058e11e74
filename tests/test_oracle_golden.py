"""The oracle against vectors recorded from the reference implementation itself
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import conv as oc
from oracle import time_fit as of


CONV_CASES = ["ragged_asym", "cube_radial", "oversize", "even_kernel", "thin",
              "prime_small", "prime_mixed", "prime_oversize", "prime_thin"]


@pytest.mark.parametrize("name", CONV_CASES)
def test_circular_conv_is_reference(golden, name):
    d = oc.reference_circular_conv(golden[f"conv_{name}_A"], golden[f"conv_{name}_K"])
    np.testing.assert_allclose(d, golden[f"conv_{name}_D"], rtol=0, atol=1e-12 * np.abs(d).max())


def test_trapezoid_is_reference(golden):
    out = oc.trapezoid_activity(list(golden["trap_maps"]), list(golden["trap_times"]))
    np.testing.assert_allclose(out, golden["trap_out"], rtol=1e-14)


def test_trapezoid_weights_reproduce_trapezoid(golden):
    w = oc.trapezoid_weights(golden["trap_times"])
    out = np.tensordot(w, golden["trap_maps"], axes=1)
    np.testing.assert_allclose(out, golden["trap_out"], rtol=1e-12)


def test_absorbed_dose_is_reference(golden):
    rates = [oc.reference_circular_conv(m, golden["absd_K"]) for m in golden["absd_maps"]]
    out = oc.absorbed_dose_from_rates(rates, list(golden["absd_times"]))
    np.testing.assert_allclose(out, golden["absd_out"], rtol=1e-12)


def test_linear_conv_equals_direct_sum():
    rng = np.random.default_rng(3)
    a = rng.random((6, 5, 7))
    k = rng.random((3, 5, 3))
    d = oc.linear_conv_same(a, k)
    c = [s // 2 for s in k.shape]
    ref = np.zeros_like(a)
    for i in np.ndindex(a.shape):
        s = 0.0
        for j in np.ndindex(k.shape):
            src = tuple(i[t] - j[t] + c[t] for t in range(3))
            if all(0 <= src[t] < a.shape[t] for t in range(3)):
                s += a[src] * k[j]
        ref[i] = s
    np.testing.assert_allclose(d, ref, rtol=1e-12, atol=1e-12)


def test_mono_fit_is_reference(golden):
    p, auc = of.fit_mono(golden["fit_times"], list(golden["fit_acts"]), 64.1)
    np.testing.assert_allclose(p, golden["fit_params"], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(np.isnan(auc), np.isnan(golden["fit_auc"]))
    np.testing.assert_allclose(auc, golden["fit_auc"], rtol=1e-12)
    p, auc = of.fit_mono(golden["fit_times"], list(golden["fit_acts"]), 64.1, weight_factors=list(golden["fit_w"]))
    np.testing.assert_allclose(p, golden["fit_params_w"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("model,name", [("nukfit", "f2"), ("lmfit", "mono-exponential")])
def test_advanced_fit_is_reference(golden, model, name):
    p, auc, ok = of.fit_advanced(golden["adv_times"], list(golden["adv_acts"]), 64.1, model=model, model_name=name)
    key = name.replace("-", "_")
    np.testing.assert_allclose(p, golden[f"adv_{key}_params"], rtol=1e-12)
    np.testing.assert_allclose(auc, golden[f"adv_{key}_auc"], rtol=1e-12)


DVH_CASES = ["f32_bool", "f32_ties", "f64_const", "f64_many_bins"]


@pytest.mark.parametrize("name", DVH_CASES)
def test_dvh_is_reference(golden, name):
    from oracle import dvh as od
    e, c = od.calculate_dvh(golden[f"dvh_{name}_dose"], golden[f"dvh_{name}_mask"], int(golden[f"dvh_{name}_bins"]))
    assert e.dtype == golden[f"dvh_{name}_edges"].dtype
    np.testing.assert_array_equal(e, golden[f"dvh_{name}_edges"])
    np.testing.assert_array_equal(c, golden[f"dvh_{name}_cum"])


def _adversarial(dtype, rng):
    """Values on, just below and just above bin edges, ties, a constant run, negatives."""
    base = rng.gamma(2.0, 3.0, 4000).astype(dtype)
    edges = np.linspace(base.min(), base.max(), 101, dtype=dtype)
    on = rng.choice(edges, 2000)
    below = np.nextafter(on, dtype(-np.inf))
    above = np.nextafter(on, dtype(np.inf))
    return np.concatenate([base, on, below, above, np.full(50, on[0]), -base[:300]]).astype(dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("bins", [1, 7, 100, 1000, 20000])
def test_restated_numpy_binning_equals_np_histogram(dtype, bins):
    """The GPU histogram follows this step-by-step restatement of numpy's uniform-bin
    arithmetic; it must give np.histogram's counts and edges exactly."""
    from oracle import dvh as od
    rng = np.random.default_rng(bins)
    for a in (_adversarial(dtype, rng), np.full(33, dtype(2.5)), rng.random(5000).astype(dtype) * 1e-30):
        h, e = np.histogram(a, bins=bins)
        h2, e2 = od.numpy_uniform_bins(a, bins)
        np.testing.assert_array_equal(e2, e)
        np.testing.assert_array_equal(h2, h)


@pytest.mark.parametrize("tissue", ["water", "bone"])
def test_y90_generator_is_reference(golden, tissue):
    from oracle import kernels as ok
    np.testing.assert_allclose(ok.y90(tissue, 2.0, (15, 15, 15), reference_r0=True), golden[f"y90k_{tissue}"],
                               rtol=1e-13, atol=0, equal_nan=True)


@pytest.mark.parametrize("tissue", ["water", "bone", "lung"])
def test_ga68_generator_is_reference(golden, tissue):
    from oracle import kernels as ok
    np.testing.assert_allclose(ok.ga68(tissue, 2.0, (9, 9, 9), reference_r0=True), golden[f"kgen_ga68_{tissue}"],
                               rtol=1e-13, atol=0, equal_nan=True)


@pytest.mark.parametrize("tissue", ["water", "bone"])
def test_lu177_generator_is_reference(golden, tissue):
    from oracle import kernels as ok
    np.testing.assert_allclose(ok.lu177(tissue, 1.5, (11, 11, 11), reference_r0=True),
                               golden[f"kgen_lu177_{tissue}"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("tissue", ["water", "bone", "lung"])
def test_ac225_terms_are_reference(golden, tissue):
    from oracle import kernels as ok
    ra, rg = golden["kgen_ac225_r_alpha"], golden["kgen_ac225_r_gamma"]
    al = np.stack([ok.ac225_alpha(ra, e, tissue) for e, _ in ok.AC_ALPHAS])
    ga = np.stack([ok.ac225_gamma(rg, e, i, tissue) for e, i in ok.AC_GAMMAS])
    np.testing.assert_allclose(al, golden[f"kgen_ac225_alpha_{tissue}"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(ga, golden[f"kgen_ac225_gamma_{tissue}"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_restated_linspace_edges_equal_numpy(dtype):
    """The GPU computes numpy's histogram edges with this restatement of linspace."""
    from oracle import dvh as od
    rng = np.random.default_rng(7)
    tiny = np.finfo(dtype).tiny
    cases = [(dtype(a), dtype(a + abs(b))) for a, b in rng.standard_normal((40, 2)) * 1e3]
    cases += [(dtype(0.0), dtype(tiny * 3)), (dtype(-tiny), dtype(tiny)), (dtype(1.0), dtype(1.0 + np.finfo(dtype).eps))]
    cases += [(dtype(x) - dtype(0.5), dtype(x) + dtype(0.5)) for x in (3.25, 1e7, -2.0)]
    for first, last in cases:
        for bins in (1, 3, 7, 1000, 20000):
            np.testing.assert_array_equal(od.numpy_linspace_edges(first, last, bins),
                                          np.linspace(first, last, bins + 1, endpoint=True, dtype=dtype))


def test_multi_kernel_oracle_equals_single_kernel_oracle():
    """The shared-forward-transform float64 oracle used at full size equals the
    complex-FFT restatement of the reference operator on small cases."""
    rng = np.random.default_rng(5)
    a = rng.random((13, 11, 17))
    rho = rng.uniform(0.0, 2.0, a.shape)
    ks = [rng.random((5, 5, 5)), rng.random((3, 7, 9)), rng.random((1, 1, 1))]
    outs = oc.linear_conv_same_multi(a, ks, density=rho, workers=2)
    for k, d in zip(ks, outs):
        ref = oc.density_scale(oc.linear_conv_same(a, k), rho)
        np.testing.assert_allclose(d, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    st = oc.error_stats(outs[0] * (1 + 1e-6), outs[0])
    assert 0.9e-6 < st["max_normwise"] < 1.1e-6 and st["mean_normwise"] <= st["max_normwise"]


def _image_copy_circular(a, k, pads):
    """The GPU plan's method for CIRCULAR axes of any length, restated in numpy: per axis a
    length P (P == n, or P >= 2n), the kernel (truncated to n) at the corner and, when
    P > n, a second copy at offset P - n; zero-padded input; keep the first n outputs."""
    kp = np.zeros(pads)
    kt = k[tuple(slice(0, min(kk, n)) for kk, n in zip(k.shape, a.shape))]
    offs = [(0,) if P == n else (0, P - n) for P, n in zip(pads, a.shape)]
    for o0 in offs[0]:
        for o1 in offs[1]:
            for o2 in offs[2]:
                kp[o0:o0 + kt.shape[0], o1:o1 + kt.shape[1], o2:o2 + kt.shape[2]] += kt
    full = np.fft.ifftn(np.fft.fftn(a, pads) * np.fft.fftn(kp)).real
    return full[:a.shape[0], :a.shape[1], :a.shape[2]]


@pytest.mark.parametrize("name", CONV_CASES)
def test_circular_by_image_copy_equals_reference(golden, name):
    """Any P >= 2n with the kernel's image copy reproduces the reference's period-n
    operator, also when only some axes are padded."""
    a, k = golden[f"conv_{name}_A"], golden[f"conv_{name}_K"]
    ref = golden[f"conv_{name}_D"]
    for pads in (tuple(2 * n for n in a.shape), tuple(2 * n + 3 for n in a.shape),
                 (a.shape[0], 2 * a.shape[1] + 1, a.shape[2])):
        d = _image_copy_circular(a, k, pads)
        np.testing.assert_allclose(d, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("name", ["odd", "thin"])
@pytest.mark.parametrize("art", [0, 1])
def test_tissue_composition_oracle_is_reference(golden, name, art):
    from oracle import tissue as ot
    ct = golden[f"tissue_{name}_ct"]
    comp = ot.composition(ct, artifacts=bool(art))
    for t, m in comp.items():
        np.testing.assert_array_equal(m, golden[f"tissue_{name}_{art}_{t}"])

"""Parity of the CUDA FFT convolution (through the C ABI) against the FP64 oracle
and against vectors recorded from the reference itself.

Tolerance (the benchmark spec): normwise relative error max|D - D_ref| / max|D_ref|
<= 1e-5 for FP32 dose against the FP64 oracle on the same inputs.
"""
import numpy as np
import pytest
import torch

from oracle import conv as oc

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel_err(d, ref):
    d = np.asarray(d, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref).max()
    return float(np.abs(d - ref).max() / scale) if scale > 0 else float(np.abs(d).max())


def run_plan(a, kernels, mode="linear", density=None, out_scale=1.0, normalize=False, scales=None, pad=None,
             tma=True):
    from pyvoxeldosimetry_gb300.conv import ConvPlan
    kmax = tuple(max(k.shape[i] for k in kernels) for i in range(3))
    with ConvPlan(a.shape, kmax=kmax, n_kernels=len(kernels), mode=mode, pad=pad, tma=tma) as p:
        for s, k in enumerate(kernels):
            p.set_kernel(s, k, scale=1.0 if scales is None else scales[s], normalize=normalize)
        at = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
        rt = None if density is None else torch.from_numpy(np.ascontiguousarray(density, np.float32)).cuda()
        out = p.execute(at, density=rt, out_scale=out_scale)
        torch.cuda.synchronize()
        p.status()
        return out.cpu().numpy().astype(np.float64)


def radial_kernel(k, lam=1.8, dx=2.0):
    c = k // 2
    idx = np.indices((k, k, k)) - c
    r = np.sqrt((idx ** 2).sum(0)) * dx
    r0 = dx * (3 / (4 * np.pi)) ** (1 / 3)
    r = np.where(r == 0, r0, r)
    return np.exp(-r / lam) / r ** 2


CONV_CASES = ["ragged_asym", "cube_radial", "oversize", "even_kernel", "thin",
              "prime_small", "prime_mixed", "prime_oversize", "prime_thin"]


@pytest.mark.parametrize("name", CONV_CASES)
def test_reference_circular_matches_reference_golden(golden, name):
    """Every shape, including dims with prime factors > 7 (11, 13, 17, 23, 29, 37, 43):
    those axes run at a padded length >= 2n with the kernel's image copy."""
    a = golden[f"conv_{name}_A"]
    k = golden[f"conv_{name}_K"]
    ref = golden[f"conv_{name}_D"]          # produced by the reference's own calculate_dose_rate
    d = run_plan(a, [k], mode="reference_circular")[0]
    assert rel_err(d, ref) <= TOL


def test_reference_circular_explicit_pads():
    """An explicit pad of n (7-smooth) or of any 7-smooth length >= 2n gives the same
    period-n result; lengths in between are rejected."""
    from pyvoxeldosimetry_gb300._native import PvdError
    rng = np.random.default_rng(41)
    a = rng.random((12, 10, 14))
    k = rng.random((5, 3, 7))
    ref = oc.reference_circular_conv(a, k)
    for pad in [(12, 10, 14), (24, 20, 28), (25, 27, 30), (12, 21, 14)]:
        assert rel_err(run_plan(a, [k], mode="reference_circular", pad=pad)[0], ref) <= TOL
    with pytest.raises(PvdError, match="at least 2n"):
        run_plan(a, [k], mode="reference_circular", pad=(16, 10, 14))


@pytest.mark.parametrize("shape,ks", [((17, 23, 29), (5, 5, 5)), ((32, 32, 32), (7, 7, 7)),
                                      ((9, 40, 33), (3, 5, 7)), ((1, 1, 64), (1, 1, 9)),
                                      ((48, 20, 70), (9, 9, 9)), ((5, 6, 7), (11, 11, 11))])
def test_linear_matches_oracle(shape, ks):
    rng = np.random.default_rng(sum(shape) + sum(ks))
    a = rng.random(shape) * 1e3
    k = rng.random(ks)
    d = run_plan(a, [k])[0]
    assert rel_err(d, oc.linear_conv_same(a, k)) <= TOL


def test_linear_symmetric_kernel_real_spectrum_and_density():
    rng = np.random.default_rng(7)
    shape = (40, 36, 44)
    a = rng.random(shape) * 1e6
    rho = rng.uniform(0.2, 2.0, shape)
    rho[0, 0, :5] = 0.0
    rho[1, 1, 1] = np.nan
    k = radial_kernel(9)
    d = run_plan(a, [k], density=rho, normalize=True, scales=[3.5e-3])[0]
    ref = oc.density_scale(oc.linear_conv_same(a, k / k.sum() * 3.5e-3), np.nan_to_num(rho, nan=0.0))
    assert rel_err(d, ref) <= TOL
    assert np.all(d[0, 0, :5] == 0) and d[1, 1, 1] == 0


def test_multi_kernel_shares_forward():
    rng = np.random.default_rng(11)
    shape = (30, 26, 34)
    a = rng.random(shape)
    ks = [radial_kernel(21, 1.8, 1.5), radial_kernel(9, 0.3, 1.5), rng.random((11, 11, 11))]
    d = run_plan(a, ks)
    for s, k in enumerate(ks):
        assert rel_err(d[s], oc.linear_conv_same(a, k)) <= TOL


def test_weighted_timepoints_equal_trapezoid(golden):
    from pyvoxeldosimetry_gb300.conv import ConvPlan
    maps = golden["absd_maps"]
    times = golden["absd_times"]
    k = golden["absd_K"]
    w = oc.trapezoid_weights(times, 3600.0)
    with ConvPlan(maps.shape[1:], kmax=k.shape, mode="reference_circular") as p:
        p.set_kernel(0, k)
        acts = [torch.from_numpy(m.astype(np.float32)).cuda() for m in maps]
        out = p.execute(acts, weights=list(w))[0].cpu().numpy()
    # kernel_convolution.py:78-106 computes one convolution per timepoint then the trapezoid;
    # by linearity this is one convolution of the trapezoid-weighted activity.
    assert rel_err(out, golden["absd_out"]) <= TOL


def test_config1_size_against_fp64_oracle():
    """128^3 at 2 mm, 15^3 Y-90 exp(-r/1.8)/r^2 kernel, normalised on the GPU in FP64."""
    from pyvoxeldosimetry_gb300.phantoms import sphere_phantom
    a = sphere_phantom()
    k = radial_kernel(15, 1.8, 2.0)
    d = run_plan(a, [k], normalize=True)[0]
    ref = oc.linear_conv_same(a.astype(np.float64), k / k.sum())
    err = rel_err(d, ref)
    print(f"cfg1 max rel err {err:.3e}, mean abs err {np.abs(d - ref).mean() / np.abs(ref).max():.3e}")
    assert err <= TOL


def test_errors_are_raised_not_faulted():
    from pyvoxeldosimetry_gb300._native import PvdError
    from pyvoxeldosimetry_gb300.conv import ConvPlan
    with pytest.raises(PvdError, match="UNSUPPORTED"):
        ConvPlan((1031, 8, 8), kmax=(3, 3, 3), mode="reference_circular")  # prime 1031: length >= 2062
    with ConvPlan((8, 8, 8), kmax=(3, 3, 3)) as p:
        with pytest.raises(PvdError, match="STATE"):
            p.execute(torch.zeros((8, 8, 8), device="cuda"))
        with pytest.raises(PvdError, match="kmax"):
            p.set_kernel(0, np.ones((5, 5, 5)))
        with pytest.raises(PvdError, match="NUMERIC"):
            p.set_kernel(0, np.full((3, 3, 3), np.nan))
        with pytest.raises(PvdError, match="NUMERIC"):
            p.set_kernel(0, np.zeros((3, 3, 3)), normalize=True)


def _fast_lengths():
    from pyvoxeldosimetry_gb300 import _native
    return _native.fast_lengths()


FAST_LENGTHS = [64, 72, 80, 96, 112, 128, 144, 160, 192, 224, 240, 252, 256, 270, 280, 288, 300, 320, 324, 336,
                360, 384, 400, 448, 480, 512, 560, 576, 640]


@pytest.mark.parametrize("tma", [True, False])
@pytest.mark.parametrize("L", FAST_LENGTHS)
def test_every_fast_length_on_every_axis(L, tma):
    """Force FFT length L on all three axes (small volume): exercises the register
    four-step x/y/z pass kernels of that length with a real-even (radial) kernel
    and a complex-spectrum (asymmetric) kernel in one plan."""
    assert L in _fast_lengths()
    rng = np.random.default_rng(L)
    shape = (min(L - 8, 37), min(L - 8, 20), min(L - 8, 45))
    a = rng.random(shape)
    ks = [radial_kernel(9, 1.8, 1.5), rng.random((5, 7, 3))]
    d = run_plan(a, ks, pad=(L, L, L), tma=tma)
    for s, k in enumerate(ks):
        assert rel_err(d[s], oc.linear_conv_same(a, k)) <= TOL


@pytest.mark.parametrize("tma", [True, False])
def test_fast_full_extent_and_many_slots(tma):
    """N = P - K + 1 on the 280 axis (no slack in the padding) and more kernel slots
    than one fast z launch takes (slot 0 transforms in place and must run last)."""
    rng = np.random.default_rng(21)
    shape = (260, 12, 24)
    a = rng.random(shape)
    ks = [radial_kernel(21, 1.8, 1.5)] + [rng.random((3, 3, 3)) for _ in range(5)] + [radial_kernel(11, 0.5, 1.5)]
    d = run_plan(a, ks, pad=(280, 64, 64), tma=tma)
    for s, k in enumerate(ks):
        assert rel_err(d[s], oc.linear_conv_same(a, k)) <= TOL


@pytest.mark.parametrize("tma", [True, False])
def test_tma_boxes_split_long_columns(tma):
    """Columns longer than one 256-row TMA box (N1 = 300, P1 = 320, N0 = 270) take
    several boxes per tile; both column-pass variants agree with the oracle."""
    rng = np.random.default_rng(31)
    shape = (270, 300, 20)
    a = rng.random(shape)
    ks = [radial_kernel(9, 1.0, 1.5), rng.random((3, 5, 3))]
    d = run_plan(a, ks, pad=(280, 320, 64), tma=tma)
    for s, k in enumerate(ks):
        assert rel_err(d[s], oc.linear_conv_same(a, k)) <= TOL


@pytest.fixture(scope="module")
def ct256():
    """The dose benchmark's own workload: seeded 256^3 CT-like phantom at 1.5 mm and the
    three nuclide kernels (Y-90 21^3, Lu-177 9^3, I-131 11^3); FP64 oracle doses to
    water (the reference's operator) and density-scaled."""
    from pyvoxeldosimetry_gb300 import phantoms
    from pyvoxeldosimetry_gb300.data import nuclides as nd
    act, rho = phantoms.ct_phantom((256, 256, 256), 1.5, seed=2)
    ks = {"Y90": 21, "Lu177": 9, "I131": 11}
    kernels = []
    for n, k in ks.items():
        kk = nd.analytic_profile(n, 1.5, (k,) * 3)
        kernels.append(kk / kk.sum() * nd.gy_per_bq_s_scale(n, 1.5))
    water = oc.linear_conv_same_multi(act, kernels)
    return act, rho, ks, water


@pytest.mark.parametrize("autotune", [True, False])
def test_bench_workload_ct256_three_nuclides_density(ct256, autotune):
    """256^3, Y-90/Lu-177/I-131 analytic kernels normalised on the GPU, through
    KernelConvolutionCalculator, with the autotuner's FFT lengths and with the default
    280^3.  Dose to water (the reference operator): within 1e-5 normwise of the FP64
    oracle.  Density-scaled dose: the energy per voxel D * rho within 1e-5 normwise, and
    the dose in tissue (rho >= 0.2) within 1e-5 of the largest tissue dose; in air
    (0.0012 g/cc) the division by rho amplifies the convolution's FP32 rounding error
    about 830-fold, so the all-voxel normwise figure is printed, not bounded."""
    from pyvoxeldosimetry_gb300.core.kernel_convolution import KernelConvolutionCalculator
    act, rho, ks, water = ct256
    calc = KernelConvolutionCalculator(list(ks), config={"kernel_size": ks, "autotune": autotune})
    a = torch.from_numpy(act).cuda()
    dw = calc.calculate_dose_rate(a, (1.5, 1.5, 1.5)).cpu().numpy()
    d = calc.calculate_dose_rate(a, (1.5, 1.5, 1.5), density=torch.from_numpy(rho).cuda()).cpu().numpy()
    if not autotune:
        assert calc._plan.fft_shape == (280, 280, 280)
    for s, ref in enumerate(water):
        stw = oc.error_stats(dw[s], ref)
        st = oc.error_stats(d[s], oc.density_scale(ref, rho), density=rho)
        print(f"{list(ks)[s]} fft {calc._plan.fft_shape}: water {stw}; density-scaled {st}")
        assert stw["max_normwise"] <= TOL
        assert st["energy_max_normwise"] <= TOL and st["tissue_max_normwise"] <= TOL
    calc.close()

"""The reference-facing API (DoseCalculator / KernelConvolutionCalculator /
ActivitySampler) on the GPU against the oracle and the reference's golden vectors."""
import math

import numpy as np
import pytest
import torch

from oracle import conv as oc

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel_err(d, ref):
    d = np.asarray(d, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.abs(d - ref).max() / np.abs(ref).max())


def analytic_S(nuc, vs, size):
    from pyvoxeldosimetry_gb300.data import nuclides as nd
    k = nd.analytic_profile(nuc, vs, (size,) * 3)
    return k / k.sum() * nd.gy_per_bq_s_scale(nuc, vs)


def test_reference_example_path_with_injected_kernel(golden):
    """examples/kernel_convolution_example.py reaches through calculator.calculator;
    with the reference's own kernel injected and mode='reference_circular' the result
    is the reference's calculate_dose_rate output."""
    from pyvoxeldosimetry_gb300 import DoseCalculator
    a, k, ref = golden["conv_cube_radial_A"], golden["conv_cube_radial_K"], golden["conv_cube_radial_D"]
    calc = DoseCalculator("Y90", method="kernel", config={"kernel_resolution": 1.0, "mode": "reference_circular",
                                                          "half_life": 64.1})
    calc.calculator.kernel = k
    d = calc.calculator.calculate_dose_rate(activity_map=a, voxel_size=(1.0, 1.0, 1.0))
    assert isinstance(d, np.ndarray) and d.shape == a.shape
    assert rel_err(d, ref) <= TOL


def test_single_timepoint_dose_rate_and_physical_decay_dose():
    from pyvoxeldosimetry_gb300 import DoseCalculator
    from pyvoxeldosimetry_gb300.phantoms import sphere_phantom
    a = sphere_phantom((64, 64, 64), 2.0, radius_mm=12.0)
    calc = DoseCalculator("Y90", method="kernel_convolution",
                          config={"single_timepoint_dose": "physical_decay", "kernel_size": 15})
    res = calc.calculate_dose(activity_maps=[a], time_points=[2.0], voxel_size=(2.0, 2.0, 2.0))
    ref = oc.linear_conv_same(a, analytic_S("Y90", 2.0, 15))
    assert res.metadata["mode"] == "single_timepoint"
    assert rel_err(res.dose_rate_maps[0], ref) <= TOL
    tau = 64.1 * 3600 / math.log(2)
    assert rel_err(res.absorbed_dose, ref * tau) <= TOL


def test_multi_timepoint_modes_agree_with_trapezoid():
    from pyvoxeldosimetry_gb300 import DoseCalculator
    rng = np.random.default_rng(5)
    maps = [rng.random((20, 24, 18)).astype(np.float32) * 1e4 for _ in range(4)]
    t = [1.0, 4.0, 24.0, 96.0]
    rho = rng.uniform(0.3, 1.8, maps[0].shape).astype(np.float32)
    calc = DoseCalculator("Lu177", method="kernel")
    S = analytic_S("Lu177", 1.0, 13)
    r_act = calc.calculate_dose(activity_maps=maps, time_points=t, voxel_size=(1.0,) * 3, tissue_densities=rho)
    ref_rates = [oc.density_scale(oc.linear_conv_same(m, S), rho) for m in maps]
    ref = oc.absorbed_dose_from_rates(ref_rates, t)
    assert r_act.metadata["mode"] == "multi_timepoint_activity"
    assert rel_err(r_act.absorbed_dose, ref) <= TOL
    r_dr = calc.calculate_dose(activity_maps=maps, time_points=t, voxel_size=(1.0,) * 3, tissue_densities=rho,
                               integration_mode="dose_rate")
    assert rel_err(r_dr.absorbed_dose, ref) <= TOL
    for d, rr in zip(r_dr.dose_rate_maps, ref_rates):
        assert rel_err(d, rr) <= TOL
    # accumulated activity (Bq h) path
    acc = oc.trapezoid_activity(maps, t)
    r_acc = calc.calculate_dose(accumulated_activity=acc.astype(np.float32), voxel_size=(1.0,) * 3,
                                tissue_densities=rho)
    assert rel_err(r_acc.absorbed_dose, ref) <= TOL


def test_activity_sampler_matches_reference(golden):
    from pyvoxeldosimetry_gb300 import ActivitySampler
    out = ActivitySampler(half_life=64.1).integrate_activity(list(golden["trap_maps"]), list(golden["trap_times"]))
    assert rel_err(out, golden["trap_out"]) <= 1e-6


def test_cuda_tensors_in_and_out_and_multi_nuclide():
    from pyvoxeldosimetry_gb300 import KernelConvolutionCalculator
    rng = np.random.default_rng(9)
    a = rng.random((32, 30, 28)).astype(np.float32)
    calc = KernelConvolutionCalculator(["Y90", "Lu177", "I131"], "water",
                                       config={"kernel_size": {"Y90": 21, "Lu177": 9, "I131": 11}})
    at = torch.from_numpy(a).cuda()
    d = calc.calculate_dose_rate(at, (1.5, 1.5, 1.5))
    assert isinstance(d, torch.Tensor) and d.is_cuda and d.shape == (3, *a.shape)
    for i, (n, s) in enumerate([("Y90", 21), ("Lu177", 9), ("I131", 11)]):
        assert rel_err(d[i].cpu().numpy(), oc.linear_conv_same(a, analytic_S(n, 1.5, s))) <= TOL


def test_api_errors_match_reference_conventions():
    from pyvoxeldosimetry_gb300 import DoseCalculator, KernelConvolutionCalculator
    with pytest.raises(ValueError):
        DoseCalculator("Y90", method="nope")
    with pytest.raises(NotImplementedError):
        DoseCalculator("Y90", method="gate_monte_carlo")
    with pytest.raises(TypeError):
        KernelConvolutionCalculator(90, "water")
    with pytest.raises(ValueError):
        DoseCalculator("Y90", config={"half_life": 0.0})
    calc = DoseCalculator("Y90")
    a = np.ones((8, 8, 8), np.float32)
    with pytest.raises(ValueError):
        calc.calculate_dose(activity_maps=[a], voxel_size=(1.0, 1.0))
    with pytest.raises(ValueError):
        calc.calculate_dose(activity_maps=[a, np.ones((8, 8, 9))], time_points=[0, 1])
    with pytest.raises(ValueError):
        calc.calculate_dose()
    # a kernel fixed at kernel_resolution (1 mm) and a 2 mm activity: the activity is
    # resampled to the kernel grid (the reference's _resample_activity is a stub) and the
    # dose comes back on the activity's grid
    calc.calculator.kernel = np.ones((3, 3, 3))
    d = calc.calculator.calculate_dose_rate(a, (2.0, 2.0, 2.0))
    assert d.shape == a.shape and np.isfinite(d).all()


def test_host_buffer_path_is_identical_to_device_path():
    """numpy / pinned-CPU-tensor inputs take the pipelined host path
    (pvd_conv_execute_host); it runs the same kernels, so the dose is bitwise equal
    to the device-resident path, for one and for several nuclides."""
    from pyvoxeldosimetry_gb300 import KernelConvolutionCalculator
    rng = np.random.default_rng(13)
    shape = (37, 30, 41)
    a = rng.random(shape).astype(np.float32) * 1e4
    rho = rng.uniform(0.2, 1.9, shape).astype(np.float32)
    for nucs in ("Y90", ["Y90", "Lu177", "I131"]):
        calc = KernelConvolutionCalculator(nucs, "water", config={"kernel_size": {"Y90": 21, "Lu177": 9, "I131": 11}})
        dev = calc.calculate_dose_rate(torch.from_numpy(a).cuda(), (1.5,) * 3, density=torch.from_numpy(rho).cuda())
        dev = dev.cpu().numpy()
        host_np = calc.calculate_dose_rate(a, (1.5,) * 3, density=rho)
        assert isinstance(host_np, np.ndarray) and host_np.shape == dev.shape
        np.testing.assert_array_equal(host_np, dev)
        at, rt = torch.from_numpy(a).pin_memory(), torch.from_numpy(rho).pin_memory()
        out = torch.empty(dev.shape, dtype=torch.float32).pin_memory()
        for _ in range(3):  # repeated calls reuse the plan's staging buffers and streams
            res = calc.calculate_dose_rate(at, (1.5,) * 3, density=rt, out=out)
            assert res is out
            np.testing.assert_array_equal(out.numpy(), dev)
        # without density
        np.testing.assert_array_equal(calc.calculate_dose_rate(a, (1.5,) * 3),
                                      calc.calculate_dose_rate(torch.from_numpy(a).cuda(), (1.5,) * 3).cpu().numpy())

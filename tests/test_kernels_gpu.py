"""GPU dose-point-kernel library (pvd_radial_kernel, KernelFactory) against the
reference's own generators (golden vectors) and the FP64 numpy oracle."""
import numpy as np
import pytest

from oracle import kernels as ok

pytestmark = pytest.mark.gpu

TISSUES = ["water", "lung", "soft_tissue", "bone", "iodine_contrast"]


@pytest.mark.parametrize("nuclide", ["Y90", "Lu177", "Ga68", "F18", "Tb161", "Ac225"])
@pytest.mark.parametrize("tissue", TISSUES)
@pytest.mark.parametrize("reference_r0", [False, True])
def test_gpu_kernel_equals_oracle(nuclide, tissue, reference_r0):
    from pyvoxeldosimetry_gb300.data.dose_kernels import generate_kernel
    vs, grid = (0.01, (9, 11, 13)) if nuclide == "Ac225" else (1.5, (17, 15, 13))
    got = generate_kernel(nuclide, tissue, vs, grid, reference_r0=reference_r0)
    ref = ok.GENERATORS[nuclide](tissue, vs, grid, reference_r0=reference_r0)
    assert got.dtype == np.float64 and got.shape == grid
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-300, equal_nan=True)


def test_gpu_kernels_equal_reference_golden(golden):
    from pyvoxeldosimetry_gb300.data.dose_kernels import generate_kernel
    for tissue in ["water", "bone"]:
        np.testing.assert_allclose(generate_kernel("Y90", tissue, 2.0, (15, 15, 15), reference_r0=True),
                                   golden[f"y90k_{tissue}"], rtol=1e-12, equal_nan=True)
        np.testing.assert_allclose(generate_kernel("Lu177", tissue, 1.5, (11, 11, 11), reference_r0=True),
                                   golden[f"kgen_lu177_{tissue}"], rtol=1e-12)
    for tissue in ["water", "bone", "lung"]:
        np.testing.assert_allclose(generate_kernel("Ga68", tissue, 2.0, (9, 9, 9), reference_r0=True),
                                   golden[f"kgen_ga68_{tissue}"], rtol=1e-12, equal_nan=True)


def test_factory_api_and_cache_key(tmp_path):
    from pyvoxeldosimetry_gb300 import KernelFactory
    f = KernelFactory(cache_dir=str(tmp_path))
    with pytest.raises(ValueError, match="Unsupported nuclide"):
        f.get_kernel("Xx99", "water")
    a = f.get_kernel("Lu177", "water", 1.0)
    assert a.shape == (81, 81, 81) and np.isfinite(a).all()        # the reference's default grid
    b = f.get_kernel("Lu177", "water", 2.0)
    assert not np.array_equal(a, b)                               # keyed by voxel size too
    c = f.get_kernel("Lu177", "bone", 1.0, (21, 21, 21))
    np.testing.assert_allclose(c, ok.lu177("bone", 1.0, (21, 21, 21)), rtol=1e-12)
    assert len(list(tmp_path.glob("*.npy"))) == 3
    f2 = KernelFactory(cache_dir=str(tmp_path))
    np.testing.assert_array_equal(f2.get_kernel("Lu177", "bone", 1.0, (21, 21, 21)), c)   # read from disk
    c[10, 10, 10] = -1.0
    assert f2.get_kernel("Lu177", "bone", 1.0, (21, 21, 21))[10, 10, 10] != -1.0      # copies handed out


@pytest.mark.parametrize("nuclide", ["Ga68", "F18", "Tb161", "Ac225"])
def test_reference_profile_convolution_for_every_library_nuclide(nuclide):
    """kernel_profile='reference' convolves with the library kernel at kernel_resolution."""
    from oracle import conv as oc
    from pyvoxeldosimetry_gb300 import KernelConvolutionCalculator
    rng = np.random.default_rng(4)
    act = (rng.random((20, 18, 22)) * 1e4).astype(np.float32)
    kr = 0.01 if nuclide == "Ac225" else 2.0
    calc = KernelConvolutionCalculator(nuclide, "soft_tissue", kernel_resolution=kr,
                                       config={"kernel_profile": "reference", "kernel_size": 7, "autotune": False})
    d = calc.calculate_dose_rate(act, (kr,) * 3)
    k = ok.GENERATORS[nuclide]("soft_tissue", kr, (7, 7, 7))
    ref = oc.linear_conv_same(act, k)
    assert np.abs(d - ref).max() <= 1e-5 * np.abs(ref).max()

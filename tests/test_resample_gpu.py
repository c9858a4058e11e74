"""GPU resampling (cubic B-spline / trilinear, mirror boundaries) against
scipy.ndimage on the same geometry, and the convolution calculator's use of it
for kernels defined at a fixed resolution."""
import numpy as np
import pytest
import torch

from oracle import conv as oc
from oracle import resample as ors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [1, 3])
@pytest.mark.parametrize("shape,sin,sout", [
    ((20, 24, 28), (2.0, 2.0, 2.0), (1.5, 1.5, 1.5)),       # upsampling
    ((33, 30, 27), (1.0, 1.2, 0.9), (2.5, 2.0, 3.1)),       # downsampling, anisotropic
    ((1, 2, 17), (1.0, 1.0, 1.0), (0.4, 0.6, 1.7)),         # axes of length 1 and 2
    ((16, 16, 16), (1.5, 1.5, 1.5), (1.5, 1.5, 1.5)),       # same spacing
])
def test_resample_matches_scipy(order, shape, sin, sout):
    from pyvoxeldosimetry_gb300.core.utils import resample_volume
    rng = np.random.default_rng(sum(shape) + order)
    v = rng.random(shape).astype(np.float32) * 100.0
    got = resample_volume(v, sin, sout, order=order)
    ref = ors.resample(v, sin, sout, order=order)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()


def test_same_spacing_reproduces_the_input_and_conservation():
    from pyvoxeldosimetry_gb300.core.utils import resample_volume
    rng = np.random.default_rng(3)
    v = rng.random((18, 20, 22)).astype(np.float32)
    same = resample_volume(torch.from_numpy(v).cuda(), (2.0,) * 3, (2.0,) * 3)
    assert isinstance(same, torch.Tensor) and same.is_cuda
    np.testing.assert_allclose(same.cpu().numpy(), v, rtol=0, atol=2e-6)
    # a smooth activity field: the total survives resampling to interpolation accuracy
    idx = np.indices((40, 40, 40)).astype(np.float64)
    act = np.exp(-((idx - 19.5) ** 2).sum(0) / (2 * 6.0 ** 2)).astype(np.float32) * 1e6
    fine = resample_volume(act, (2.0,) * 3, (1.5,) * 3, conserve_total=True)
    coarse = resample_volume(act, (2.0,) * 3, (3.0,) * 3, conserve_total=True)
    assert abs(fine.sum() / act.sum() - 1) < 2e-3 and abs(coarse.sum() / act.sum() - 1) < 2e-3


def test_resample_dose_map_affine():
    from pyvoxeldosimetry_gb300.core.utils import resample_dose_map
    d = np.ones((10, 12, 14), np.float32)
    r, aff = resample_dose_map(d, (2.0, 2.0, 2.0), (1.0, 4.0, 2.0))
    assert r.shape == (20, 6, 14)
    np.testing.assert_allclose(r, 1.0, atol=1e-6)
    np.testing.assert_allclose(np.diag(aff)[:3], [1.0, 4.0, 2.0])
    np.testing.assert_allclose(aff[:3, 3], [-0.5, 1.0, 0.0])


def test_fixed_resolution_kernel_resamples_activity_and_dose():
    """An explicit kernel at kernel_resolution 2 mm on a 1.5 mm activity grid: the
    pipeline equals resample -> linear convolution -> resample back on the oracle."""
    from pyvoxeldosimetry_gb300.core.kernel_convolution import KernelConvolutionCalculator
    rng = np.random.default_rng(11)
    act = (rng.random((30, 28, 26)) ** 3 * 1e5).astype(np.float32)
    idx = np.indices((9, 9, 9)) - 4.0
    r = np.sqrt((idx ** 2).sum(0))
    k = np.exp(-r / 1.8) / np.maximum(r, 0.62) ** 2
    vs, kr = (1.5, 1.5, 1.5), 2.0
    calc = KernelConvolutionCalculator("Y90", kernel_resolution=kr, config={"kernel": k, "autotune": False})
    d = calc.calculate_dose_rate(act, vs)
    assert d.shape == act.shape
    a2 = ors.resample(act, vs, (kr,) * 3, conserve_total=True)
    d2 = oc.linear_conv_same(a2, k)
    ref = ors.resample(d2, (kr,) * 3, vs, output_shape=act.shape)
    assert np.abs(d - ref).max() <= 1e-4 * np.abs(ref).max()
    calc2 = KernelConvolutionCalculator("Y90", kernel_resolution=kr,
                                        config={"kernel": k, "autotune": False, "resample_output": "kernel"})
    dk = calc2.calculate_dose_rate(act, vs)
    assert dk.shape == a2.shape
    assert np.abs(dk - d2).max() <= 1e-4 * np.abs(d2).max()


@pytest.mark.parametrize("order", [1, 3])
def test_direct_and_separable_entry_points_agree(order):
    """pvd_resample (3-D evaluation) and pvd_resample_separable (three one-axis passes)
    compute the same interpolant."""
    import ctypes as C
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    rng = np.random.default_rng(order)
    shape, m = (13, 17, 21), (19, 11, 30)
    v = torch.from_numpy(rng.random(shape).astype(np.float32)).cuda()
    step = [(shape[i] / m[i]) for i in range(3)]
    origin = [0.5 * s - 0.5 for s in step]
    sh = torch.cuda.current_stream().cuda_stream
    src = v
    if order == 3:
        src, scratch = torch.empty_like(v), torch.empty_like(v)
        N.check(lib.pvd_bspline_prefilter(v.data_ptr(), src.data_ptr(), scratch.data_ptr(), *shape, sh))
    a = torch.empty(m, device="cuda")
    b = torch.empty(m, device="cuda")
    st3, or3 = (C.c_double * 3)(*step), (C.c_double * 3)(*origin)
    N.check(lib.pvd_resample(src.data_ptr(), *shape, a.data_ptr(), *m, st3, or3, order, 2.0, sh))
    n_scr = shape[0] * shape[1] * m[2] + shape[0] * m[1] * m[2] + 8 * sum(m)
    scr = torch.empty(n_scr, device="cuda")
    N.check(lib.pvd_resample_separable(src.data_ptr(), *shape, b.data_ptr(), *m, st3, or3, order, 2.0,
                                       scr.data_ptr(), n_scr, sh))
    ref = 2.0 * ors.resample(v.cpu().numpy(), (1.0,) * 3, [1.0 * s for s in step], order=order, output_shape=m)
    for x in (a, b):
        assert np.abs(x.cpu().numpy() - ref).max() <= 2e-5 * np.abs(ref).max()
    with pytest.raises(N.PvdError):
        N.check(lib.pvd_resample_separable(src.data_ptr(), *shape, b.data_ptr(), *m, st3, or3, order, 2.0,
                                           scr.data_ptr(), n_scr - 1, sh))


def test_fixed_resolution_kernel_with_density():
    """The density map is resampled to the kernel grid (trilinear, no volume scaling) and
    used there; the pipeline equals the oracle's resample -> conv / rho -> resample."""
    from pyvoxeldosimetry_gb300.core.kernel_convolution import KernelConvolutionCalculator
    rng = np.random.default_rng(21)
    act = (rng.random((24, 22, 26)) ** 3 * 1e5).astype(np.float32)
    rho = rng.uniform(0.5, 1.5, act.shape).astype(np.float32)
    idx = np.indices((7, 7, 7)) - 3.0
    k = np.exp(-np.sqrt((idx ** 2).sum(0)) / 1.8) / np.maximum(np.sqrt((idx ** 2).sum(0)), 0.62) ** 2
    vs, kr = (1.5, 1.5, 1.5), 2.0
    calc = KernelConvolutionCalculator("Y90", kernel_resolution=kr, config={"kernel": k, "autotune": False})
    d = calc.calculate_dose_rate(act, vs, density=rho)
    a2 = ors.resample(act, vs, (kr,) * 3, conserve_total=True)
    r2 = ors.resample(rho, vs, (kr,) * 3, order=1)
    d2 = oc.density_scale(oc.linear_conv_same(a2, k), r2)
    ref = ors.resample(d2, (kr,) * 3, vs, output_shape=act.shape)
    assert np.abs(d - ref).max() <= 1e-4 * np.abs(ref).max()

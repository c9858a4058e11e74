"""GPU dose-volume histogram against the reference's calculate_dvh
(core/utils.py:233-262): golden vectors produced by the reference itself, and
the oracle (np.histogram) on larger volumes.  Counts are integer work, so the
results must be identical, not close."""
import numpy as np
import pytest
import torch

from oracle import dvh as od

pytestmark = pytest.mark.gpu

CASES = ["f32_bool", "f32_ties", "f64_const", "f64_many_bins"]


@pytest.mark.parametrize("name", CASES)
def test_dvh_equals_reference_golden(golden, name):
    from pyvoxeldosimetry_gb300.core.utils import calculate_dvh
    e, c = calculate_dvh(golden[f"dvh_{name}_dose"], golden[f"dvh_{name}_mask"], int(golden[f"dvh_{name}_bins"]))
    assert e.dtype == golden[f"dvh_{name}_edges"].dtype
    np.testing.assert_array_equal(e, golden[f"dvh_{name}_edges"])
    np.testing.assert_array_equal(c, golden[f"dvh_{name}_cum"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("bins", [1, 3, 1000, 12288, 12289, 50000])
def test_dvh_equals_oracle_on_a_dose_volume(dtype, bins):
    from pyvoxeldosimetry_gb300.core.utils import calculate_dvh
    rng = np.random.default_rng(bins)
    shape = (64, 72, 80)
    dose = (rng.gamma(1.5, 4.0, shape)).astype(dtype)
    dose[::7] = np.round(dose[::7] * 8) / 8  # ties on a grid
    mask = rng.random(shape) > 0.35
    e, c = calculate_dvh(dose, mask, bins)
    e0, c0 = od.calculate_dvh(dose, mask, bins)
    np.testing.assert_array_equal(e, e0)
    np.testing.assert_array_equal(c, c0)


def test_dvh_device_tensors_and_mask_kinds():
    from pyvoxeldosimetry_gb300.core.utils import calculate_dvh
    rng = np.random.default_rng(5)
    shape = (40, 50, 60)
    dose = rng.random(shape).astype(np.float32) * 70.0
    fmask = rng.random(shape).astype(np.float32) - 0.2       # float mask: > 0 counts
    imask = (rng.random(shape) * 3).astype(np.int32)          # int mask: promoted to (mask > 0)
    for m in (fmask, imask, torch.from_numpy(fmask).cuda(), torch.from_numpy(imask > 0).cuda()):
        e, c = calculate_dvh(torch.from_numpy(dose).cuda(), m, 256)
        mm = m.cpu().numpy() if isinstance(m, torch.Tensor) else m
        e0, c0 = od.calculate_dvh(dose, mm, 256)
        np.testing.assert_array_equal(e, e0)
        np.testing.assert_array_equal(c, c0)


def test_dvh_errors_match_the_reference():
    from pyvoxeldosimetry_gb300.core.utils import calculate_dvh
    d = np.ones((4, 5, 6), np.float32)
    with pytest.raises(ValueError, match="same dimensions"):
        calculate_dvh(d, np.ones((4, 5, 7), bool))
    with pytest.raises(ValueError, match="empty"):
        calculate_dvh(d, np.zeros((4, 5, 6), bool))
    d2 = d.copy()
    d2[1, 1, 1] = np.nan
    with pytest.raises(ValueError, match="not finite"):
        calculate_dvh(d2, np.ones((4, 5, 6), bool))
    d2[1, 1, 1] = np.inf
    with pytest.raises(ValueError, match="not finite"):
        calculate_dvh(d2, np.ones((4, 5, 6), bool))
    # a non-finite dose outside the ROI is ignored, as in the reference
    m = np.ones((4, 5, 6), bool)
    m[1, 1, 1] = False
    e, c = calculate_dvh(d2, m, 10)
    e0, c0 = od.calculate_dvh(d2, m, 10)
    np.testing.assert_array_equal(e, e0)
    np.testing.assert_array_equal(c, c0)
    with pytest.raises(ValueError):
        calculate_dvh(d, m, 0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_device_edges_equal_numpy_linspace(dtype):
    """pvd_dvh computes numpy's histogram edges on the device; they must be np.linspace's."""
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    rng = np.random.default_rng(12)
    tiny = np.finfo(dtype).tiny
    cases = [rng.gamma(2.0, 5.0, 5000).astype(dtype), np.full(100, dtype(3.25)),
             (rng.random(777) * 3 * tiny).astype(dtype), (rng.standard_normal(999) * 1e6).astype(dtype)]
    for dose in cases:
        for bins in (1, 7, 1000):
            d = torch.from_numpy(dose).cuda()
            m = torch.ones(dose.shape, dtype=torch.uint8, device="cuda")
            res = torch.empty(4 + bins, dtype=torch.int64, device="cuda")
            edges = torch.empty(bins + 1, dtype=d.dtype, device="cuda")
            dt = N.PVD_DTYPE_F32 if dtype is np.float32 else N.PVD_DTYPE_F64
            N.check(lib.pvd_dvh(d.data_ptr(), dt, m.data_ptr(), N.PVD_DTYPE_U8, dose.size, bins, edges.data_ptr(),
                                res.data_ptr(), torch.cuda.current_stream().cuda_stream))
            first, last = dose.min(), dose.max()
            if first == last:
                first, last = first - 0.5, last + 0.5
            np.testing.assert_array_equal(edges.cpu().numpy(), np.linspace(first, last, bins + 1, dtype=dtype))
            h, _ = np.histogram(dose, bins=bins)
            np.testing.assert_array_equal(res.cpu().numpy()[4:], h)

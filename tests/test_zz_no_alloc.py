"""The allocation-free convolution entry point, pvd_conv_execute_static.

It exists for callers that cannot allocate device memory (a host framework
that owns the allocator, a plugin that must not call cudaMalloc/cudaFree,
which synchronise the device).  Through the C ABI it must give the same dose
as the plan-based entry point (pvd_plan_create + pvd_plan_set_kernel +
pvd_conv_execute), within the tolerance of the other parity tests, on two
calls in a row that share its static scratch array, without changing the
device's free memory.  This file is collected last so that a run stopping at
the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-5  # normwise relative error, as in the other convolution parity tests


def rel_err(d, ref):
    d = np.asarray(d, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.abs(d - ref).max() / np.abs(ref).max())


def radial_kernel(k, lam, dx):
    c = k // 2
    idx = np.indices((k, k, k)) - c
    r = np.sqrt((idx ** 2).sum(0)) * dx
    r = np.where(r == 0, dx * (3 / (4 * np.pi)) ** (1 / 3), r)
    return np.exp(-r / lam) / r ** 2


def plan_dose(lib, act_d, rho_d, kernel, scale, flags, out_scale):
    """Dose through the existing plan-based entry point."""
    from pyvoxeldosimetry_gb300 import _native as N
    shape = tuple(act_d.shape)
    d = N.ConvDesc()
    for i in range(3):
        d.n[i], d.kmax[i], d.pad[i] = shape[i], kernel.shape[i], 0
    d.mode, d.n_kernels, d.flags = N.PVD_MODE_LINEAR, 1, 0
    h = C.c_void_p()
    N.check(lib.pvd_plan_create(C.byref(d), C.byref(h)))
    try:
        k = np.ascontiguousarray(kernel, np.float64)
        N.check(lib.pvd_plan_set_kernel(h, 0, k.ctypes.data, *k.shape, scale, flags))
        out = torch.empty(shape, dtype=torch.float32, device="cuda")
        N.check(lib.pvd_conv_execute(h, act_d.data_ptr(), rho_d.data_ptr() if rho_d is not None else None,
                                     out.data_ptr(), C.c_float(out_scale), torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        return out.cpu().numpy()
    finally:
        lib.pvd_plan_destroy(h)


def static_dose(lib, act_d, rho_d, out_d, kernel, scale, flags, out_scale):
    """Dose through pvd_conv_execute_static; `out_d` is allocated by the caller."""
    from pyvoxeldosimetry_gb300 import _native as N
    k = np.ascontiguousarray(kernel, np.float64)
    n0, n1, n2 = act_d.shape
    N.check(lib.pvd_conv_execute_static(act_d.data_ptr(), rho_d.data_ptr() if rho_d is not None else None,
                                        out_d.data_ptr(), n0, n1, n2, k.ctypes.data, *k.shape, scale, flags,
                                        C.c_float(out_scale), torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return out_d.cpu().numpy()


def test_static_entry_point_matches_plan_on_two_calls():
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    rng = np.random.default_rng(17)
    shape = (96, 80, 112)
    act = torch.from_numpy((rng.random(shape) * 1e5).astype(np.float32)).cuda()
    rho = torch.from_numpy(rng.uniform(0.3, 1.9, shape).astype(np.float32)).cuda()
    k_radial = radial_kernel(15, 1.8, 2.0)           # real-even spectrum, normalised on the GPU
    k_asym = rng.random((5, 9, 7))                   # complex spectrum, used as given
    out = torch.empty(shape, dtype=torch.float32, device="cuda")

    ref1 = plan_dose(lib, act, rho, k_radial, 2.5e-3, N.PVD_KERNEL_NORMALIZE, 3.0)
    ref2 = plan_dose(lib, act, None, k_asym, 1.0, 0, 1.0)

    d1 = static_dose(lib, act, rho, out, k_radial, 2.5e-3, N.PVD_KERNEL_NORMALIZE, 3.0)
    assert rel_err(d1, ref1) <= TOL
    free_before = torch.cuda.mem_get_info()[0]
    d2 = static_dose(lib, act, None, out, k_asym, 1.0, 0, 1.0)   # second call, different kernel and mode
    assert torch.cuda.mem_get_info()[0] == free_before           # nothing allocated by the call
    assert rel_err(d2, ref2) <= TOL
    d3 = static_dose(lib, act, rho, out, k_radial, 2.5e-3, N.PVD_KERNEL_NORMALIZE, 3.0)
    np.testing.assert_array_equal(d3, d1)                        # the shared array's old contents do not leak


def test_static_entry_point_rejects_sizes_beyond_its_array():
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    k = np.ones((21, 21, 21))
    st = lib.pvd_conv_execute_static(C.c_void_p(16), None, C.c_void_p(16), 256, 256, 256, k.ctypes.data,
                                     21, 21, 21, 1.0, 0, C.c_float(1.0), None)
    assert st == 6  # PVD_ERR_UNSUPPORTED, before any device work
    assert "static maximum" in N.last_error()


def test_static_entry_point_capacity_128cube_15kernel():
    """The size the header names as fitting the static array (128^3 with a 15^3 kernel)
    runs and agrees with the plan path."""
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    rng = np.random.default_rng(23)
    shape = (128, 128, 128)
    act = torch.from_numpy((rng.random(shape) * 1e5).astype(np.float32)).cuda()
    k = radial_kernel(15, 1.8, 2.0)
    out = torch.empty(shape, dtype=torch.float32, device="cuda")
    ref = plan_dose(lib, act, None, k, 1.0, N.PVD_KERNEL_NORMALIZE, 1.0)
    d = static_dose(lib, act, None, out, k, 1.0, N.PVD_KERNEL_NORMALIZE, 1.0)
    assert rel_err(d, ref) <= TOL


def test_static_entry_point_rejects_a_kernel_it_cannot_normalise():
    """A kernel summing to zero (a difference kernel) cannot be normalised: the call
    returns PVD_ERR_NUMERIC like pvd_plan_set_kernel, instead of an Inf/NaN dose."""
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    k = np.zeros((3, 3, 3))
    k[0, 1, 1], k[2, 1, 1] = 1.0, -1.0
    act = torch.ones((8, 8, 8), dtype=torch.float32, device="cuda")
    out = torch.empty_like(act)
    st = lib.pvd_conv_execute_static(act.data_ptr(), None, out.data_ptr(), 8, 8, 8, k.ctypes.data, 3, 3, 3, 1.0,
                                     N.PVD_KERNEL_NORMALIZE, C.c_float(1.0), None)
    assert st == 5  # PVD_ERR_NUMERIC
    assert "cannot normalise" in N.last_error()
    d = static_dose(lib, act, None, out, k, 1.0, 0, 1.0)  # used as given, it is a valid kernel
    assert np.isfinite(d).all()

"""Failure detection without a GPU fault.

* Every bounded device wait's timeout path: pvd_wait_check waits, through the same
  bounded wait and failure recording as the plan's TMA column passes and the U-Net's
  tensor-core pipeline, on an mbarrier phase that nothing completes (no copy or MMA is
  in flight), with a 1 ms limit.  The timeout is reported as PVD_ERR_TIMEOUT by
  pvd_plan_status / pvd_unet_status, the status word is then clear, and the context
  still computes correct results.
* Allocation failure: a host-side cap on a plan's device bytes makes pvd_plan_create
  and pvd_plan_set_kernel fail with PVD_ERR_OOM, as an exhausted device would, without
  leaking what they had allocated.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TIMEOUT = 4


def _plan(lib, N, shape=(16, 16, 16), k=(3, 3, 3), tma=False):
    d = N.ConvDesc()
    for i in range(3):
        d.n[i], d.kmax[i], d.pad[i] = shape[i], k[i], 0
    d.mode, d.n_kernels, d.flags = N.PVD_MODE_LINEAR, 1, N.PVD_PLAN_TMA if tma else 0
    h = C.c_void_p()
    st = lib.pvd_plan_create(C.byref(d), C.byref(h))
    return st, h


@pytest.mark.parametrize("tma", [False, True])
def test_plan_wait_timeout_is_reported_then_cleared(tma):
    from oracle import conv as oc
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    st, h = _plan(lib, N, tma=tma)
    N.check(st)
    try:
        assert lib.pvd_plan_status(h) == 0
        N.check(lib.pvd_wait_check(N.PVD_WAITCHECK_PLAN, h, 1_000_000, None))
        assert lib.pvd_plan_status(h) == TIMEOUT
        assert "bounded wait" in N.last_error()
        assert lib.pvd_plan_status(h) == 0          # reported once, then clear
        # the context and the plan still work
        rng = np.random.default_rng(3)
        a = rng.random((16, 16, 16)).astype(np.float32)
        k = rng.random((3, 3, 3))
        N.check(lib.pvd_plan_set_kernel(h, 0, k.ctypes.data, 3, 3, 3, 1.0, 0))
        at = torch.from_numpy(a).cuda()
        out = torch.empty_like(at)
        N.check(lib.pvd_conv_execute(h, at.data_ptr(), None, out.data_ptr(), C.c_float(1.0), None))
        torch.cuda.synchronize()
        ref = oc.linear_conv_same(a.astype(np.float64), k)
        assert np.abs(out.cpu().numpy() - ref).max() / np.abs(ref).max() <= 1e-5
        assert lib.pvd_plan_status(h) == 0
    finally:
        lib.pvd_plan_destroy(h)


def test_unet_wait_timeout_is_reported_then_cleared():
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    code = C.c_int()
    N.check(lib.pvd_unet_status(C.byref(code), 1))
    N.check(lib.pvd_wait_check(N.PVD_WAITCHECK_UNET, None, 1_000_000, None))
    assert lib.pvd_unet_status(C.byref(code), 1) == TIMEOUT and code.value == 1   # the load warp's code
    assert lib.pvd_unet_status(C.byref(code), 0) == 0 and code.value == 0        # reset by the read above
    torch.cuda.synchronize()


def test_wait_check_arguments():
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    assert lib.pvd_wait_check(N.PVD_WAITCHECK_PLAN, None, 1000, None) == 1
    assert lib.pvd_wait_check(7, None, 1000, None) == 1
    assert lib.pvd_wait_check(N.PVD_WAITCHECK_UNET, None, 0, None) == 1
    assert lib.pvd_wait_check(N.PVD_WAITCHECK_UNET, None, 3_000_000_000, None) == 1


def test_allocation_cap_gives_oom_without_leaking():
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    for shape, k in (((128, 128, 128), (15, 15, 15)), ((8, 8, 8), (3, 3, 3))):
        st, h = _plan(lib, N, shape=shape, k=k)   # loads the kernels' code before the baseline
        N.check(st)
        lib.pvd_plan_destroy(h)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    try:
        N.check(lib.pvd_set_plan_alloc_cap(1 << 20))                 # 1 MiB: a 128^3 plan needs far more
        st, h = _plan(lib, N, shape=(128, 128, 128), k=(15, 15, 15))
        assert st == 3 and not h.value                              # PVD_ERR_OOM, no handle
        assert "allocation cap" in N.last_error()
        # a plan that fits, whose kernel spectrum then does not
        st, h = _plan(lib, N, shape=(8, 8, 8), k=(3, 3, 3))
        N.check(st)
        info = N.PlanInfo()
        N.check(lib.pvd_plan_get_info(h, C.byref(info)))
        N.check(lib.pvd_set_plan_alloc_cap(int(info.workspace_bytes) + 16))
        k = np.ones((3, 3, 3))
        assert lib.pvd_plan_set_kernel(h, 0, k.ctypes.data, 3, 3, 3, 1.0, 0) == 3
        lib.pvd_plan_destroy(h)
    finally:
        N.check(lib.pvd_set_plan_alloc_cap(0))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0                     # nothing left allocated
    st, h = _plan(lib, N, shape=(128, 128, 128), k=(15, 15, 15))     # without the cap it works
    N.check(st)
    lib.pvd_plan_destroy(h)

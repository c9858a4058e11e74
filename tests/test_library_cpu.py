"""The C-ABI library builds, loads and exports every symbol include/pvd.h
declares (no compute calls: there is no GPU here)."""
import ctypes
import re
from pathlib import Path

from pyvoxeldosimetry_gb300 import _build, _native

HEADER = Path(__file__).resolve().parents[1] / "include" / "pvd.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"\b(pvd_[a-z0-9_]+)\s*\(", text)


def test_header_and_binding_agree():
    assert declared_symbols() == _native.EXPORTED_SYMBOLS


def test_library_loads_and_exports_all_symbols():
    lib = _native.load()
    assert Path(_build.LIB_PATH).exists()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.pvd_version() >= 100
    assert lib.pvd_launch_count(1) >= 0


def test_errors_without_gpu_are_status_codes():
    lib = _native.load()
    # null arguments are rejected before any CUDA call
    assert lib.pvd_plan_create(None, None) == 1
    assert _native.last_error().startswith("pvd_plan_create")
    assert lib.pvd_conv_execute(None, None, None, None, ctypes.c_float(1.0), None) == 1


def test_fit_flag_validation_happens_before_any_cuda_call():
    lib = _native.load()
    t = (ctypes.c_double * 4)(1.0, 4.0, 24.0, 96.0)
    p0 = (ctypes.c_double * 5)(1.0, 0.1, 0.5, 0.01, 0.0)
    fake = ctypes.c_void_p(16)  # never dereferenced: every call below fails validation first

    def fit(model, flags, n_times=4, max_fev=100):
        return lib.pvd_tac_fit(model, t, None, n_times, p0, 0.0, 0.0, max_fev, flags, fake, 10,
                               fake, fake, None, None, 1.0, None)

    assert fit(_native.PVD_FIT_F2, _native.PVD_FIT_VARPRO) == 1
    assert "PVD_FIT_VARPRO" in _native.last_error()
    assert fit(_native.PVD_FIT_F3, _native.PVD_FIT_AUC_INF) == 1
    assert fit(_native.PVD_FIT_F2, _native.PVD_FIT_P0_FROM_DATA) == 1
    assert fit(_native.PVD_FIT_F4A, _native.PVD_FIT_VARPRO, n_times=17) == 1
    assert fit(_native.PVD_FIT_F4A, _native.PVD_FIT_VARPRO, max_fev=0) == 1
    assert fit(42, 0) == 1


def test_batch_validation_happens_before_any_cuda_call():
    lib = _native.load()
    t = (ctypes.c_double * 4)(1.0, 4.0, 24.0, 96.0)
    it = (_native.BatchItem * 1)()
    for f in ("plan", "activity_d", "params_d", "auc_d", "cum_d", "dose_d"):
        setattr(it[0], f, 16)  # never dereferenced: validation fails before the plan is looked at
    it[0].times = ctypes.cast(t, ctypes.c_void_p)
    it[0].n_times = 3
    assert lib.pvd_batch_execute(it, 1, 0, 100, 3600.0, None) == 1
    assert "n_times" in _native.last_error()
    it[0].n_times = 4
    t[2] = 4.0
    assert lib.pvd_batch_execute(it, 1, 0, 100, 3600.0, None) == 1
    assert "increase" in _native.last_error()
    it[0].plan = None
    assert lib.pvd_batch_execute(it, 1, 0, 100, 3600.0, None) == 1
    assert lib.pvd_batch_execute(it, 1, 0, 0, 3600.0, None) == 1
    h = ctypes.c_void_p()
    assert lib.pvd_batch_create(it, 1, 0, 100, 3600.0, ctypes.byref(h)) == 1 and not h.value
    assert lib.pvd_batch_run(None, None) == 1
    assert lib.pvd_batch_destroy(None) == 0


def test_fast_length_registry():
    from tests.test_conv_gpu import FAST_LENGTHS
    lens = _native.fast_lengths()
    assert lens == FAST_LENGTHS  # every registered length is exercised by the GPU tests
    assert lens == sorted(lens) and 280 in lens and 144 in lens
    for L in lens:
        r = L
        for p in (2, 3, 5, 7):
            while r % p == 0:
                r //= p
        assert r == 1

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

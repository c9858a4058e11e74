"""ORACLE — test infrastructure only: ctypes front end of oracle/mc_oracle.c."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_c

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build_c()))
        f = _lib.pvd_mc_oracle_run
        f.restype = C.c_int
        f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                      C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_void_p, C.c_int,
                      C.c_float, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_uint64, C.c_uint64,
                      C.c_uint64, C.c_void_p, C.c_void_p]
    return _lib


def run(activity, density, voxel_mm, tables, n_histories, seed, h_begin=0):
    """Energy grid (uint64, 2^-32 MeV units) and counters [weight, emitted, escaped, steps]
    of histories [h_begin, h_begin + n_histories) with Philox stream `seed`.

    ``tables`` is the dict built by pyvoxeldosimetry_gb300.core.monte_carlo.physics_tables."""
    lib = _load()
    a = np.ascontiguousarray(activity, np.float32)
    r = None if density is None else np.ascontiguousarray(density, np.float32)
    vm = np.ascontiguousarray(voxel_mm, np.float64)
    t = {k: (np.ascontiguousarray(v, np.float32) if isinstance(v, np.ndarray) else v) for k, v in tables.items()}
    ge = np.zeros(8, np.float32)
    gp = np.zeros(8, np.float32)
    ng = len(t["gamma_e"])
    ge[:ng] = t["gamma_e"]
    gp[:ng] = t["gamma_yield"]
    edep = np.zeros(a.size, np.uint64)
    cnt = np.zeros(4, np.uint64)
    lib.pvd_mc_oracle_run(a.shape[0], a.shape[1], a.shape[2], vm.ctypes.data, a.ctypes.data,
                          None if r is None else r.ctypes.data,
                          t["beta_icdf"].ctypes.data, len(t["beta_icdf"]), t["range"].ctypes.data, len(t["range"]),
                          float(t["range_de"]), t["mu_rho"].ctypes.data, t["compton_frac"].ctypes.data,
                          len(t["mu_rho"]), float(t["photon_de"]), ng, ge.ctypes.data, gp.ctypes.data,
                          float(t["beta_yield"]), float(t["e_cut"]), int(seed), int(h_begin),
                          int(h_begin + n_histories), edep.ctypes.data, cnt.ctypes.data)
    return edep.reshape(a.shape), cnt

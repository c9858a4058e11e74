"""The Monte Carlo oracle (C restatement, CPU): known answers for its random
number generator and physics sanity.  No GPU."""
import ctypes as C

import numpy as np
import pytest

from oracle import build_c
from oracle import mc as omc


def philox(ctr, key):
    lib = C.CDLL(str(build_c()))
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    lib.pvd_mc_oracle_philox(c, k)
    return list(c)


def test_philox4x32_10_known_answers():
    # known-answer vectors published with the Random123 library for philox4x32-10
    assert philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.fixture(scope="module")
def y90_tables():
    from pyvoxeldosimetry_gb300.core.monte_carlo import physics_tables
    return physics_tables("Y90")


def test_energy_is_conserved(y90_tables):
    rng = np.random.default_rng(0)
    shape = (16, 14, 18)
    act = rng.random(shape).astype(np.float32)
    rho = rng.uniform(0.2, 1.9, shape).astype(np.float32)
    edep, cnt = omc.run(act, rho, (2.0, 2.0, 2.0), y90_tables, 4000, seed=7)
    dep = int(edep.astype(np.uint64).sum(dtype=np.uint64))
    emitted, escaped = int(cnt[1]), int(cnt[2])
    assert emitted > 0 and escaped > 0
    assert abs(dep + escaped - emitted) <= 1e-5 * emitted


def test_mean_beta_energy_matches_spectrum(y90_tables):
    from pyvoxeldosimetry_gb300.data import mc_physics as mp
    act = np.zeros((3, 3, 3), np.float32)
    act[1, 1, 1] = 1.0
    n = 20000
    _, cnt = omc.run(act, None, (1.0, 1.0, 1.0), y90_tables, n, seed=3)
    mean = int(cnt[1]) * 2.0 ** -32 / n
    assert mean == pytest.approx(mp.spectrum_mean("Y90"), rel=0.02)


def test_point_source_stays_within_csda_range(y90_tables):
    from pyvoxeldosimetry_gb300.data import mc_physics as mp
    shape = (41, 41, 41)
    act = np.zeros(shape, np.float32)
    act[20, 20, 20] = 1.0
    edep, _ = omc.run(act, None, (1.0, 1.0, 1.0), y90_tables, 3000, seed=11)
    idx = np.argwhere(edep > 0)
    r_mm = np.sqrt(((idx - 20) ** 2).sum(1)).max()
    r_csda_mm = 10.0 * float(mp.katz_penfold_range(2.28))  # water, cm -> mm
    assert r_mm <= r_csda_mm + 2.0     # voxel size slack
    assert edep[20, 20, 20] == edep.max()

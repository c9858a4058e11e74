"""GPU Monte Carlo (pvd_mc_run through the C ABI) against the CPU oracle.

The reference's own MC cannot run (core/monte_carlo.py:38-40), so parity is
against the oracle's independent C restatement of the same algorithm: identical
Philox4x32-10 streams and IEEE single-precision operation sequences, energy in
64-bit fixed point, hence a bit-identical energy grid.  Plus physics known
answers (energy conservation, charged-particle equilibrium).
"""
import numpy as np
import pytest
import torch

from oracle import mc as omc

pytestmark = pytest.mark.gpu


def phantom(shape, seed):
    rng = np.random.default_rng(seed)
    act = (rng.random(shape) ** 4 * 1e6).astype(np.float32)
    act[0, :, :] = 0.0
    act[1, 1, 1] = np.nan          # NaN activity counts as zero
    rho = np.full(shape, 1.05, np.float32)
    rho[:, : shape[1] // 3, :] = 0.3      # lung slab
    rho[:, :, -3:] = 1.85                 # bone slab
    rho[2, 2, :] = 0.0012                 # air channel
    rho[3, 3, 3] = 0.0                    # zero-density voxel: dose 0
    return act, rho


@pytest.mark.parametrize("nuc", ["Y90", "Lu177", "I131"])
def test_gpu_energy_grid_is_bit_identical_to_oracle(nuc):
    from pyvoxeldosimetry_gb300.core.monte_carlo import McPlan, physics_tables
    tables = physics_tables(nuc)
    shape = (14, 12, 16)
    vox = (2.0, 1.5, 2.5)
    act, rho = phantom(shape, 3)
    n_hist, seed = 20000, 12345
    plan = McPlan(shape, vox, tables)
    edep, dose, st = plan.run(torch.from_numpy(act).cuda(), torch.from_numpy(rho).cuda(), n_hist, seed,
                              dose=True, stats=True)
    g = edep.cpu().numpy().view(np.uint64)
    ref, cnt = omc.run(act, rho, vox, tables, n_hist, seed)
    assert st["total_weight"] == int(cnt[0])
    assert st["emitted"] == int(cnt[1]) and st["escaped"] == int(cnt[2]) and st["steps"] == int(cnt[3])
    np.testing.assert_array_equal(g, ref)
    # dose-rate conversion: E / N * activity * J/MeV / (rho dV)
    d = dose.cpu().numpy().astype(np.float64)
    bq = st["activity_bq"]
    with np.errstate(divide="ignore"):
        ref_d = ref.astype(np.float64) * 2.0 ** -32 * bq / n_hist * 1.602176634e-13 / (rho * np.prod(vox) * 1e-6)
    ref_d[rho <= 0] = 0.0
    np.testing.assert_allclose(d, ref_d, rtol=1e-6, atol=0)
    assert d[3, 3, 3] == 0.0
    plan.close()


def test_gpu_mc_is_deterministic_and_conserves_energy():
    from pyvoxeldosimetry_gb300.core.monte_carlo import McPlan, physics_tables
    tables = physics_tables("Lu177")
    shape = (32, 30, 28)
    act, rho = phantom(shape, 8)
    a, r = torch.from_numpy(act).cuda(), torch.from_numpy(rho).cuda()
    plan = McPlan(shape, (2.0, 2.0, 2.0), tables)
    e1, _, s1 = plan.run(a, r, 200000, 99, dose=False, stats=True)
    e2, _, s2 = plan.run(a, r, 200000, 99, dose=False, stats=True)
    e3, _, _ = plan.run(a, r, 200000, 100, dose=False, stats=True)
    assert torch.equal(e1, e2) and s1 == s2
    assert not torch.equal(e1, e3)
    dep = int(e1.cpu().numpy().view(np.uint64).sum(dtype=np.uint64))
    assert abs(dep + s1["escaped"] - s1["emitted"]) <= 1e-5 * s1["emitted"]


def test_charged_particle_equilibrium_known_answer():
    """Uniform Y-90 concentration in water: far from the edges every voxel absorbs
    what it emits, so the dose rate is A_voxel * E_mean * J/MeV / m_voxel."""
    from pyvoxeldosimetry_gb300 import DoseCalculator
    from pyvoxeldosimetry_gb300.data import mc_physics as mp
    shape = (64, 64, 64)
    vox = 1.0
    act = np.full(shape, 1000.0, np.float32)
    calc = DoseCalculator("Y90", method="monte_carlo", config={"n_particles": 4_000_000, "random_seed": 5})
    d = calc.calculator.calculate_dose_rate(act, (vox,) * 3)
    inner = d[16:48, 16:48, 16:48]      # > 11 mm (the Y-90 CSDA range) from every face
    expect = 1000.0 * mp.spectrum_mean("Y90") * 1.602176634e-13 / (1.0 * vox ** 3 * 1e-6)
    assert inner.mean() == pytest.approx(expect, rel=0.01)
    # statistical scatter of the voxel doses around the mean
    assert inner.std() / inner.mean() < 0.2


def test_mc_calculator_api():
    from pyvoxeldosimetry_gb300 import DoseCalculator
    from pyvoxeldosimetry_gb300.core.monte_carlo import MonteCarloCalculator
    act = np.zeros((20, 20, 20), np.float32)
    act[8:12, 8:12, 8:12] = 1e6
    calc = DoseCalculator("I131", method="gpu_monte_carlo", config={"n_particles": 50000})
    assert isinstance(calc.calculator, MonteCarloCalculator)
    r = calc.calculate_dose(activity_maps=[act], time_points=[0.0], voxel_size=(2.0, 2.0, 2.0))
    assert r.dose_rate_maps[0].shape == act.shape and np.isfinite(r.dose_rate_maps[0]).all()
    assert r.dose_rate_maps[0][10, 10, 10] > r.dose_rate_maps[0][0, 0, 0]
    maps = [act, act * 0.5]
    dose = calc.calculator.calculate_absorbed_dose(maps, [0.0, 10.0], (2.0, 2.0, 2.0))
    assert dose.shape == act.shape and dose.max() > 0

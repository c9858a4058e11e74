"""HU -> tissue masks and density on the GPU (pvd_hu_composition through
TissueComposition) against the reference's own masks (tests/golden, tissue_*) and the
oracle's density calibration, and fed into the density-scaled convolution."""
import numpy as np
import pytest
import torch

from oracle import conv as oc
from oracle import tissue as ot

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["odd", "thin"])
@pytest.mark.parametrize("art", [0, 1])
def test_masks_equal_reference(golden, name, art):
    from pyvoxeldosimetry_gb300.tissue import TissueComposition
    ct = golden[f"tissue_{name}_ct"]          # integer HU, exact in float32
    comp = TissueComposition().calculate_composition(ct, handle_artifacts=bool(art))
    assert list(comp) == ["air", "lung", "soft_tissue", "bone", "water"]
    for t, m in comp.items():
        assert m.dtype == np.float64
        np.testing.assert_array_equal(m, golden[f"tissue_{name}_{art}_{t}"], err_msg=t)


@pytest.mark.parametrize("art", [False, True])
def test_density_and_corrected_hu_against_oracle(art):
    from pyvoxeldosimetry_gb300.tissue import DEFAULT_HU_DENSITY, TissueComposition
    rng = np.random.default_rng(8)
    ct = np.round(rng.uniform(-1200.0, 3500.0, (21, 18, 26))).astype(np.float32)
    ct[3, 4, 5] = np.nan
    ct[10, 8:11, 12:15] = 3100.0
    tc = TissueComposition()
    masks, rho = tc.calculate_composition_and_density(torch.from_numpy(ct).cuda(), handle_artifacts=art)
    ref = ot.density(ct.astype(np.float64), DEFAULT_HU_DENSITY, artifacts=art)
    r = rho.cpu().numpy()
    assert r[3, 4, 5] == 0.0
    np.testing.assert_allclose(r, ref, rtol=1e-6, atol=1e-6)
    refm = ot.composition(ct.astype(np.float64), artifacts=art)
    for i, t in enumerate(["air", "lung", "soft_tissue", "bone", "water"]):
        np.testing.assert_array_equal(masks[t].cpu().numpy(), refm[t].astype(np.float32))


def test_ct_density_feeds_the_density_scaled_dose():
    """DoseCalculator.calculate_dose(ct_image=HU) == the density-scaled dose with the
    density the calibration gives."""
    from pyvoxeldosimetry_gb300 import DoseCalculator
    from pyvoxeldosimetry_gb300.data import nuclides as nd
    from pyvoxeldosimetry_gb300.tissue import DEFAULT_HU_DENSITY
    rng = np.random.default_rng(9)
    shape = (30, 28, 32)
    ct = np.full(shape, -1000.0, np.float32)
    ct[4:26, 4:24, 4:28] = 40.0
    ct[8:14, 8:20, 8:14] = -750.0
    ct[18:22, 10:14, 16:22] = 1200.0
    act = (rng.random(shape) * 1e5).astype(np.float32)
    dc = DoseCalculator("Y90", config={"kernel_resolution": 2.0, "autotune": False})
    res = dc.calculate_dose(activity_maps=[act], time_points=[0.0], voxel_size=(2.0, 2.0, 2.0), ct_image=ct)
    k = nd.analytic_profile("Y90", 2.0)
    rho = ot.density(ct.astype(np.float64), DEFAULT_HU_DENSITY)
    ref = oc.density_scale(oc.linear_conv_same(act.astype(np.float64), k / k.sum() * nd.gy_per_bq_s_scale("Y90", 2.0)),
                           rho)
    st = oc.error_stats(res.dose_rate_maps[0], ref, density=rho)
    assert st["energy_max_normwise"] <= 1e-5 and st["tissue_max_normwise"] <= 1e-5

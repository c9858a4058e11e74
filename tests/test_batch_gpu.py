"""Batched time-integrated dose (per-voxel two-exponential fit + convolution of
the cumulated activity, all volumes captured in one CUDA graph) against the
analytic truth and the FP64 convolution oracle."""
import numpy as np
import pytest
import torch

from oracle import conv as oc

pytestmark = pytest.mark.gpu

TIMES = [1.0, 4.0, 24.0, 96.0]


def biexp_volume(shape, seed):
    rng = np.random.default_rng(seed)
    a0 = (rng.random(shape) ** 2 * 1e5 + 10.0)
    t1 = np.exp(rng.uniform(np.log(6), np.log(160), shape))
    t2 = np.exp(rng.uniform(np.log(6), np.log(160), shape))
    w = rng.uniform(0.2, 0.8, shape)
    k1, k2 = np.log(2) / t1, np.log(2) / t2
    acts = np.stack([a0 * (w * np.exp(-k1 * t) + (1 - w) * np.exp(-k2 * t)) for t in TIMES]).astype(np.float32)
    auc = a0 * (w / k1 + (1 - w) / k2)          # exact cumulated activity, Bq h
    return acts, auc


def kernel_S(nuc, vs):
    from pyvoxeldosimetry_gb300.data import nuclides as nd
    k = nd.analytic_profile(nuc, vs, nd.default_kernel_size(nuc, vs))
    return k / k.sum() * nd.gy_per_bq_s_scale(nuc, vs)


@pytest.fixture(scope="module")
def batch_case():
    specs = [((40, 36, 44), 2.0, False), ((52, 30, 38), 1.5, True), ((24, 64, 32), 2.0, False)]
    vols, truth = [], []
    for i, (shape, vs, dens) in enumerate(specs):
        acts, auc = biexp_volume(shape, 100 + i)
        rho = np.random.default_rng(i).uniform(0.3, 1.9, shape).astype(np.float32) if dens else None
        vols.append({"activity": torch.from_numpy(acts).cuda(), "times": TIMES, "voxel_size": (vs,) * 3,
                     "density": None if rho is None else torch.from_numpy(rho).cuda()})
        truth.append((auc, vs, rho))
    return vols, truth


def test_batch_dose_matches_truth_and_oracle(batch_case):
    from pyvoxeldosimetry_gb300.batch import BatchDoseCalculator
    vols, truth = batch_case
    bc = BatchDoseCalculator("Y90", use_graph=True)
    doses = bc.calculate(vols)
    for i, (d, (auc, vs, rho)) in enumerate(zip(doses, truth)):
        _, fit_auc, ok = bc.fit_results(i)
        ok = ok.cpu().numpy()
        assert ok.mean() > 0.99
        fa = fit_auc.cpu().numpy()
        rel = np.abs(fa - auc) / auc
        assert np.quantile(rel[ok], 0.999) < 1e-4
        ref = oc.density_scale(oc.linear_conv_same(auc * 3600.0, kernel_S("Y90", vs)), rho)
        dd = d.cpu().numpy().astype(np.float64)
        assert np.abs(dd - ref).max() / np.abs(ref).max() < 1e-3
    bc.close()


def test_graph_replay_equals_eager_and_mixed_equals_fp64(batch_case):
    from pyvoxeldosimetry_gb300.batch import BatchDoseCalculator
    vols, _ = batch_case
    g = BatchDoseCalculator("Y90", use_graph=True)
    e = BatchDoseCalculator("Y90", use_graph=False)
    dg = [x.clone() for x in g.calculate(vols)]
    dg2 = [x.clone() for x in g.run()]                 # a second replay of the same graph
    de = e.calculate(vols)
    for a, b, c in zip(dg, dg2, de):
        assert torch.equal(a, b) and torch.equal(a, c)
    f64 = BatchDoseCalculator("Y90", use_graph=False, mixed_fit=False)
    df = f64.calculate(vols)
    for i in range(len(vols)):
        _, auc_m, ok_m = g.fit_results(i)
        _, auc_d, ok_d = f64.fit_results(i)
        both = (ok_m & ok_d)
        rel = ((auc_m - auc_d).abs() / auc_d.abs())[both]
        assert float(torch.quantile(rel.float(), 0.999)) < 1e-6
        assert float((df[i] - de[i]).abs().max() / de[i].abs().max()) < 1e-5
    for c in (g, e, f64):
        c.close()

"""Per-voxel time-activity-curve fits (FP64 on the GPU, through the C ABI) against
the reference's own outputs (golden vectors) and the scipy oracle."""
import numpy as np
import pytest

from oracle import time_fit as of

pytestmark = pytest.mark.gpu

# MINPACK stops at a relative cost reduction of 1.49e-8, the GPU LM converges
# further; parameters of the same minimum agree to this relative tolerance.
PTOL = 2e-5


def auc_rtol(params, limit):
    """AUC = A0/lam (1 - exp(-lam L)) amplifies a relative error in lam by about
    1 + |lam L|; the parameter tolerance is scaled accordingly."""
    lam = np.abs(np.asarray(params)[1])
    return PTOL * (1.0 + lam * limit)


def assert_auc_close(auc, ref_auc, params, limit):
    tol = auc_rtol(params, limit)
    err = np.abs(auc - ref_auc)
    assert np.all(err <= tol * np.abs(ref_auc) + 1e-300), float(np.max(err / (np.abs(ref_auc) + 1e-300) / tol))


def test_mono_fit_matches_reference_golden(golden):
    from pyvoxeldosimetry_gb300.time_integration import TimeCurveFitting
    tf = TimeCurveFitting(64.1)
    p, auc = tf.fit_time_activity_curve(list(golden["fit_times"]), list(golden["fit_acts"]))
    ref_p, ref_auc = golden["fit_params"], golden["fit_auc"]
    np.testing.assert_allclose(p, ref_p, rtol=PTOL, atol=1e-9 * np.abs(ref_p).max())
    np.testing.assert_array_equal(np.isnan(auc), np.isnan(ref_auc))
    assert_auc_close(auc, ref_auc, ref_p, 100 * 64.1)
    # edge cases recorded in the golden set: all-zero curve, growing curve, NaN sample
    flat_p = p.reshape(2, -1)
    assert flat_p[0, 0] == 0 and flat_p[1, 0] == pytest.approx(np.log(2) / 64.1)
    assert flat_p[1, 1] < 0
    assert flat_p[0, 2] == 0 and flat_p[1, 2] == pytest.approx(np.log(2) / 64.1)  # NaN -> fallback
    p_w, auc_w = tf.fit_time_activity_curve(list(golden["fit_times"]), list(golden["fit_acts"]),
                                            weight_factors=list(golden["fit_w"]))
    np.testing.assert_allclose(p_w, golden["fit_params_w"], rtol=PTOL, atol=1e-9 * np.abs(ref_p).max())
    assert_auc_close(auc_w, golden["fit_auc_w"], golden["fit_params_w"], 100 * 64.1)


@pytest.mark.parametrize("model,name", [("nukfit", "f2"), ("lmfit", "mono-exponential")])
def test_advanced_fit_matches_reference_golden(golden, model, name):
    from pyvoxeldosimetry_gb300.time_integration import TimeCurveFitting
    tf = TimeCurveFitting(64.1)
    p, auc = tf.fit_time_activity_curve_advanced(list(golden["adv_times"]), list(golden["adv_acts"]), model=model,
                                                 model_name=name)
    key = name.replace("-", "_")
    np.testing.assert_allclose(p, golden[f"adv_{key}_params"], rtol=PTOL)
    np.testing.assert_allclose(auc, golden[f"adv_{key}_auc"], rtol=PTOL)


@pytest.mark.parametrize("name", ["f3a", "f4a", "bi-exponential"])
def test_advanced_models_against_scipy_oracle(name):
    """Well-posed synthetic curves generated from each model: GPU and scipy reach the
    same minimum (compared through the fitted curve and the AUC, which are
    invariant to parameter permutations such as swapping the two exponentials)."""
    from pyvoxeldosimetry_gb300.time_integration import TimeCurveFitting
    rng = np.random.default_rng(4)
    t = np.array([1.0, 4.0, 24.0, 48.0, 96.0, 144.0])
    nv = 40
    lp = np.log(2) / 64.1
    if name == "f3a":
        a1, al, l1 = rng.uniform(0.5, 2, nv), rng.uniform(0.2, 0.8, nv), rng.uniform(0.02, 0.2, nv)
        y = a1 * (al * np.exp(-(l1 + lp) * t[:, None]) + (1 - al) * np.exp(-lp * t[:, None]))
        model = "nukfit"
    elif name == "f4a":
        a1, l1 = rng.uniform(0.5, 2, nv), rng.uniform(0.08, 0.2, nv)
        a2, l2 = rng.uniform(0.2, 1, nv), rng.uniform(0.002, 0.02, nv)
        y = a1 * np.exp(-(l1 + lp) * t[:, None]) + a2 * np.exp(-(l2 + lp) * t[:, None])
        model = "nukfit"
    else:
        a1, t1, t2 = rng.uniform(0.5, 2, nv), rng.uniform(40, 90, nv), rng.uniform(5, 15, nv)
        y = a1 * (np.exp(-np.log(2) * t[:, None] / t1) - np.exp(-np.log(2) * t[:, None] / t2))
        model = "lmfit"
    acts = [y[k].reshape(5, 8) for k in range(len(t))]
    tf = TimeCurveFitting(64.1)
    p, auc, info = tf.fit_time_activity_curve_advanced(list(t), acts, model=model, model_name=name,
                                                       return_fit_params=True)
    rp, rauc, rok = of.fit_advanced(t, acts, 64.1, model=model, model_name=name)
    both = info["success"].reshape(-1) & rok
    assert both.mean() > 0.8
    fn = of.model_functions(64.1)[0 if model == "nukfit" else 1][name][0]
    pf, rpf = p.reshape(len(p), -1), rp.reshape(len(rp), -1)
    for v in np.nonzero(both)[0]:
        np.testing.assert_allclose(fn(t, *pf[:, v]), fn(t, *rpf[:, v]), rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(auc.reshape(-1)[both], rauc.reshape(-1)[both], rtol=1e-4)


def test_fit_large_volume_runs_and_is_deterministic():
    import torch
    from pyvoxeldosimetry_gb300.phantoms import biexp_timeseries
    from pyvoxeldosimetry_gb300.time_integration import TimeCurveFitting
    rng = np.random.default_rng(0)
    a0 = rng.uniform(1e3, 1e5, (64, 64, 64)).astype(np.float32)
    ts, _ = biexp_timeseries(a0, [1.0, 4.0, 24.0, 96.0])
    acts = torch.from_numpy(ts).cuda()
    tf = TimeCurveFitting(64.1)
    p1, auc1 = tf.fit_time_activity_curve([1.0, 4.0, 24.0, 96.0], acts)
    p2, auc2 = tf.fit_time_activity_curve([1.0, 4.0, 24.0, 96.0], acts)
    assert torch.equal(p1, p2) and torch.equal(auc1, auc2)
    # spot-check against scipy on a seeded subsample
    idx = rng.choice(a0.size, 200, replace=False)
    sub = [ts[k].reshape(-1)[idx].reshape(10, 20) for k in range(4)]
    rp, rauc = of.fit_mono(np.array([1.0, 4.0, 24.0, 96.0]), sub, 64.1)
    np.testing.assert_allclose(p1.reshape(2, -1)[:, idx].cpu().numpy(), rp.reshape(2, -1), rtol=PTOL)

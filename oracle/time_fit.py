"""ORACLE — test infrastructure only, never the product path.

scipy restatement of the reference's per-voxel time-activity-curve fits
(pyvoxeldosimetry/time_integration/curve_fitting.py).  Same models, initial
guesses, sigma weighting, failure fallbacks and AUC formulas; runs scipy's
MINPACK Levenberg-Marquardt (scipy.optimize.curve_fit, method 'lm').  Pinned
against vectors produced by the reference itself
(tests/golden/reference_golden.npz).
"""
from __future__ import annotations

import warnings

import numpy as np
from scipy.optimize import curve_fit

LN2 = float(np.log(2.0))


def fit_mono(times, activities, half_life, weight_factors=None):
    """TimeCurveFitting.fit_time_activity_curve (curve_fitting.py:19-65) and
    _calculate_accumulated_dose (:74-84).

    Per voxel: curve_fit(A0*exp(-lam*t), p0=[A(t0), ln2/T_half], sigma=1/w);
    any exception -> [0, ln2/T_half]; AUC = A0/lam*(1-exp(-lam*100*T_half)).
    Returns (params (2, *shape), auc (*shape)).
    """
    lam_phys = np.log(2) / half_life
    times = np.array(times)
    acts = np.array(activities)
    if weight_factors is None:
        weight_factors = np.ones_like(times)
    n_t = len(times)
    shape = acts[0].shape
    y = acts.reshape(n_t, -1)
    params = np.zeros((2, y.shape[1]))

    def f(t, a0, lam):
        return a0 * np.exp(-lam * t)

    for i in range(y.shape[1]):
        try:
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                popt, _ = curve_fit(f, times, y[:, i], p0=[y[0, i], lam_phys], sigma=1 / np.array(weight_factors))
            params[:, i] = popt
        except Exception:
            params[:, i] = [0, lam_phys]
    limit = 100 * half_life
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        auc = params[0] / params[1] * (1 - np.exp(-params[1] * limit))
    return params.reshape((2, *shape)), auc.reshape(shape)


def model_functions(half_life, phys_half_life=None):
    """The model table of fit_time_activity_curve_advanced (curve_fitting.py:132-168)."""
    lam_default = np.log(2) / half_life

    def lp():
        return lam_default if phys_half_life is None else np.log(2) / phys_half_life

    def f2(t, a1, l1):
        return a1 * np.exp(-(l1 + lp()) * t)

    def f3(t, a1, l1, l2):
        return a1 * (np.exp(-(l1 + lp()) * t) - np.exp(-(l2 + lp()) * t))

    def f3a(t, a1, alpha, l1):
        return a1 * (alpha * np.exp(-(l1 + lp()) * t) + (1 - alpha) * np.exp(-lp() * t))

    def f4a(t, a1, l1, a2, l2):
        return a1 * np.exp(-(l1 + lp()) * t) + a2 * np.exp(-(l2 + lp()) * t)

    def f4b(t, a1, l1, a2, l2, lbc):
        return (a1 * np.exp(-(l1 + lp()) * t) - a2 * np.exp(-(l2 + lp()) * t)
                - (a1 - a2) * np.exp(-(lbc + lp()) * t))

    def f4c(t, a1, l1, a2, l2, lbc):
        return (a1 * np.exp(-(l1 + lp()) * t) + a2 * np.exp(-(l2 + lp()) * t)
                - (a1 + a2) * np.exp(-(lbc + lp()) * t))

    def mono(t, a1, t1):
        return a1 * np.exp(-np.log(2) * t / t1)

    def bi(t, a1, t1, t2):
        return a1 * (np.exp(-np.log(2) * t / t1) - np.exp(-np.log(2) * t / t2))

    def tri(t, a1, t1, a2, t2, tphys):
        return (a1 * np.exp(-np.log(2) * t / t1) - a2 * np.exp(-np.log(2) * t / t2)
                - (a1 - a2) * np.exp(-np.log(2) * t / tphys))

    nukfit = {"f2": (f2, [1.0, 0.1]), "f3": (f3, [1.0, 0.1, 0.01]), "f3a": (f3a, [1.0, 0.5, 0.1]),
              "f4a": (f4a, [1.0, 0.1, 0.5, 0.01]), "f4b": (f4b, [1.0, 0.1, 0.5, 0.01, 0.693]),
              "f4c": (f4c, [1.0, 0.1, 0.5, 0.01, 0.693])}
    lmfit = {"mono-exponential": (mono, [1.0, half_life]),
             "bi-exponential": (bi, [1.0, half_life, half_life / 2]),
             "tri-exponential": (tri, [1.0, half_life, 0.5, half_life / 2, half_life])}
    return nukfit, lmfit


def fit_advanced(times, activities, half_life, model="nukfit", model_name=None, weight_factors=None,
                 force_zero_at_t0=False, phys_half_life=None):
    """fit_time_activity_curve_advanced (curve_fitting.py:112-219).

    Per voxel curve_fit(..., p0=model p0, sigma=1/w, maxfev=10000); failure ->
    zeros; AUC = trapezoid of the fitted curve over the SAMPLED times only
    (:215, ``np.trapz``; ``np.trapezoid`` in numpy 2).
    Returns (params (n_p, *shape), auc (*shape), success (n_vox,) bool).
    """
    times = np.array(times)
    acts = np.array(activities)
    if weight_factors is None:
        weight_factors = np.ones_like(times)
    nukfit, lmfit = model_functions(half_life, phys_half_life)
    if model.lower() == "nukfit":
        models = nukfit
    elif model.lower() == "lmfit":
        models = lmfit
    else:
        raise ValueError(f"Unknown model type: {model}")
    if model_name is None:
        model_name = list(models.keys())[0]
    fn, p0 = models[model_name]
    n_t = len(times)
    shape = acts[0].shape
    y_all = acts.reshape(n_t, -1)
    params = np.zeros((len(p0), y_all.shape[1]))
    aucs = np.zeros(y_all.shape[1])
    ok = np.zeros(y_all.shape[1], dtype=bool)
    for i in range(y_all.shape[1]):
        y = y_all[:, i]
        if force_zero_at_t0:
            y = y - y[0]
            y[0] = 0
        try:
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                popt, _ = curve_fit(fn, times, y, p0=p0, sigma=1 / np.array(weight_factors), maxfev=10000)
            params[:, i] = popt
            ok[i] = True
        except Exception:
            params[:, i] = 0
        with np.errstate(all="ignore"):
            aucs[i] = np.trapezoid(fn(times, *params[:, i]), times)
    return params.reshape((len(p0), *shape)), aucs.reshape(shape), ok

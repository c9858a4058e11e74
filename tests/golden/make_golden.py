"""Generate golden vectors by running the reference implementation itself.

Imports devhliu/PyVoxelDosimetry from a read-only checkout (the directory named
by the PVD_REFERENCE environment variable) and records inputs/outputs of
the functions on the dose hot path into ``reference_golden.npz`` next to this
file.  The GPU machine has no reference checkout: the committed .npz is what the
tests read there.

The reference imports cupy, SimpleITK, nibabel, pydicom and matplotlib at
module import time; none is needed by the functions recorded here, so
permissive stub modules stand in for them.  numpy 2 removed ``np.trapz``
(used at time_integration/curve_fitting.py:215), so it is aliased to
``np.trapezoid``.

Recorded (reference file:line in parentheses):
  conv_*   KernelConvolutionCalculator.calculate_dose_rate (core/kernel_convolution.py:48-76)
  trap_*   ActivitySampler.integrate_activity (core/activity_sampler.py:48-78)
  absd_*   KernelConvolutionCalculator.calculate_absorbed_dose (core/kernel_convolution.py:78-106)
  fit_*    TimeCurveFitting.fit_time_activity_curve (time_integration/curve_fitting.py:19-84)
  adv_*    TimeCurveFitting.fit_time_activity_curve_advanced (curve_fitting.py:112-219)
  y90k_*   Y90KernelGenerator.generate_kernel (data/dose_kernels/y90_kernel.py:20-55)
  dvh_*    calculate_dvh (core/utils.py:233-262)
  tissue_* TissueComposition.calculate_composition (tissue/composition.py:48-93)
  reference_mc_decay.json: load_decay_data (data/mc_decay/__init__.py:10-24) of Y90, Lu177, I131
  kgen_*   Ga68KernelGenerator.generate_kernel (data/dose_kernels/ga68_kernel.py:19-106),
           Lu177KernelGenerator.generate_kernel (lu177_kernel.py:52-184), and the
           alpha / gamma terms of Ac225KernelGenerator (ac225_kernel.py:140-184; its
           generate_kernel calls a method the class does not define).  The generators'
           JSON files carry // comments, which json.load rejects; they are read with
           the comments stripped.

Run:  PVD_REFERENCE=<checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

REF = Path(os.environ["PVD_REFERENCE"]) if "PVD_REFERENCE" in os.environ else None
OUT = Path(__file__).resolve().parent / "reference_golden.npz"
DECAY_OUT = Path(__file__).resolve().parent / "reference_mc_decay.json"


class _Stub(types.ModuleType):
    """Module whose every attribute is a callable no-op stub."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Anything()


class _Anything:
    def __call__(self, *a, **k):
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]  # used as a decorator, e.g. @cp.fuse()
        return _Anything()

    def __getattr__(self, name):
        return _Anything()


def _install_stubs():
    for name in ["cupy", "SimpleITK", "nibabel", "pydicom", "matplotlib", "matplotlib.pyplot"]:
        sys.modules[name] = _Stub(name)
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid


def strip_json_comments(text: str) -> str:
    """Drop // comments outside string literals (the reference's kernel JSON files use them)."""
    out = []
    for line in text.splitlines():
        in_str, esc, cut = False, False, len(line)
        for i, ch in enumerate(line):
            if esc:
                esc = False
            elif ch == "\\":
                esc = True
            elif ch == '"':
                in_str = not in_str
            elif not in_str and line.startswith("//", i):
                cut = i
                break
        out.append(line[:cut])
    return "\n".join(out)


def main():
    if REF is None or not (REF / "pyvoxeldosimetry").is_dir():
        raise SystemExit("set PVD_REFERENCE to a checkout of devhliu/PyVoxelDosimetry")
    sys.dont_write_bytecode = True
    _install_stubs()
    sys.path.insert(0, str(REF))
    from pyvoxeldosimetry.core.activity_sampler import ActivitySampler
    from pyvoxeldosimetry.core.kernel_convolution import KernelConvolutionCalculator
    from pyvoxeldosimetry.data.dose_kernels.y90_kernel import Y90KernelGenerator
    from pyvoxeldosimetry.time_integration.curve_fitting import TimeCurveFitting

    rng = np.random.default_rng(20250208)
    g = {}

    def conv_calc(kernel, res=1.0):
        # bypass __init__ (it writes a kernel cache into the package directory) and inject the
        # kernel the way the reference's own examples reach into `calculator.kernel`
        c = KernelConvolutionCalculator.__new__(KernelConvolutionCalculator)
        c.kernel = kernel
        c.kernel_resolution = res
        c.radionuclide = "Y90"
        c.tissue_name = "water"
        c.config = {}
        return c

    # ---- convolution: ragged shapes, asymmetric / radial / oversize kernels ----
    cases = {
        "ragged_asym": ((12, 10, 14), (5, 3, 7), "rand"),
        "cube_radial": ((16, 16, 16), (5, 5, 5), "radial"),
        "oversize": ((6, 7, 8), (9, 9, 9), "rand"),      # kernel truncated to A.shape
        "even_kernel": ((10, 12, 8), (4, 4, 4), "rand"),
        "thin": ((1, 9, 20), (3, 3, 3), "rand"),
    }
    for name, (shape, kshape, kind) in cases.items():
        a = rng.random(shape) * 100.0
        if kind == "radial":
            c = [s // 2 for s in kshape]
            idx = np.indices(kshape)
            r = np.sqrt(sum((idx[i] - c[i]) ** 2 for i in range(3)) * 1.0)
            k = np.exp(-r / 1.8) / np.maximum(r, 0.62) ** 2
        else:
            k = rng.random(kshape)
        d = conv_calc(k).calculate_dose_rate(a, (1.0, 1.0, 1.0))
        g[f"conv_{name}_A"] = a
        g[f"conv_{name}_K"] = k
        g[f"conv_{name}_D"] = d

    # ---- trapezoid of activity (hours) ----
    maps = [rng.random((6, 5, 4)) * 1e3 for _ in range(4)]
    times = [1.0, 4.0, 24.0, 96.0]
    g["trap_maps"] = np.stack(maps)
    g["trap_times"] = np.array(times)
    g["trap_out"] = ActivitySampler(half_life=64.1).integrate_activity(maps, times)

    # ---- absorbed dose by trapezoid over per-timepoint dose rates ----
    k = rng.random((3, 3, 3))
    amaps = [rng.random((8, 6, 7)) * 10 for _ in range(3)]
    at = [0.0, 2.5, 24.0]
    g["absd_maps"] = np.stack(amaps)
    g["absd_times"] = np.array(at)
    g["absd_K"] = k
    g["absd_out"] = conv_calc(k).calculate_absorbed_dose(amaps, at, (1.0, 1.0, 1.0))

    # ---- mono-exponential per-voxel fit ----
    half_life = 64.1
    ft = np.array([1.0, 4.0, 24.0, 96.0])
    nvox = 60
    a0 = rng.uniform(1e2, 1e5, nvox)
    lam = np.log(2) / rng.uniform(6.0, 160.0, nvox)
    y = a0[None, :] * np.exp(-lam[None, :] * ft[:, None]) * (1 + 0.03 * rng.standard_normal((4, nvox)))
    y[:, 0] = 0.0               # all-zero curve
    y[:, 1] = [5.0, 6.0, 7.0, 8.0]  # growing curve (negative decay rate)
    y[2, 2] = np.nan            # non-finite sample -> exception -> fallback
    acts = [y[t].reshape(3, 4, 5) for t in range(4)]
    tf = TimeCurveFitting(half_life)
    params, auc = tf.fit_time_activity_curve(list(ft), acts)
    g["fit_times"] = ft
    g["fit_acts"] = np.stack(acts)
    g["fit_params"] = params
    g["fit_auc"] = auc
    wts = [1.0, 2.0, 1.0, 0.5]
    params_w, auc_w = tf.fit_time_activity_curve(list(ft), acts, weight_factors=wts)
    g["fit_w"] = np.array(wts)
    g["fit_params_w"] = params_w
    g["fit_auc_w"] = auc_w

    # ---- advanced models on well-posed curves ----
    nv = 24
    t5 = np.array([1.0, 4.0, 24.0, 48.0, 96.0])
    a1 = rng.uniform(0.5, 2.0, nv)
    l1 = rng.uniform(0.01, 0.2, nv)
    ya = a1[None, :] * np.exp(-(l1[None, :] + np.log(2) / half_life) * t5[:, None])
    acts5 = [ya[t].reshape(2, 3, 4) for t in range(5)]
    for mname, model in [("f2", "nukfit"), ("mono-exponential", "lmfit")]:
        p, au = tf.fit_time_activity_curve_advanced(list(t5), acts5, model=model, model_name=mname)
        key = mname.replace("-", "_")
        g[f"adv_{key}_params"] = p
        g[f"adv_{key}_auc"] = au
    g["adv_times"] = t5
    g["adv_acts"] = np.stack(acts5)

    # ---- Y-90 reference kernel generator (NaN at r = 0) ----
    for tissue in ["water", "bone"]:
        kk = Y90KernelGenerator(tissue).generate_kernel(2.0, (15, 15, 15))
        g[f"y90k_{tissue}"] = kk

    # ---- dose-volume histograms (own generator: the vectors above stay as they were) ----
    from pyvoxeldosimetry.core.utils import calculate_dvh
    r2 = np.random.default_rng(233)
    dvh_cases = {
        "f32_bool": ((r2.random((10, 12, 14)) * 40.0).astype(np.float32),
                     r2.random((10, 12, 14)) > 0.4, 50),
        # doses on a 0.25 Gy grid: many values exactly on bin edges
        "f32_ties": ((np.round(r2.random((9, 11, 13)) * 100.0) / 4.0).astype(np.float32),
                     (r2.random((9, 11, 13)) > 0.3).astype(np.uint8), 100),
        "f64_const": (np.full((6, 7, 8), 3.25), r2.random((6, 7, 8)).astype(np.float32) - 0.5, 7),
        "f64_many_bins": (r2.gamma(2.0, 5.0, (16, 16, 16)), r2.random((16, 16, 16)) > 0.1, 20000),
    }
    for name, (dose, mask, nb) in dvh_cases.items():
        e, c = calculate_dvh(dose, mask, bins=nb)
        g[f"dvh_{name}_dose"] = dose
        g[f"dvh_{name}_mask"] = mask
        g[f"dvh_{name}_bins"] = np.array(nb)
        g[f"dvh_{name}_edges"] = e
        g[f"dvh_{name}_cum"] = c

    # ---- kernel generators (configs read with the // comments stripped) ----
    import json
    from pyvoxeldosimetry.data.dose_kernels import base_kernel
    base_kernel.BaseKernelGenerator._load_config = lambda self, path: json.loads(
        strip_json_comments(Path(path).read_text()))
    from pyvoxeldosimetry.data.dose_kernels.ac225_kernel import Ac225KernelGenerator
    from pyvoxeldosimetry.data.dose_kernels.ga68_kernel import Ga68KernelGenerator
    from pyvoxeldosimetry.data.dose_kernels.lu177_kernel import Lu177KernelGenerator
    for tissue in ["water", "bone", "lung"]:
        g[f"kgen_ga68_{tissue}"] = Ga68KernelGenerator(tissue).generate_kernel(2.0, (9, 9, 9))
    for tissue in ["water", "bone"]:
        g[f"kgen_lu177_{tissue}"] = Lu177KernelGenerator(tissue).generate_kernel(1.5, (11, 11, 11))
    r_alpha = np.linspace(0.0, 0.06, 49)
    g["kgen_ac225_r_alpha"] = r_alpha
    c = [s // 2 for s in (7, 7, 7)]
    xx, yy, zz = np.meshgrid(*(np.arange(7) - cc for cc in c), indexing="ij")
    r_gamma = np.sqrt(xx ** 2 + yy ** 2 + zz ** 2) * 1.0
    g["kgen_ac225_r_gamma"] = r_gamma
    for tissue in ["water", "bone", "lung"]:
        ac = Ac225KernelGenerator(tissue)
        g[f"kgen_ac225_alpha_{tissue}"] = np.stack([ac._calculate_alpha_contribution(r_alpha, a["energy"])
                                                   for a in ac.alpha_energies])
        g[f"kgen_ac225_gamma_{tissue}"] = np.stack([ac._calculate_gamma_contribution(r_gamma, gl["energy"],
                                                                                     gl["intensity"])
                                                   for gl in ac.gamma_lines])

    # ---- convolution on shapes with prime factors > 7 (own generator: the vectors above stay) ----
    r3 = np.random.default_rng(1117)
    prime_cases = {
        "prime_small": ((11, 13, 17), (5, 5, 5)),
        "prime_mixed": ((37, 16, 43), (7, 9, 5)),
        "prime_oversize": ((5, 7, 11), (9, 9, 13)),   # kernel truncated to A.shape
        "prime_thin": ((1, 23, 29), (1, 3, 3)),
    }
    for name, (shape, kshape) in prime_cases.items():
        a = r3.random(shape) * 100.0
        k = r3.random(kshape)
        g[f"conv_{name}_A"] = a
        g[f"conv_{name}_K"] = k
        g[f"conv_{name}_D"] = conv_calc(k).calculate_dose_rate(a, (1.0, 1.0, 1.0))

    # ---- tissue composition from HU, with and without the metal-artefact step ----
    from pyvoxeldosimetry.tissue.composition import TissueComposition
    r4 = np.random.default_rng(4242)
    for name, shape in (("odd", (14, 17, 19)), ("thin", (3, 40, 33))):
        ct = np.round(r4.uniform(-1100.0, 3600.0, shape))
        edges = [-1000, -900, -500, -100, 100, 300, 3000, -10, 10, 2000, 2001]
        flat = ct.reshape(-1)
        flat[:len(edges)] = edges                       # values on every range boundary
        flat[len(edges)] = np.nan
        ct[0, :2, :3] = 2500.0                          # metal on the boundary (reflect)
        ct[shape[0] // 2, 5:9, 6:10] = 3200.0           # a metal block
        for art in (True, False):
            comp = TissueComposition().calculate_composition(ct.copy(), handle_artifacts=art)
            for t, m in comp.items():
                g[f"tissue_{name}_{int(art)}_{t}"] = m
        g[f"tissue_{name}_ct"] = ct

    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(g)} arrays)")

    # ---- Monte Carlo decay data as the reference loads it (data/mc_decay/__init__.py:10-24) ----
    from pyvoxeldosimetry.data.mc_decay import load_decay_data
    decay = {n: load_decay_data(n) for n in ("Y90", "Lu177", "I131")}
    DECAY_OUT.write_text(json.dumps(decay, indent=1, sort_keys=True) + "\n")
    print(f"wrote {DECAY_OUT}")


if __name__ == "__main__":
    with tempfile.TemporaryDirectory() as td:
        os.chdir(td)
        main()

"""The Monte Carlo decay data (``load_decay_data``) against the reference's data files
as the reference itself loads them (tests/golden/reference_mc_decay.json, written by
tests/golden/make_golden.py from data/mc_decay/__init__.py:10-24), and the tables the
GPU Monte Carlo and the kernels are built from against that data."""
import json
from pathlib import Path

import numpy as np
import pytest

from pyvoxeldosimetry_gb300.data import mc_decay, mc_physics, nuclides

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "reference_mc_decay.json").read_text())


@pytest.mark.parametrize("nuc", ["Y90", "Lu177", "I131"])
def test_load_decay_data_equals_reference_files(nuc):
    assert mc_decay.load_decay_data(nuc) == GOLDEN[nuc]


def test_unknown_nuclide_raises_like_the_reference():
    with pytest.raises(ValueError, match="Decay data not found for Xx99"):
        mc_decay.load_decay_data("Xx99")


def test_load_returns_a_copy():
    d = mc_decay.load_decay_data("Y90")
    d["half_life"] = 0.0
    assert mc_decay.load_decay_data("Y90")["half_life"] == 64.053


@pytest.mark.parametrize("nuc", ["Y90", "Lu177", "I131"])
def test_monte_carlo_tables_use_the_reference_data(nuc):
    ref = GOLDEN[nuc]
    sp = ref["decay_modes"][0]["spectrum"]
    n = nuclides.get_nuclide(nuc)
    assert list(n.spectrum_e) == sp["spectrum_points"]["energy"]
    assert list(n.spectrum_p) == sp["spectrum_points"]["probability"]
    assert n.beta_mean_mev == sp["mean_energy"] and n.beta_max_mev == sp["max_energy"]
    assert [list(g) for g in n.gammas] == [[g["energy"], g["intensity"]] for g in ref.get("gamma_emissions", [])]
    assert mc_physics.emission_lines(nuc) == [(g["energy"], g["intensity"]) for g in ref.get("gamma_emissions", [])]
    assert n.beta_csda_range_mm == ref["physics_parameters"]["beta_csda_range"]
    if nuc != "Y90":   # Y-90's kernel half-life is the dose-kernel file's 64.1 h
        hours = ref["half_life"] * {"days": 24.0, "hours": 1.0}[ref["half_life_unit"]]
        assert n.half_life_h == pytest.approx(hours, rel=1e-15)
    # the sampled spectrum is the piecewise-linear density through the points
    icdf = mc_physics.beta_inverse_cdf(nuc).astype(np.float64)
    assert icdf[0] == sp["spectrum_points"]["energy"][0] and icdf[-1] == pytest.approx(sp["max_energy"], rel=1e-7)
    assert np.mean(icdf) == pytest.approx(mc_physics.spectrum_mean(nuc), rel=2e-3)

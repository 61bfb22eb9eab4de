"""Closed-form thermodynamics of the sampling model (the reference takes these from its Julia
toolkit, which is not available: parity there is unpinned).  Checked here against finite
differences of the closed-form ln Z, against a one-surface one-mode textbook case, against the
reference's results-file layout and reader semantics, and against the reference's alpha estimator
formulas (stats.py:58-80) on synthetic data."""
import json
import math

import numpy as np
import pytest

from pibronic_gb300 import analytic, constants, synthetic, vibronic_io
from pibronic_gb300.file_structure import FileStructure


def _rho(A=3, N=5, seed=2):
    return synthetic.diagonal_of(synthetic.make_coupled_model(A, N, seed))


@pytest.mark.parametrize("T", [100.0, 300.0, 500.0])
def test_energy_and_heat_capacity_are_derivatives_of_log_z(T):
    rho = _rho()
    b = constants.beta(T)
    th = analytic.thermodynamics(rho, b)
    eps, w = analytic.surface_energies(rho)
    h = 1e-4 * b
    lz = [analytic.log_z(eps, w, b + k * h) for k in (-1, 0, 1)]
    E_fd = -(lz[2] - lz[0]) / (2 * h)
    Cv_fd = constants.boltzman * b ** 2 * (lz[2] - 2 * lz[1] + lz[0]) / h ** 2
    assert math.isclose(th["E_sampling"], E_fd, rel_tol=1e-7)
    assert math.isclose(th["Cv_sampling"], Cv_fd, rel_tol=1e-4)
    assert math.isclose(th["alpha_plus"], th["Z_sampling"] / th["Z_sampling+beta"], rel_tol=1e-12)
    assert math.isclose(th["alpha_minus"], th["Z_sampling"] / th["Z_sampling-beta"], rel_tol=1e-12)
    assert th["Z_rho"] == th["Z_sampling"] and th["E_rho"] == th["E_sampling"]


def test_single_oscillator_textbook():
    """One surface, one mode, no linear term: Z = e^{-b E} / (2 sinh(b w / 2)),
    E = E0 + (w/2) coth(b w / 2), Cv = k_B (b w / 2)^2 csch^2(b w / 2)."""
    VMK = vibronic_io.VMK
    E0, w0 = 0.3, 0.1
    rho = {VMK.N: 1, VMK.A: 1, VMK.E: np.array([E0]), VMK.w: np.array([w0]), VMK.G1: np.zeros((1, 1)),
           VMK.G2: np.zeros((1, 1, 1))}
    b = constants.beta(250.0)
    th = analytic.thermodynamics(rho, b)
    x = 0.5 * b * w0
    assert math.isclose(th["Z_sampling"], math.exp(-b * E0) / (2 * math.sinh(x)), rel_tol=1e-13)
    assert math.isclose(th["E_sampling"], E0 + 0.5 * w0 / math.tanh(x), rel_tol=1e-13)
    assert math.isclose(th["Cv_sampling"], constants.boltzman * (x / math.sinh(x)) ** 2, rel_tol=1e-12)


def test_linear_terms_fold_into_surface_energies():
    VMK = vibronic_io.VMK
    rho = _rho(A=2, N=3)
    eps, w = analytic.surface_energies(rho)
    L = rho[VMK.G1]
    expect = rho[VMK.E] - 0.5 * np.sum(L ** 2 / w[:, None], axis=0)
    assert np.allclose(eps, expect, rtol=1e-14)


def test_results_file_round_trip_and_hash_check(tmp_path):
    FS = FileStructure(str(tmp_path), 0, 0)
    synthetic.write_model_pair(FS, 3, 4, 11)
    b = constants.beta(300.0)
    th = analytic.analytic_of_sampling_model(FS, b)
    analytic.analytic_of_sampling_model(FS, constants.beta(200.0))
    with open(FS.path_analytic_rho) as f:
        d = json.load(f)
    assert set(d) >= {"hash_vib", "hash_rho", "300.00", "200.00"}
    got = analytic.load_analytic_data(FS, 300.0, {})
    assert math.isclose(got["Z"], th["Z_sampling"], rel_tol=1e-15)
    assert math.isclose(got["E"], th["E_sampling"], rel_tol=1e-15)
    assert math.isclose(got["alpha_plus"], th["alpha_plus"], rel_tol=1e-12)
    with pytest.raises(AssertionError):
        analytic.load_analytic_data(FS, 123.0, {})
    # a changed sampling model invalidates the stored results (postprocessing.py:325-326)
    d["hash_rho"] = "stale"
    with open(FS.path_analytic_rho, "w") as f:
        json.dump(d, f)
    with pytest.raises(AssertionError):
        analytic.load_analytic_data(FS, 300.0, {})
    analytic.analytic_of_sampling_model(FS, b)                 # rewritten with the current hashes
    with open(FS.path_analytic_rho) as f:
        d2 = json.load(f)
    assert "200.00" not in d2 and "300.00" in d2


def test_alpha_estimator_terms_match_reference_formulas():
    """calculate_alpha_terms (stats.py:58-80) with the closed-form alphas, on synthetic draws."""
    from oracle import stats_oracle as so
    from pibronic_gb300 import stats
    rng = np.random.default_rng(5)
    X = 4000
    rho = rng.uniform(0.5, 2.0, X)
    g = rho * rng.uniform(0.8, 1.2, X)
    gp, gm = g * (1 - 1e-3), g * (1 + 1e-3)
    th = analytic.thermodynamics(_rho(), constants.beta(300.0))
    args = (constants.delta_beta, rho, g, gp, gm, np.full(X, th["alpha_plus"]), np.full(X, th["alpha_minus"]))
    ours = stats.calculate_alpha_terms(*args)
    ref = so.alpha_terms(*args)
    for a, r in zip(ours, ref):
        assert np.allclose(a, r, rtol=1e-14, atol=0)


def test_statistical_analysis_flows_on_a_result_object():
    """basic / alpha statistical analysis (stats.py:182-216) on a BoxResultPM-like object with the
    analytic data read back from the results file: the alpha form reduces to the basic one when
    alpha_pm = 1, and both add the harmonic contribution."""
    from types import SimpleNamespace
    from oracle import stats_oracle as so
    from pibronic_gb300 import stats
    rng = np.random.default_rng(9)
    X = 5000
    rho = rng.uniform(0.5, 2.0, X)
    g = rho * rng.uniform(0.8, 1.2, X)
    gp, gm = g * rng.uniform(0.99, 1.0, X), g * rng.uniform(1.0, 1.01, X)
    res = SimpleNamespace(scaled_rho=rho, scaled_g=g, scaled_gofr_plus=gp, scaled_gofr_minus=gm, samples=X)
    db = constants.delta_beta
    ana = {"E": 0.25, "Cv": 1e-4, "alpha_plus": 1.0, "alpha_minus": 1.0}
    basic = stats.basic_statistical_analysis(300.0, res, ana, db)
    alpha = stats.alpha_statistical_analysis(300.0, res, ana, db)
    ref = so.estimate_basic(X, 300.0, *so.basic_terms(db, rho, g, gp, gm))
    so.add_harmonic(ref, 0.25, 1e-4)
    for k in ("Z", "E", "Cv"):
        assert np.isclose(basic[k], ref[k], rtol=1e-12), k
        assert np.isclose(alpha[k], basic[k], rtol=1e-9), k

"""The estimator module's API cases as the reference's own stats tests state them
(tests/stats/test_stats.py:46-330, tests/stats/test_jackknife.py:22-57 of the reference), run on
this package's host modules: the same inputs, the same expected values and error messages.

Host logic only: no device is touched."""
import json
import math
import os
import random
import string

import numpy as np
import pytest

from pibronic_gb300 import file_structure, jackknife as jk, stats as st, vibronic_io as vIO
from pibronic_gb300.constants import boltzman
from pibronic_gb300.pimc import BoxResultPM


def random_string(rng, length):
    chars = string.ascii_letters + string.punctuation + string.digits
    return "".join(rng.choice(chars) for _ in range(length))


@pytest.fixture
def rng():
    return random.Random(20181127)


@pytest.fixture
def temp_FS(tmp_path, rng):
    return file_structure.FileStructure(str(tmp_path), id_data=rng.randint(0, 100), id_rho=rng.randint(0, 100))


def test_calculate_basic_property_terms():
    X = 100
    rho, g, g_plus, g_minus = np.ones(X), np.ones(X), np.ones(X) + 1, np.ones(X)
    ret = st.calculate_basic_property_terms(1.0, rho, g, g_plus, g_minus)
    assert np.all(ret[0] == g / rho)
    assert np.all(ret[1] == 0.5)
    assert np.all(ret[2] == 1.0)


def test_calculate_alpha_terms():
    X = 100
    rho, g, g_plus, g_minus = np.ones(X), np.ones(X), np.ones(X) + 1, np.ones(X)
    ret = st.calculate_alpha_terms(1.0, rho, g, g_plus, g_minus, 2.0, 2.0)
    assert np.all(ret[0] == 1.0)
    assert ret[1] == 1.0
    assert ret[2] == 4.0
    assert np.all(ret[3] == 2.0)
    assert ret[4] == 2.0
    assert np.all(ret[5] == 1.0)
    assert ret[6] == 2.0


def test_estimate_basic_properties():
    X, T = 100, 300.0
    ret = st.estimate_basic_properties(X, T, np.ones(X), np.ones(X), np.ones(X) + 1)
    kBT = boltzman * pow(T, 2.0)
    assert ret["Z"] == 1.0 and ret["Z error"] == 0.0
    assert ret["E"] == -1.0 and ret["E error"] == 0.0
    assert ret["Cv"] == 1.0 / kBT and ret["Cv error"] == 0.0


def test_add_harmonic_contribution():
    nums = np.random.default_rng(4).integers(0, 1000, size=4)
    d = {"E": nums[0], "Cv": nums[1]}
    st.add_harmonic_contribution(d, nums[2], nums[3])
    assert d["E"] == nums[0] + nums[2] and d["Cv"] == nums[1] + nums[3]


def test_apply_parameter_restrictions():
    st.apply_parameter_restrictions(None)


def test_estimate_jackknife():
    X, T = 100, 300.0
    kBT = boltzman * pow(T, 2.0)
    ret = jk.estimate_jackknife(X, T, 1.0, {"E": -1.0, "Cv": 1.0 / kBT}, np.ones(X), np.ones(X), np.ones(X) + 1)
    assert ret["E"] == -1.0 and ret["E error"] == 0.0
    assert math.isclose(ret["Cv"], 1.0 / kBT)
    assert math.isclose(ret["Cv error"], 2.7755575615628914e-16)


def test_starmap_wrapper(monkeypatch, temp_FS, rng):
    from pibronic_gb300 import postprocessing
    P, T, X = rng.randint(0, 1000), rng.uniform(5.0, 1000.0), rng.randint(1, int(1e6))

    def load_pimc_one(FS, P, T, pimc_results):
        assert isinstance(pimc_results, BoxResultPM)

    def load_analytical(FS, T, rho_data):
        assert not rho_data and isinstance(rho_data, dict)

    monkeypatch.setattr(postprocessing, "load_pimc_data", load_pimc_one)
    monkeypatch.setattr(postprocessing, "load_analytic_data", load_analytical)

    def stat_op(T, pimc_results, rho_data):
        return {"test": True}

    with pytest.raises(AttributeError) as e_info:
        st.starmap_wrapper(temp_FS, P, T, stat_op)
    assert str(e_info.value) == f"FS {temp_FS:} doesn't have hash_vib or hash_rho attributes!"
    temp_FS.hash_vib = vIO._hash(random_string(rng, 200))
    temp_FS.hash_rho = vIO._hash(random_string(rng, 200))
    with pytest.raises(AssertionError) as e_info:
        st.starmap_wrapper(temp_FS, P, T, stat_op)
    assert str(e_info.value) == "pimc_results has 0 samples! reading the data failed?!"

    def load_pimc_two(FS, P, T, pimc_results):
        pimc_results.samples = X

    monkeypatch.setattr(postprocessing, "load_pimc_data", load_pimc_two)
    st.starmap_wrapper(temp_FS, P, T, stat_op)
    path = temp_FS.template_jackknife.format(P=P, T=T, X=X)
    with open(path, mode="r", encoding="UTF8") as fh:
        data = json.loads(fh.read())
    assert data["test"] is True
    assert data["hash_vib"] == temp_FS.hash_vib and data["hash_rho"] == temp_FS.hash_rho


@pytest.fixture
def pimc_result(rng):
    X = rng.randint(2, 1000)
    res = BoxResultPM(X=X)
    res.scaled_rho = np.array(rng.sample(range(X), k=X), dtype=float)
    res.scaled_g = np.array(rng.sample(range(X), k=X), dtype=float)
    res.scaled_gofr_plus = np.array(rng.sample(range(X), k=X), dtype=float)
    res.scaled_gofr_minus = np.array(rng.sample(range(X), k=X), dtype=float)
    return res


@pytest.mark.parametrize("kind", ["basic", "alpha"])
def test_statistical_analysis_types(monkeypatch, pimc_result, rng, kind):
    T, X = rng.uniform(5.0, 1000.0), pimc_result.samples
    analytic_data = {"E": 1.0, "Cv": 2.0, "alpha_plus": 3.0, "alpha_minus": 4.0}
    test_terms = rng.sample(range(1, 100), k=5 if kind == "basic" else 9)

    def monkey_one(db, *arrays):
        for got, want in zip(arrays, (pimc_result.scaled_rho, pimc_result.scaled_g,
                                      pimc_result.scaled_gofr_plus, pimc_result.scaled_gofr_minus,
                                      analytic_data["alpha_plus"], analytic_data["alpha_minus"])):
            assert np.allclose(got, want)
        return test_terms

    def monkey_two(X_arg, T_arg, *terms):
        assert X_arg == X and T_arg == T
        allowed = test_terms if kind == "basic" else test_terms[:-4]
        assert all(t in allowed for t in terms)
        return {"E": 0.0, "Cv": 0.0}

    name = "calculate_basic_property_terms" if kind == "basic" else "calculate_alpha_terms"
    monkeypatch.setattr(st, name, monkey_one)
    monkeypatch.setattr(st, "estimate_basic_properties", monkey_two)
    op = st.basic_statistical_analysis if kind == "basic" else st.alpha_statistical_analysis
    out = op(T, pimc_result, analytic_data)
    assert out["E"] == analytic_data["E"] and out["Cv"] == analytic_data["Cv"]


def test_statistical_analysis_of_pimc_argument_errors(monkeypatch, temp_FS, rng):
    from pibronic_gb300 import postprocessing
    temp_FS.hash_vib = vIO._hash(random_string(rng, 200))
    temp_FS.hash_rho = vIO._hash(random_string(rng, 200))
    listing = rng.sample(range(1, 100), k=10)
    monkeypatch.setattr(postprocessing, "retrive_pimc_file_list", lambda FS: listing)
    monkeypatch.setattr(postprocessing, "extract_bead_paramater_list", lambda lp: rng.sample(range(1, 100), k=10))
    monkeypatch.setattr(postprocessing, "extract_temperature_paramater_list", lambda lp: rng.sample(range(1, 100), k=10))
    with pytest.raises(Exception) as e_info:
        st.statistical_analysis_of_pimc(temp_FS, method=9)
    assert str(e_info.value) == "Invalid value for parameter method:(9)"
    with pytest.raises(AssertionError) as e_info:
        st.statistical_analysis_of_pimc(temp_FS, location="server")
    assert str(e_info.value) == "Need to write this code"
    with pytest.raises(Exception) as e_info:
        st.statistical_analysis_of_pimc(temp_FS, location=12)
    assert str(e_info.value) == "Invalid value for parameter location:(12)"
    assert not os.listdir(temp_FS.path_rho_results)


def test_alpha_estimators_are_the_basic_ones_on_scaled_g_plus_minus(rng):
    """The identity device_alpha_estimates relies on: the alpha estimates and their jackknife
    equal the basic ones with g(beta +- dbeta) multiplied by alpha_pm (host arrays, reference
    formulas on both sides)."""
    X, T, db = 500, 275.0, 2e-4
    r = np.random.default_rng(9)
    res = BoxResultPM(X=X)
    res.scaled_rho = r.uniform(0.5, 1.5, X)
    res.scaled_g = res.scaled_rho * r.uniform(0.8, 1.2, X)
    res.scaled_gofr_plus = res.scaled_g * (1 - 0.3 * db * r.uniform(0.5, 1.5, X))
    res.scaled_gofr_minus = res.scaled_g * (1 + 0.3 * db * r.uniform(0.5, 1.5, X))
    analytic_data = {"E": 0.25, "Cv": 1e-4, "alpha_plus": 1.00011, "alpha_minus": 0.99987}
    alpha = st.alpha_jackknife_analysis(T, res, analytic_data, db)
    scaled = BoxResultPM(X=X)
    scaled.scaled_rho, scaled.scaled_g = res.scaled_rho, res.scaled_g
    scaled.scaled_gofr_plus = res.scaled_gofr_plus * analytic_data["alpha_plus"]
    scaled.scaled_gofr_minus = res.scaled_gofr_minus * analytic_data["alpha_minus"]
    basic = st.basic_jackknife_analysis(T, scaled, analytic_data, db)
    assert list(alpha) == list(basic)
    # the two sides round differently (alpha+ mean(r+) against mean(alpha+ r+)); E cancels ~1/db
    # and its jackknife ~X on top, so FP64 agreement is ~1e-8 relative, not 1e-16
    for k in alpha:
        assert np.isclose(alpha[k], basic[k], rtol=1e-7, atol=1e-15), (k, alpha[k], basic[k])

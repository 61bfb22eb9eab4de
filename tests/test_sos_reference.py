"""Exact thermodynamics the reference ships with its test data sets (tests/test_models/data_set_{0,1}:
sos_B60.json / sos_B80.json, sum-over-states results written by its Julia toolkit,
julia_wrapper.py:185-197), packed by tests/golden/make_golden.py.

(1) The closed-form sampling-model quantities of analytic.py -- Z, E, Cv and Z(beta +- dbeta), the
    inputs of the reference's estimators (postprocessing.py:313-340) -- against the toolkit's.
(2) The PIMC estimator of the oracle (which the reference runs pin) against the toolkit's exact
    ratio Z_coupled / Z_sampling on the reference's own test models: <g/rho> estimates it.

Host only."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import pimc_oracle as po
from oracle import stats_oracle as so
from pibronic_gb300 import analytic, vibronic_io


@pytest.fixture(scope="module")
def sos():
    with np.load(os.path.join(GOLDEN, "reference_sos_results.npz")) as d:
        return {k: str(d[k]) for k in d.files}


def _entries(sos, sampling):
    names = sorted({k.rsplit("/", 1)[0] for k in sos})
    return [n for n in names if ("rho_" in n) == sampling]


def test_sampling_model_closed_form_matches_sum_over_states(sos, tmp_path):
    entries = _entries(sos, sampling=True)
    assert len(entries) == 5
    for name in entries:
        path = tmp_path / "sampling_model.json"
        path.write_text(sos[name + "/model"])
        rho = vibronic_io.load_diagonal_model_from_JSON(str(path))
        ref = json.loads(sos[name + "/sos"])
        beta = ref["beta"][0]
        got = analytic.thermodynamics(rho, beta)
        for k in ("Z_sampling", "E_sampling", "Z_sampling+beta", "Z_sampling-beta"):
            assert np.isclose(got[k], ref[k][0], rtol=1e-12, atol=0), (name, k)
        # the toolkit's heat capacity carries a finite-difference error of a few 1e-9
        assert np.isclose(got["Cv_sampling"], ref["Cv_sampling"][0], rtol=1e-7, atol=0), name


@pytest.mark.parametrize("data_set,rho_id", [(0, 0), (1, 1)])
def test_pimc_partition_ratio_matches_sum_over_states(sos, data_set, rho_id):
    vib_key = f"data_set_{data_set}/parameters/sos_B80.json"
    rho_key = f"data_set_{data_set}/rho_{rho_id}/parameters/sos_B80.json"
    vib = po.model_from_text(sos[vib_key + "/model"])
    rho = po.model_from_text(sos[rho_key + "/model"], diagonal=True)
    exact = json.loads(sos[vib_key + "/sos"])["Z_coupled"][0] / json.loads(sos[rho_key + "/sos"])["Z_sampling"][0]
    T, X, P, db = 300.0, 4000, 16, 2e-4
    np.random.seed(1000 + 10 * data_set + rho_id)
    box = po.OracleBox(vib, rho, X, 500, P, T, delta_beta=db)
    r = box.block_compute(plus_minus=True)
    est = so.estimate_basic(X, T, *so.basic_terms(db, r["s_rho"], r["s_g"], r["s_gP"], r["s_gM"]))
    # statistical error only: the Trotter error at 16 beads is far below it for these models
    assert abs(est["Z"] - exact) < 4.0 * est["Z error"] + 1e-12, (est["Z"], est["Z error"], exact)

"""The oracle (oracle/pimc_oracle.py) pinned against the reference's own data.

(1) The reference's known-answer test data (tests/pimc/test_pimc_explicit_example.py,
    explicit_data/: A=2, N=2, P=5, T=300 K, X=10), at the reference test's tolerances.
(2) Runs of the reference engine itself on seeded models (tests/golden/make_golden.py): with the
    same numpy seed the oracle must reproduce the reference's q stream and every output.
"""
import numpy as np
import pytest

from oracle import pimc_oracle as po
from oracle import stats_oracle as so

from conftest import case_of

RTOL, ATOL = 1e-05, 1e-08   # test_pimc_explicit_example.py:23-24


@pytest.fixture(scope="module")
def ex_box(explicit):
    vib = po.model_from_text(str(explicit["coupled_model_json"]))
    rho = po.model_from_text(str(explicit["sampling_model_json"]), diagonal=True)
    return po.OracleBox(vib, rho, samples=10, block_size=2, beads=5, temperature=300.0,
                        draw_sources=False)


def test_beta():
    assert np.allclose(po.beta_of(300.0), 38.68174020133669, rtol=RTOL, atol=ATOL)


def test_surface_weights(ex_box, explicit):
    w = explicit["sampling_surface_weights"] / explicit["sampling_surface_weights"].sum()
    assert np.allclose(w, ex_box.rho["state_weight"], rtol=RTOL, atol=ATOL)


def test_means_and_covariance(ex_box, explicit):
    assert np.allclose(explicit["coupled_means"][..., 0], ex_box.vib["state_shift"], rtol=RTOL, atol=ATOL)
    assert np.allclose(explicit["sampling_means"][..., 0], ex_box.rho["state_shift"], rtol=RTOL, atol=ATOL)
    c = ex_box.rho["const"]
    inv = 2.0 * c["coth"][..., None, None] * np.eye(5) - c["csch"][..., None, None] * ex_box.C[None, None]
    assert np.allclose(explicit["sampling_covariance"], np.linalg.inv(inv), rtol=RTOL, atol=ATOL)


def test_energy_and_position_offsets(ex_box, explicit):
    assert np.allclose(explicit["coupled_Edeltas"], ex_box.vib["delta"], rtol=RTOL, atol=ATOL)
    assert np.allclose(explicit["sampling_Edeltas"], ex_box.rho["delta"], rtol=RTOL, atol=ATOL)
    assert np.allclose(explicit["coupled_ds"], ex_box.vib["state_shift"], rtol=RTOL, atol=ATOL)
    assert np.allclose(explicit["sampling_ds"], ex_box.rho["state_shift"], rtol=RTOL, atol=ATOL)


def test_coth_csch(ex_box, explicit):
    for model, pre in ((ex_box.vib, "coupled"), (ex_box.rho, "sampling")):
        cosh, sinh = explicit[pre + "_cosh"], explicit[pre + "_sinh"]
        assert np.allclose(cosh / sinh, model["const"]["coth"], rtol=RTOL, atol=ATOL)
        assert np.allclose(sinh ** -1.0, model["const"]["csch"], rtol=RTOL, atol=ATOL)


def test_explicit_block_compute(ex_box, explicit):
    """Per-block O^rho, O^vib, M, g, rho on the fixed samples (test_pimc_explicit_example.py:168-211)."""
    samples = explicit["samples"]                       # (X, A, N, P)
    g_all, rho_all = np.empty(10), np.empty(10)
    for blk in range(5):
        v = slice(2 * blk, 2 * blk + 2)
        q = samples[v]
        o_rho = po.o_matrix(q, ex_box.rho["state_shift"], ex_box.rho["const"], 2)
        assert np.allclose(o_rho, explicit["rho_oMat"][v], rtol=RTOL, atol=ATOL)
        o_vib = po.o_matrix(q, ex_box.vib["state_shift"], ex_box.vib["const"], 2)
        assert np.allclose(o_vib, explicit["vib_oMat"][v], rtol=RTOL, atol=ATOL)
        rho_all[v] = po.denominator(o_rho)
        M = po.m_matrix(po.coupling_matrix(q, ex_box.vib), ex_box.tau)
        assert np.allclose(M, explicit["vib_mMat"][v], rtol=RTOL, atol=ATOL)
        g_all[v] = po.numerator(M, o_vib)
    assert np.allclose(rho_all, explicit["denominator_rho"], rtol=RTOL, atol=ATOL)
    assert np.allclose(g_all, explicit["numerator_g"], rtol=RTOL, atol=ATOL)


CASES = ["cfg1", "cfg2", "cfg2_cold", "odd", "plain", "arho", "single_surface", "testmodel",
         "cfg4", "a8", "a7", "a12", "a16", "p3_n1", "hot", "frozen", "cfg2_hot", "degen2",
         "degen4", "degen7", "degen12"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_run(runs, name):
    """Same numpy seed -> same sample sources, same q, same scaled outputs as the reference."""
    import json
    c = case_of(runs, name)
    cases = json.load(open(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "cases.json")))
    spec = cases.get(name, dict(P=12, T=300.0, X=40, B=20, rng_seed=242351))
    vib = po.model_from_text(str(c["vib_json"]))
    rho = po.model_from_text(str(c["rho_json"]), diagonal=True)
    pm = "s_gP" in c
    np.random.seed(spec["rng_seed"])
    T = 1.0 / (float(c["beta"]) * po.KB_EV)
    box = po.OracleBox(vib, rho, spec["X"], spec["B"], spec["P"], T,
                       delta_beta=float(c["delta_beta"]) if pm else None)
    assert np.array_equal(box.rho["sample_sources"], c["sample_sources"])
    assert np.allclose(box.rho["state_weight"], c["state_weight"], rtol=1e-13, atol=0)
    res = box.block_compute(plus_minus=pm)
    assert np.allclose(res["q"], c["q"], rtol=1e-12, atol=1e-12)
    keys = ("s_rho", "s_g", "s_gP", "s_gM") if pm else ("s_rho", "s_g")
    for k in keys:
        assert np.allclose(res[k], c[k], rtol=1e-10, atol=0), k


def test_stats_match_reference(runs):
    c = case_of(runs, "cfg1")
    db = float(c["delta_beta"])
    terms = so.basic_terms(db, c["s_rho"], c["s_g"], c["s_gP"], c["s_gM"])
    X = len(c["s_rho"])
    basic = so.estimate_basic(X, 300.0, *terms)
    jk = so.estimate_jackknife(X, 300.0, db, basic, *[so.jackknife_term(X, t) for t in terms])
    for k, v in basic.items():
        assert np.isclose(v, float(runs[f"stats/basic/{k}"]), rtol=1e-12, atol=0), k
    for k, v in jk.items():
        assert np.isclose(v, float(runs[f"stats/jk/{k}"]), rtol=1e-9, atol=0), k


def test_ml_data_path_matches_reference(runs):
    c = case_of(runs, "ml")
    vib = po.model_from_text(str(c["vib_json"]))
    rho = po.model_from_text(str(c["rho_json"]), diagonal=True)
    box = po.OracleBox(vib, rho, 30, 15, 8, 300.0, draw_sources=False)
    assert np.allclose(box.g_of_R(c["R"]), c["g"], rtol=1e-10, atol=0)
    assert np.allclose(box.rho_of_R(c["R"]), c["rho"], rtol=1e-10, atol=0)

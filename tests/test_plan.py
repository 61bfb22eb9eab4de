"""Host precompute (pibronic_gb300.plan) and the kernel's formulation, checked on the CPU.

kernel_model.evaluate runs the fused kernel's arithmetic in FP64 numpy on the plan's tables; it
must agree with the oracle on the reference's own q (golden runs)."""
import math

import numpy as np
import pytest

from pibronic_gb300 import plan as pl

from conftest import case_of, oracle_box_from_case, prepared_from_case
import kernel_model


def test_series_against_direct_evaluation():
    w, beta, P, K = np.array([0.02, 0.11, 0.3]), 38.7, 64, 4
    cs, th, ls = pl.harmonic_series(w, beta, P, K)
    for h in (-3e-3, 1e-3, 4e-3):
        x = w * (beta + h) / P
        hp = h ** np.arange(K + 1)
        assert np.allclose(cs @ hp, 1 / np.sinh(x), rtol=1e-12)
        assert np.allclose(th @ hp, np.tanh(x / 2), rtol=1e-12)
        assert np.allclose(ls @ hp, np.log(np.sinh(x)), rtol=1e-12)


def test_ring_basis_is_orthonormal_eigenbasis():
    for P in (3, 4, 5, 12, 64, 65):
        B = pl.ring_mode_basis(P)
        lam = pl.ring_mode_eigenvalues(P)
        C = np.zeros((P, P))
        for p in range(P):
            C[p, (p + 1) % P] = C[p, (p - 1) % P] = 1.0
        assert np.allclose(B.T @ B, np.eye(P), atol=1e-12)
        assert np.allclose(C @ B, B * lam[None, :], atol=1e-12)
        assert np.allclose(np.sort(lam), np.sort(np.linalg.eigvalsh(C)), atol=1e-12)


@pytest.mark.parametrize("name", ["cfg1", "cfg2", "cfg2_cold", "odd", "plain", "arho",
                                  "single_surface", "testmodel", "cfg4", "a8", "a7", "p3_n1",
                                  "hot", "frozen"])
def test_kernel_formulation_matches_oracle(runs, name):
    c = case_of(runs, name)
    q = c["q"]
    P = q.shape[2]
    box = oracle_box_from_case(c, P)
    ref = box.evaluate(q, plus_minus="s_gP" in c)
    prep = prepared_from_case(c, P)
    got = kernel_model.evaluate(prep, q)
    assert np.allclose(got["s_rho"], ref["rho"], rtol=1e-9, atol=0)
    assert np.allclose(got["s_g"], ref["g"], rtol=1e-9, atol=0)
    assert np.allclose(got["s_rho"], c["s_rho"], rtol=1e-9, atol=0)
    assert np.allclose(got["s_g"], c["s_g"], rtol=1e-9, atol=0)
    if "s_gP" in c:
        assert np.allclose(got["s_gp"], c["s_gP"], rtol=1e-9, atol=0)
        assert np.allclose(got["s_gm"], c["s_gM"], rtol=1e-9, atol=0)
        # finite-difference terms the estimators use (stats.py:38-55)
        db = float(c["delta_beta"])
        d1_ref = (c["s_gP"] - c["s_gM"]) / (2 * db * c["s_rho"])
        d1 = (got["s_gp"] - got["s_gm"]) / (2 * db * got["s_rho"])
        assert np.allclose(d1, d1_ref, rtol=1e-6, atol=0)
        d2_ref = (c["s_gP"] - 2 * c["s_g"] + c["s_gM"]) / (db ** 2 * c["s_rho"])
        d2 = (got["s_gp"] - 2 * got["s_g"] + got["s_gm"]) / (db ** 2 * got["s_rho"])
        assert np.allclose(d2, d2_ref, rtol=1e-4, atol=1e-6 * np.abs(d2_ref).max())

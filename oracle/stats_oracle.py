"""FP64 numpy restatement of Pibronic's estimators (Z, E, Cv and the jackknife).

TEST INFRASTRUCTURE ONLY: the checker for ``pibronic_gb300.stats`` and the device reduction.
Follows ``pibronic/stats/stats.py:38-130`` and ``pibronic/stats/jackknife.py:14-105``.
"""
from __future__ import annotations

import numpy as np

from .pimc_oracle import KB_EV


def basic_terms(delta_beta, rho, g, g_plus, g_minus):
    """g/rho, (g+ - g-)/(2 db rho), (g+ - 2g + g-)/(db^2 rho) (stats.py:38-55)."""
    ratio = g / rho
    d1 = (g_plus - g_minus) / rho / (2.0 * delta_beta)
    d2 = (g_plus - 2.0 * g + g_minus) / rho / delta_beta ** 2
    return [ratio, d1, d2]


def alpha_terms(delta_beta, rho, g, g_plus, g_minus, alpha_plus, alpha_minus):
    """Difference form with alpha+- = Z_rho / Z_rho(beta +- db) (stats.py:58-81)."""
    ratio, rp, rm = g / rho, g_plus / rho, g_minus / rho
    d1 = (np.mean(rp) * np.mean(alpha_plus) - np.mean(rm) * np.mean(alpha_minus)) / (2.0 * delta_beta)
    d2 = (np.mean(rp) * np.mean(alpha_plus) - 2.0 * np.mean(ratio)
          + np.mean(rm) * np.mean(alpha_minus)) / delta_beta ** 2
    return [ratio, d1, d2, rp, alpha_plus, rm, alpha_minus]


def estimate_basic(X, T, g_r, sym1, sym2):
    """Z = mean(g/rho), its error std/sqrt(X-1); E = -mean(sym1)/Z; Cv = (mean(sym2)/Z - E^2)/(kB T^2)
    (stats.py:84-123)."""
    Z = np.mean(g_r)
    Z_err = np.std(g_r, ddof=0) / np.sqrt(X - 1)
    E = -1.0 * np.mean(sym1) / np.mean(Z)
    Cv = (np.mean(sym2) / np.mean(Z) - E ** 2) / (KB_EV * T ** 2)
    return {"Z": Z, "Z error": Z_err, "E": E, "E error": 0.0, "Cv": Cv, "Cv error": 0.0}


def add_harmonic(d, E_sampling, Cv_sampling):
    """stats.py:126-130."""
    d["E"] += E_sampling
    d["Cv"] += Cv_sampling


def jackknife_term(X, arr):
    """(sum - x_i) / (X - 1) (jackknife.py:60-70)."""
    return (np.full(X, np.sum(arr)) - arr) / (X - 1)


def alpha_jackknife_terms(X, delta_beta, ratio, LN, alpha_plus, RN, alpha_minus):
    """jackknife.py:14-57."""
    jr, jl, jm = (jackknife_term(X, a) for a in (ratio, LN, RN))
    d1 = (jl * alpha_plus - jm * alpha_minus) / (2.0 * delta_beta)
    d2 = (jl * alpha_plus - 2.0 * jr + jm * alpha_minus) / delta_beta ** 2
    return [jr, d1, d2]


def estimate_jackknife(X, T, delta_beta, input_dict, jk_g_rho, jk_sym1, jk_sym2):
    """jackknife.py:77-105."""
    f_E = -1.0 * jk_sym1 / jk_g_rho
    E = X * input_dict["E"] - (X - 1.0) * np.mean(f_E)
    E_err = np.sqrt(X - 1.0) * np.std(f_E, ddof=1)
    f_C = (jk_sym2 / jk_g_rho - f_E ** 2) / (KB_EV * T ** 2)
    Cv = X * input_dict["Cv"] - (X - 1.0) * np.mean(f_C)
    Cv_err = np.sqrt(X - 1.0) * np.std(f_C, ddof=1)
    return {"E": E, "E error": E_err, "Cv": Cv, "Cv error": Cv_err}


def basic_jackknife(T, delta_beta, rho, g, gp, gm, E_sampling=0.0, Cv_sampling=0.0):
    """stats.py:271-301 without the file layer."""
    X = rho.shape[0]
    terms = basic_terms(delta_beta, rho, g, gp, gm)
    jk = [jackknife_term(X, t) for t in terms]
    basic = estimate_basic(X, T, *terms)
    jkd = estimate_jackknife(X, T, delta_beta, basic, *jk)
    add_harmonic(basic, E_sampling, Cv_sampling)
    add_harmonic(jkd, E_sampling, Cv_sampling)
    out = dict(basic)
    out.update({"jk_" + k: v for k, v in jkd.items()})
    return out

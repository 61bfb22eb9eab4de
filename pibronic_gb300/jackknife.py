"""Jackknife estimators (pibronic/stats/jackknife.py:14-105), host FP64, reference signatures."""
import numpy as np

from .constants import boltzman


def calculate_alpha_jackknife_terms(*args):
    """Leave-one-out ratio and alpha-form symmetric derivatives (jackknife.py:14-57)."""
    X, delta_beta, ratio, LN, alpha_plus, RN, alpha_minus = args
    jk_ratio = (np.full(X, np.sum(ratio)) - ratio) / (X - 1)
    jk_LN = (np.full(X, np.sum(LN)) - LN) / (X - 1)
    jk_RN = (np.full(X, np.sum(RN)) - RN) / (X - 1)
    d1 = (jk_LN * alpha_plus - jk_RN * alpha_minus) / (2.0 * delta_beta)
    d2 = (jk_LN * alpha_plus - 2.0 * jk_ratio + jk_RN * alpha_minus) / pow(delta_beta, 2)
    return [jk_ratio, d1, d2]


def calculate_jackknife_term(length, array):
    """(sum - x_i) / (X - 1) (jackknife.py:60-70)."""
    return (np.full(length, np.sum(array)) - array) / (length - 1)


def calculate_jackknife_terms(length, list_of_arrays):
    return [calculate_jackknife_term(length, a) for a in list_of_arrays]


def estimate_jackknife(*args):
    """Jackknife E, Cv and their errors (jackknife.py:77-105)."""
    X, T, delta_beta, input_dict, jk_g_rho, jk_sym1, jk_sym2 = args
    f_EJ = -1.0 * jk_sym1 / jk_g_rho
    E = X * input_dict["E"] - (X - 1.0) * np.mean(f_EJ)
    E_err = np.sqrt(X - 1.0) * np.std(f_EJ, ddof=1)
    f_CJ = (jk_sym2 / jk_g_rho - pow(f_EJ, 2.0)) / (boltzman * pow(T, 2.0))
    Cv = X * input_dict["Cv"] - (X - 1.0) * np.mean(f_CJ)
    Cv_err = np.sqrt(X - 1.0) * np.std(f_CJ, ddof=1)
    return {"E": E, "E error": E_err, "Cv": Cv, "Cv error": Cv_err}

"""Closed-form thermodynamics of the sampling model rho (the quantities the reference obtains from
its Julia toolkit: julia_wrapper.py:185-197 writes them, postprocessing.py:313-340 reads them).

rho is diagonal and harmonic: surface a has the energy eps_a = E_aa + Delta_a (Delta_a =
-1/2 sum_j L_jaa^2 / w_j, the linear terms folded in, pimc.py:172-177) and the modes w_j, so

    Z(beta)   = sum_a exp(-beta eps_a) prod_j 1 / (2 sinh(beta w_j / 2))
    E         = -d ln Z / d beta = <eps>_beta + sum_j (w_j / 2) coth(beta w_j / 2)
    Cv        = k_B beta^2 d^2 ln Z / d beta^2
              = k_B beta^2 [ Var_beta(eps) + sum_j (w_j / 2)^2 csch^2(beta w_j / 2) ]

with <.>_beta and Var_beta over the Boltzmann weights of the surfaces.  Everything in FP64 with a
log-sum-exp over surfaces.  alpha_plus / alpha_minus = Z(beta) / Z(beta +- dbeta) are the factors of
the reference's alpha estimator (stats.py:58-80).

The results file keeps the reference's layout: a JSON object with "hash_vib", "hash_rho" and one
entry per temperature "T.2f" holding both key families the reference uses (julia_wrapper.py:25-52
writes Z_rho / E_rho / Cv_rho; postprocessing.py:330-335 reads Z_sampling / E_sampling /
Cv_sampling / Z_sampling+beta / Z_sampling-beta).
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import constants
from . import vibronic_io as vIO
from .vibronic_io import VMK

__all__ = ["surface_energies", "log_z", "thermodynamics", "analytic_of_sampling_model", "load_analytic_data"]


def surface_energies(rho_model):
    """(eps_a, w_j) of a diagonal sampling model dict (vibronic_io keys)."""
    w = np.asarray(rho_model[VMK.w], dtype=np.float64)
    E = np.asarray(rho_model[VMK.E], dtype=np.float64)
    E = np.diagonal(E).copy() if E.ndim == 2 else E.copy()
    L = np.asarray(rho_model[VMK.G1], dtype=np.float64)
    if L.ndim == 3:
        L = np.diagonal(L, axis1=1, axis2=2)
    delta = -0.5 * np.einsum("ja,j->a", L ** 2, 1.0 / w)
    return E + delta, w


def log_z(eps, w, beta):
    """ln Z(beta) of the harmonic sampling model."""
    x = -beta * eps
    m = x.max()
    return m + np.log(np.exp(x - m).sum()) - np.sum(np.log(2.0 * np.sinh(0.5 * beta * w)))


def thermodynamics(rho_model, beta, delta_beta=constants.delta_beta):
    """Z, E, Cv of rho at beta and Z at beta +- delta_beta (dict, the reference's key names)."""
    eps, w = surface_energies(rho_model)
    x = -beta * eps
    p = np.exp(x - x.max())
    p /= p.sum()
    mean_eps = float(np.dot(p, eps))
    var_eps = float(np.dot(p, (eps - mean_eps) ** 2))
    hw = 0.5 * w
    arg = beta * hw
    E = mean_eps + float(np.sum(hw / np.tanh(arg)))
    d2 = var_eps + float(np.sum((hw / np.sinh(arg)) ** 2))
    Cv = constants.boltzman * beta ** 2 * d2
    lz = log_z(eps, w, beta)
    lzp, lzm = log_z(eps, w, beta + delta_beta), log_z(eps, w, beta - delta_beta)
    out = {"beta": beta, "Z_sampling": float(np.exp(lz)), "E_sampling": E, "Cv_sampling": Cv,
           "Z_sampling+beta": float(np.exp(lzp)), "Z_sampling-beta": float(np.exp(lzm)),
           "alpha_plus": float(np.exp(lz - lzp)), "alpha_minus": float(np.exp(lz - lzm)),
           "delta_beta": delta_beta}
    out.update({"Z_rho": out["Z_sampling"], "E_rho": E, "Cv_rho": Cv})
    return out


def analytic_of_sampling_model(FS, beta, delta_beta=constants.delta_beta):
    """Add the closed-form results at beta to FS.path_analytic_rho (kept, or replaced when the
    stored hashes do not match the model files) -- the file the reference's Julia run writes."""
    rho_model = vIO.load_diagonal_model_from_JSON(FS.path_rho_model)
    FS.generate_model_hashes()
    old = {}
    if os.path.isfile(FS.path_analytic_rho):
        with open(FS.path_analytic_rho) as f:
            text = f.read()
        if len(text) > 1:
            old = json.loads(text)
    if old.get("hash_vib") != FS.hash_vib or old.get("hash_rho") != FS.hash_rho:
        old = {}
    old["hash_vib"], old["hash_rho"] = FS.hash_vib, FS.hash_rho
    T = constants.extract_T_from_beta(beta)
    old[f"{T:.2f}"] = thermodynamics(rho_model, beta, delta_beta)
    os.makedirs(os.path.dirname(FS.path_analytic_rho), exist_ok=True)
    with open(FS.path_analytic_rho, "w") as f:
        json.dump(old, f)
    return old[f"{T:.2f}"]


def load_analytic_data(FS, T, analytic):
    """Fill `analytic` with Z, E, Cv, alpha_plus, alpha_minus at temperature T from the results
    file, checking the model hashes (postprocessing.py:313-340); AssertionError as there."""
    path = FS.path_analytic_rho
    assert os.path.isfile(path), f"This file doesn't exist:\n{path:s}"
    with open(path) as f:
        in_dict = json.loads(f.read())
    FS.generate_model_hashes()
    assert in_dict["hash_vib"] == FS.hash_vib, "wrong vib hash"
    assert in_dict["hash_rho"] == FS.hash_rho, "wrong rho hash"
    key = f"{T:.2f}"
    assert key in in_dict, f"no analytical results for temperature {key:s} in file {path:s}"
    d = in_dict[key]
    analytic["Z"] = d["Z_sampling"]
    analytic["E"] = d["E_sampling"]
    analytic["Cv"] = d["Cv_sampling"]
    analytic["alpha_plus"] = analytic["Z"] / d["Z_sampling+beta"]
    analytic["alpha_minus"] = analytic["Z"] / d["Z_sampling-beta"]
    return analytic

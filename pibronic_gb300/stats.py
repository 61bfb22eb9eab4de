"""Estimators of Z, E, Cv: the reference's functions (pibronic/stats/stats.py:38-333) on host FP64
arrays, plus the device path that reduces the per-sample outputs on the GPU.

Device path: ``device_estimates(rho, g, gp, gm, T, delta_beta)`` takes CUDA tensors (the
``result.device`` arrays block_compute_pm leaves behind) and runs two FP64 reduction kernels:
the moments of r = g/rho, s1, s2 (pbr_reduce_terms) and the jackknife pass over the leave-one-out
estimators (pbr_reduce_jackknife).  Only a handful of doubles come back to the host.
"""
from __future__ import annotations

import json
import math

import numpy as np

from . import _native
from . import constants
from . import jackknife as jk
from .constants import boltzman

__all__ = ["calculate_alpha_terms", "add_harmonic_contribution", "estimate_basic_properties",
           "calculate_basic_property_terms", "basic_statistical_analysis", "alpha_statistical_analysis",
           "basic_jackknife_analysis", "alpha_jackknife_analysis", "statistical_analysis_of_pimc",
           "jackknife_analysis_of_pimc", "device_estimates", "device_alpha_estimates", "ess"]


def calculate_basic_property_terms(*args):
    """g/rho, (g+ - g-)/(2 db rho), (g+ - 2g + g-)/(db^2 rho) (stats.py:38-55)."""
    delta_beta, rho, g, g_plus, g_minus = args
    ratio = g / rho
    d1 = (g_plus - g_minus) / rho / (2.0 * delta_beta)
    d2 = (g_plus - (2.0 * g) + g_minus) / rho / pow(delta_beta, 2)
    return [ratio, d1, d2]


def calculate_alpha_terms(*args):
    """stats.py:58-81."""
    delta_beta, rho, g, g_plus, g_minus, alpha_plus, alpha_minus = args
    ratio, rp, rm = g / rho, g_plus / rho, g_minus / rho
    d1 = (np.mean(rp) * np.mean(alpha_plus) - np.mean(rm) * np.mean(alpha_minus)) / (2.0 * delta_beta)
    d2 = (np.mean(rp) * np.mean(alpha_plus) - 2.0 * np.mean(ratio)
          + np.mean(rm) * np.mean(alpha_minus)) / pow(delta_beta, 2)
    return [ratio, d1, d2, rp, alpha_plus, rm, alpha_minus]


def basic_estimate_Z_monte_carlo(g_over_rho, number_of_samples):
    Z = np.mean(g_over_rho)
    return Z, np.std(g_over_rho, ddof=0) / np.sqrt(number_of_samples - 1)


def basic_estimate_internal_energy(first_symmetric_derivative, Z_MC):
    return -1.0 * np.mean(first_symmetric_derivative) / np.mean(Z_MC), 0.0


def basic_estimate_heat_capacity(second_symmetric_derivative, Z_MC, internal_energy, temperature):
    Cv = (np.mean(second_symmetric_derivative) / np.mean(Z_MC) - pow(internal_energy, 2.0))
    return Cv / (boltzman * pow(temperature, 2.0)), 0.0


def estimate_basic_properties(*args):
    """Z, E, Cv and errors (stats.py:109-123)."""
    X, T, g_r, sym1, sym2 = args
    Z, Z_err = basic_estimate_Z_monte_carlo(g_r, X)
    E, E_err = basic_estimate_internal_energy(sym1, Z)
    Cv, Cv_err = basic_estimate_heat_capacity(sym2, Z, E, T)
    return {"Z": Z, "Z error": Z_err, "E": E, "E error": E_err, "Cv": Cv, "Cv error": Cv_err}


def add_harmonic_contribution(input_dict, E_sampling, Cv_sampling):
    """stats.py:126-130."""
    input_dict["E"] += E_sampling
    input_dict["Cv"] += Cv_sampling


def _result_arrays(pimc_result):
    return [pimc_result.scaled_rho, pimc_result.scaled_g, pimc_result.scaled_gofr_plus,
            pimc_result.scaled_gofr_minus]


def basic_statistical_analysis(temperature, pimc_result, analytic_data, delta_beta=constants.delta_beta):
    """stats.py:182-196: Z, E, Cv from a BoxResultPM and the sampling model's analytic data (as
    written by analytic.analytic_of_sampling_model and read by analytic.load_analytic_data)."""
    terms = calculate_basic_property_terms(delta_beta, *_result_arrays(pimc_result))
    out = estimate_basic_properties(pimc_result.samples, temperature, *terms)
    add_harmonic_contribution(out, analytic_data["E"], analytic_data["Cv"])
    return out


def alpha_statistical_analysis(temperature, pimc_result, analytic_data, delta_beta=constants.delta_beta):
    """stats.py:199-216: the alpha estimator, g(beta +- dbeta) / rho weighted by the closed-form
    alpha_pm = Z_rho(beta) / Z_rho(beta +- dbeta) of the sampling model."""
    terms = calculate_alpha_terms(delta_beta, *_result_arrays(pimc_result), analytic_data["alpha_plus"],
                                  analytic_data["alpha_minus"])
    out = estimate_basic_properties(pimc_result.samples, temperature, *terms[:-4])
    add_harmonic_contribution(out, analytic_data["E"], analytic_data["Cv"])
    return out


def _with_jackknife(basic, jkd, analytic_data):
    add_harmonic_contribution(basic, analytic_data["E"], analytic_data["Cv"])
    add_harmonic_contribution(jkd, analytic_data["E"], analytic_data["Cv"])
    out = dict(basic)
    out.update({"jk_" + k: v for k, v in jkd.items()})
    return out


def basic_jackknife_analysis(temperature, pimc_result, analytic_data, delta_beta=constants.delta_beta):
    """stats.py:271-299: the basic estimates plus their jackknife ("jk_" keys).  The reference
    always uses the module constant delta_beta; a run made with another step passes its own."""
    X = pimc_result.samples
    terms = calculate_basic_property_terms(delta_beta, *_result_arrays(pimc_result))
    jk_terms = jk.calculate_jackknife_terms(X, terms)
    basic = estimate_basic_properties(X, temperature, *terms)
    jkd = jk.estimate_jackknife(X, temperature, delta_beta, basic, *jk_terms)
    return _with_jackknife(basic, jkd, analytic_data)


def alpha_jackknife_analysis(temperature, pimc_result, analytic_data, delta_beta=constants.delta_beta):
    """stats.py:302-333: the alpha estimates plus their jackknife, whose leave-one-out terms weight
    g(beta +- dbeta) / rho by the closed-form alpha_pm (jackknife.py:14-57)."""
    X = pimc_result.samples
    terms = calculate_alpha_terms(delta_beta, *_result_arrays(pimc_result), analytic_data["alpha_plus"],
                                  analytic_data["alpha_minus"])
    jk_terms = jk.calculate_alpha_jackknife_terms(X, delta_beta, terms[0], *terms[3:7])
    alpha = estimate_basic_properties(X, temperature, *terms[:-4])
    jkd = jk.estimate_jackknife(X, temperature, delta_beta, alpha, *jk_terms)
    return _with_jackknife(alpha, jkd, analytic_data)


def apply_parameter_restrictions(args):
    """A placeholder of the reference that leaves the (P, T) lists unchanged (stats.py:133-145)."""
    return


# ---------------------------------------------------------------------------------------------
# file-driven analyses (one *_thermo file per (P, T) found among the data set's result files)
# ---------------------------------------------------------------------------------------------
def starmap_wrapper(FS, P, T, statistical_operation):
    """Merge every job's results at (P, T), read the analytic data at T, run the operation and
    write its dict with the model hashes to P{P}_T{T:.2f}_X{X}_thermo (stats.py:148-179)."""
    from . import postprocessing as pp
    from .pimc import BoxResultPM
    pimc_results = BoxResultPM()
    rho_data = {}
    pp.load_pimc_data(FS, P, T, pimc_results)
    pp.load_analytic_data(FS, T, rho_data)
    out = statistical_operation(T, pimc_results, rho_data)
    if not (hasattr(FS, "hash_vib") and hasattr(FS, "hash_rho")):
        raise AttributeError(f"FS {FS} doesn't have hash_vib or hash_rho attributes!")
    out["hash_vib"], out["hash_rho"] = FS.hash_vib, FS.hash_rho
    assert pimc_results.samples != 0, "pimc_results has 0 samples! reading the data failed?!"
    path = FS.template_jackknife.format(P=P, T=T, X=int(pimc_results.samples))
    with open(path, mode="w", encoding="UTF8") as fh:
        fh.write(json.dumps({k: (float(v) if isinstance(v, (np.floating, float)) else v)
                             for k, v in out.items()}))
    return path


_OPERATIONS = {("basic", False): basic_statistical_analysis, ("alpha", False): alpha_statistical_analysis,
               ("basic", True): basic_jackknife_analysis, ("alpha", True): alpha_jackknife_analysis}


def _analysis_of_pimc(FS, method, location, jackknife):
    from . import postprocessing as pp
    FS.generate_model_hashes()
    list_pimc = pp.retrive_pimc_file_list(FS)
    args = {"pimc_beads": pp.extract_bead_paramater_list(list_pimc),
            "temperatures": pp.extract_temperature_paramater_list(list_pimc)}
    apply_parameter_restrictions(args)
    beads, temperatures = args["pimc_beads"], args["temperatures"]
    operation = _OPERATIONS.get((method, jackknife))
    if operation is None:
        raise Exception(f"Invalid value for parameter method:({method})")
    if location == "server":
        raise AssertionError("Need to write this code")
    if location != "local":
        raise Exception(f"Invalid value for parameter location:({location})")
    return [starmap_wrapper(FS, P, T, operation) for P in beads for T in temperatures]


def statistical_analysis_of_pimc(FS, method="basic", location="local", samples=None):
    """Z, E, Cv ("basic" or "alpha" estimator) for every (P, T) of the data set's result files,
    one *_thermo file each (stats.py:219-265).  The reference runs the (P, T) pairs in a pool of 12
    processes; here they run in turn (each is a pass over host arrays); returns the written paths.
    `samples` is accepted and unused, as in the reference."""
    return _analysis_of_pimc(FS, method, location, jackknife=False)


def jackknife_analysis_of_pimc(FS, method="basic", location="local", samples=None):
    """As statistical_analysis_of_pimc with the jackknife estimates added (stats.py:336-377)."""
    return _analysis_of_pimc(FS, method, location, jackknife=True)


# ---------------------------------------------------------------------------------------------
# device path
# ---------------------------------------------------------------------------------------------
class DeviceReducer:
    """Preallocated scratch for the reduction kernels of X samples (no allocation per call)."""

    def __init__(self, X):
        torch = _native.require_cuda()
        lib = _native.load()
        nb = int(lib.pbr_reduce_blocks(int(X)))
        self.X = X
        self.scratch = torch.empty(nb * 9, dtype=torch.float64, device="cuda")
        self.moments = torch.empty(7, dtype=torch.float64, device="cuda")
        self.jk = torch.empty(5, dtype=torch.float64, device="cuda")
        self.totals = torch.empty(3, dtype=torch.float64, device="cuda")

    def launch(self, rho, g, gp, gm, delta_beta, temperature, stream=None):
        """Queue both passes on the stream (nothing is read back)."""
        self.launch_terms(rho, g, gp, gm, delta_beta, stream)
        if gp is None:
            return 3
        # totals S_r, S_1, S_2 = n * mean, computed on the device without a host round trip
        self.totals.copy_(self.moments[[1, 3, 5]] * self.moments[0])
        self.launch_jackknife(rho, g, gp, gm, delta_beta, temperature, stream)
        return 5

    def launch_terms(self, rho, g, gp, gm, delta_beta, stream=None):
        """First pass: moments of r, s1, s2 over these samples into self.moments."""
        lib = _native.load()
        p = _native.ptr
        _native.check(lib.pbr_reduce_terms(p(rho), p(g), p(gp), p(gm), self.X, float(delta_beta),
                                           p(self.scratch), p(self.moments), _native.stream_handle(stream)),
                      "reduce_terms")

    def launch_jackknife(self, rho, g, gp, gm, delta_beta, temperature, stream=None):
        """Second pass over these samples against the totals in self.totals (which may be the
        totals of a larger sample set, e.g. all ranks' samples) into self.jk."""
        lib = _native.load()
        p = _native.ptr
        kT2 = boltzman * temperature ** 2
        _native.check(lib.pbr_reduce_jackknife(p(rho), p(g), p(gp), p(gm), self.X, float(delta_beta),
                                               float(kT2), p(self.totals), p(self.scratch),
                                               p(self.jk), _native.stream_handle(stream)), "reduce_jackknife")

    def pooled(self, rho, g, gp, gm, delta_beta, temperature, group=None, stream=None):
        """Both passes with the estimates and the jackknife taken over every rank's samples
        (torch.distributed): see shard.pooled_moments.  Returns the estimates dict."""
        from .shard import pooled_moments
        torch = _native.require_cuda()

        def pass1():
            self.launch_terms(rho, g, gp, gm, delta_beta, stream)
            return self.moments.cpu().numpy()

        def pass2(totals):
            self.totals.copy_(torch.as_tensor(totals, dtype=torch.float64))
            self.launch_jackknife(rho, g, gp, gm, delta_beta, temperature, stream)
            return self.jk.cpu().numpy()
        m, j = pooled_moments(pass1, pass2, group)
        return estimates_from_moments(m, j, temperature)

    def read(self, temperature):
        m = self.moments.cpu().numpy()
        j = self.jk.cpu().numpy()
        return estimates_from_moments(m, j, temperature)


def estimates_from_moments(m, j, temperature):
    """Z, E, Cv (basic, stats.py:84-123) and the jackknife E, Cv with errors (jackknife.py:77-105)
    from the device moments; also the effective sample size (sum r)^2 / sum r^2."""
    n, mr, m2r, m1, _, m2, _ = (float(x) for x in m)
    Z = mr
    Z_err = math.sqrt(max(m2r, 0.0) / n) / math.sqrt(n - 1)
    E = -m1 / Z
    Cv = (m2 / Z - E * E) / (boltzman * temperature ** 2)
    out = {"X": n, "Z": Z, "Z error": Z_err, "E": E, "E error": 0.0, "Cv": Cv, "Cv error": 0.0,
           "ESS": (n * mr) ** 2 / (m2r + n * mr * mr)}
    if j is not None and len(j) == 5 and n > 1:
        _, mdE, m2dE, mdC, m2dC = (float(x) for x in j)
        # f_i = E0 + dE_i; jackknife E = X E - (X-1) mean f = E0 - (X-1) mean dE
        out["jk_E"] = E - (n - 1.0) * mdE
        out["jk_E error"] = math.sqrt(n - 1.0) * math.sqrt(max(m2dE, 0.0) / (n - 1.0))
        out["jk_Cv"] = Cv - (n - 1.0) * mdC
        out["jk_Cv error"] = math.sqrt(n - 1.0) * math.sqrt(max(m2dC, 0.0) / (n - 1.0))
    return out


def device_estimates(rho, g, gp, gm, temperature, delta_beta):
    """Z, E, Cv, jackknife errors and ESS from CUDA tensors of per-sample outputs."""
    red = DeviceReducer(rho.shape[0])
    red.launch(rho, g, gp, gm, delta_beta, temperature)
    return red.read(temperature)


def device_alpha_estimates(rho, g, gp, gm, temperature, delta_beta, alpha_plus, alpha_minus):
    """The alpha estimator and its jackknife (stats.py:58-81, 302-333; jackknife.py:14-57) from
    CUDA tensors.  Its terms are the basic ones with g(beta +- dbeta) scaled by the constants
    alpha_pm: (alpha+ g+ - alpha- g-) / (2 db rho) and (alpha+ g+ - 2 g + alpha- g-) / (db^2 rho),
    and a leave-one-out mean of such a linear combination is the combination of the leave-one-out
    means.  So the basic reduction kernels run on (rho, g, alpha+ g+, alpha- g-)."""
    return device_estimates(rho, g, gp * float(alpha_plus), gm * float(alpha_minus), temperature,
                            delta_beta)


def ess(weights):
    """Effective sample size (sum w)^2 / sum w^2 (host)."""
    w = np.asarray(weights, dtype=np.float64)
    return w.sum() ** 2 / (w * w).sum()

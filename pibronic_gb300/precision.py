"""Precision of the FP32 production kernels against the FP64 build of the same kernels on
identical q.

``compare`` draws X samples with the FP32 sampler (the kernel returns the q its own evaluation
used), evaluates exactly those q with the FP64 build (``DevicePlan(precision=64)``, whose
per-sample outputs agree with the reference's FP64 block_compute_pm, pimc.py:1388-1462, to a
relative 1e-9 on the reference's own q), and reports

* per-sample relative errors of rho, g, g(beta + dbeta) and g(beta - dbeta) (max and 99.9th
  percentile over the samples);
* per-sample errors of the finite-difference terms s1 = (g+ - g-) / (2 dbeta rho) and
  s2 = (g+ - 2 g + g-) / (dbeta^2 rho) (stats.py:38-56), relative to their rms over the samples;
* Z, E and Cv of both runs with the reference's estimators (stats.py:87-130; the jackknife of
  jackknife.py:60-105), and their differences in units of the FP64 run's statistical errors.

The aggregate differences are arithmetic error only (both runs see the same q), so they show how
much of an estimate's error bar the FP32 bulk arithmetic uses up.
"""
from __future__ import annotations

from . import constants, stats
from .pimc import evaluate_device
from .plan import DevicePlan

KEYS = ("s_rho", "s_g", "s_gp", "s_gm")


def _rel(a, b):
    import torch
    d = (a - b).abs() / b.abs()
    d = torch.nan_to_num(d, nan=0.0, posinf=float("inf"))
    return float(d.max()), float(torch.quantile(d[: min(d.numel(), 1 << 24)].float(), 0.999))


def compare(prep, X, seed=1, offset=0, chunk=200_000, variant=0, temperature=None):
    """FP32 (``variant``: 0 automatic, or a DevicePlan.VARIANT_*) against FP64 on the same X
    samples; ``prep`` is a PreparedModels with beta +- dbeta series (K > 0) and at most 8
    surfaces (the FP64 build's range).  Returns a dict of the figures listed in the module
    docstring."""
    import torch
    assert prep.K > 0, "compare needs the beta +- dbeta outputs"
    assert prep.A <= 8, "the FP64 build holds at most 8 surfaces"
    T = temperature if temperature is not None else 1.0 / (prep.beta * constants.boltzman)
    p32 = DevicePlan(prep, precision=32, variant=variant)
    p64 = DevicePlan(prep, precision=64)
    out = {k: [] for k in KEYS}
    ref = {k: [] for k in KEYS}
    for start in range(0, X, chunk):
        n = min(chunk, X - start)
        o32 = evaluate_device(p32, n, seed=seed, offset=offset + start, want_q=True)
        q = o32.pop("q").double()
        o64 = evaluate_device(p64, n, q=q)
        del q
        for k in KEYS:
            out[k].append(o32[k])
            ref[k].append(o64[k])
        if int(o32["status"].item()) != 0 or int(o64["status"].item()) != 0:
            raise AssertionError("non-finite outputs in the precision comparison")
    out = {k: torch.cat(v) for k, v in out.items()}
    ref = {k: torch.cat(v) for k, v in ref.items()}
    res = {"X": X, "A": prep.A, "N": prep.N, "P": prep.P, "T": T, "form_fp32": (
        "tensor-core" if p32.use_tc else {0: "auto", 1: "chunks", 2: "teams", 3: "tensor-core"}[variant])}
    per = {}
    for k in KEYS:
        mx, p999 = _rel(out[k], ref[k])
        per[k] = {"max_rel": mx, "p999_rel": p999}
    db = prep.delta_beta

    def fd(o):
        s1 = (o["s_gp"] - o["s_gm"]) / (2 * db * o["s_rho"])
        s2 = (o["s_gp"] - 2 * o["s_g"] + o["s_gm"]) / (db * db * o["s_rho"])
        return s1, s2
    s1, s2 = fd(out)
    r1, r2 = fd(ref)
    for name, a, b in (("s1", s1, r1), ("s2", s2, r2)):
        rms = float(b.pow(2).mean().sqrt())
        per[name] = {"max_err_over_rms": float((a - b).abs().max()) / rms,
                     "mean_err_over_rms": float((a - b).mean()) / rms}
    res["per_sample"] = per
    e32 = stats.device_estimates(out["s_rho"], out["s_g"], out["s_gp"], out["s_gm"], T, db)
    e64 = stats.device_estimates(ref["s_rho"], ref["s_g"], ref["s_gp"], ref["s_gm"], T, db)
    agg = {}
    for name, key, err in (("Z", "Z", "Z error"), ("E", "jk_E", "jk_E error"), ("Cv", "jk_Cv", "jk_Cv error")):
        d = e32[key] - e64[key]
        agg[name] = {"fp32": e32[key], "fp64": e64[key], "sigma": e64[err],
                     "delta_over_sigma": d / e64[err] if e64[err] > 0 else float("inf"),
                     "delta_rel": abs(d) / abs(e64[key]) if e64[key] != 0 else float("inf")}
    res["estimates"] = agg
    res["ess_per_sample"] = e64["ESS"] / X
    return res


def worst(res):
    """(largest per-sample relative error of rho, g, g+-; largest |delta| / sigma of Z, E, Cv)."""
    return (max(res["per_sample"][k]["max_rel"] for k in KEYS),
            max(abs(v["delta_over_sigma"]) for v in res["estimates"].values()))


def summary_line(res):
    ps, est = res["per_sample"], res["estimates"]
    return (f"A={res['A']} N={res['N']} P={res['P']} T={res['T']:.0f}K X={res['X']}: per-sample max rel "
            + ", ".join(f"{k} {ps[k]['max_rel']:.2e}" for k in KEYS)
            + f"; s1 {ps['s1']['max_err_over_rms']:.2e}, s2 {ps['s2']['max_err_over_rms']:.2e} of rms; "
            + ", ".join(f"d{k}/sigma {v['delta_over_sigma']:+.2e}" for k, v in est.items()))


__all__ = ["compare", "worst", "summary_line"]

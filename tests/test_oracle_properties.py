"""A size-independent property of the reference algorithm, checked on the FP64 oracle (which the
golden reference runs pin): the ring trace and rho's product are invariant under a cyclic
relabelling of the beads, so every output -- rho, g, g(beta +- dbeta), scaled by the product of
the per-bead S12 factors -- is unchanged when the beads of a sample are rotated, and likewise when
the ring is traversed backwards."""
import numpy as np
import pytest

from conftest import case_of, oracle_box_from_case


@pytest.mark.parametrize("name", ["cfg2", "a8", "a12", "odd", "hot", "frozen"])
@pytest.mark.parametrize("shift", [1, 5])
def test_cyclic_bead_relabelling_leaves_outputs_unchanged(runs, name, shift):
    c = case_of(runs, name)
    q = c["q"][:6]
    box = oracle_box_from_case(c, q.shape[2], X=6, B=6)
    a = box.evaluate(q)
    b = box.evaluate(np.roll(q, shift, axis=2))
    for k in ("rho", "g", "gP", "gM"):
        assert np.allclose(a[k], b[k], rtol=1e-11, atol=0), k


@pytest.mark.parametrize("name", ["cfg2", "a8", "odd", "hot"])
def test_reversed_bead_order_leaves_outputs_unchanged(runs, name):
    """Reversing the ring maps each bead pair (p, p+1) to a pair of the reversed ring, so every O
    and S12 factor reappears, and the reversed product is the transpose of the original one (M
    and O are symmetric): its trace is unchanged."""
    c = case_of(runs, name)
    q = c["q"][:6]
    box = oracle_box_from_case(c, q.shape[2], X=6, B=6)
    a = box.evaluate(q)
    b = box.evaluate(np.ascontiguousarray(q[..., ::-1]))
    for k in ("rho", "g", "gP", "gM"):
        assert np.allclose(a[k], b[k], rtol=1e-11, atol=0), k


@pytest.mark.parametrize("name", ["cfg2", "odd", "a8"])
def test_energy_shift_scales_the_ratios_exactly(runs, name):
    """Shifting every diagonal energy of the coupled model by c moves into the O prefactors
    (pimc.py:208-235, 1087-1129): g / rho scales by exp(-beta c) and g(beta +- dbeta) / rho by
    exp(-(beta +- dbeta) c), per sample (the S12 scaling is common to numerator and denominator)."""
    import json
    from oracle import pimc_oracle as po
    c = case_of(runs, name)
    q = c["q"][:5]
    P = q.shape[2]
    beta, db = float(c["beta"]), float(c["delta_beta"])
    T = 1.0 / (beta * po.KB_EV)
    vib = json.loads(str(c["vib_json"]))
    shift = 0.037
    shifted = dict(vib, energies=(np.array(vib["energies"]) + shift * np.eye(len(vib["energies"]))).tolist())
    rho = po.model_from_text(str(c["rho_json"]), diagonal=True)
    a, b = (po.OracleBox(po.model_from_text(json.dumps(v)), rho, 5, 5, P, T, delta_beta=db,
                         draw_sources=False).evaluate(q) for v in (vib, shifted))
    for k, bk in (("g", beta), ("gP", beta + db), ("gM", beta - db)):
        assert np.allclose((b[k] / b["rho"]) / (a[k] / a["rho"]), np.exp(-bk * shift), rtol=1e-11, atol=0), k


@pytest.mark.parametrize("name", ["cfg2", "odd"])
def test_energy_shift_scaling_holds_in_the_kernel_formulation(runs, name):
    """The same property for the kernel's own formulation (tests/kernel_model.py: the tables the
    device uses, the beta series of order 4 for g(beta +- dbeta)), so the series carries the
    exp(-(beta +- dbeta) c) factor to its truncation order."""
    import json
    import kernel_model
    from conftest import prepared_from_case
    c = case_of(runs, name)
    q = c["q"][:5]
    P = q.shape[2]
    beta, db = float(c["beta"]), float(c["delta_beta"])
    vib = json.loads(str(c["vib_json"]))
    shift = 0.037
    shifted = dict(c, vib_json=np.array(json.dumps(dict(
        vib, energies=(np.array(vib["energies"]) + shift * np.eye(len(vib["energies"]))).tolist()))))
    a = kernel_model.evaluate(prepared_from_case(c, P), q)
    b = kernel_model.evaluate(prepared_from_case(shifted, P), q)
    for k, bk in (("s_g", beta), ("s_gp", beta + db), ("s_gm", beta - db)):
        assert np.allclose((b[k] / b["s_rho"]) / (a[k] / a["s_rho"]), np.exp(-bk * shift), rtol=1e-11, atol=0), k

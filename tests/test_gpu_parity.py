"""GPU parity: the CUDA path (through the C ABI) against the reference's recorded outputs and the
FP64 oracle, on identical q.

Tolerances (stated per output):
  * FP64 validation kernels (precision=64): rtol 1e-9 on rho, g, g(beta +- db) -- the algorithm
    itself, bit-for-bit up to rounding (the reference's own O exponent carries ~1e-12 rounding).
  * FP32 production kernel: rtol 2e-4 on rho, g, g(beta +- db); the finite-difference terms
    s1 = (g+ - g-)/(2 db rho) rtol 2e-3; s2 = (g+ - 2g + g-)/(db^2 rho) within 2e-4 of max|s2|
    per sample (measured on GB300: at most 6.2e-5, on the reference's test model; 1e-7 .. 2e-5
    on the synthetic cases).  The kernel forms g+- from one ring product of series in beta, so
    the FP32 rounding of g, g+ and g- is shared and s2 does not inherit the cancellation of
    g+ - 2g + g-.
  * Stage kernels (FP64): the reference test's rtol 1e-5, atol 1e-8.
"""
import numpy as np
import pytest

from conftest import case_of, oracle_box_from_case, prepared_from_case

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CASES = ["cfg1", "cfg2", "cfg2_cold", "cfg2_hot", "odd", "plain", "arho", "single_surface",
         "testmodel", "cfg4", "a8", "a7", "p3_n1", "hot", "frozen", "degen2", "degen4", "degen7"]
WIDE = {"cfg4", "a8", "a7", "degen7"}             # A > 4: the row-team form only
# (case, kernel form): 1 = register-resident chunks, 2 = bead-parallel records + row teams
FORMS = [(c, v) for c in CASES for v in (1, 2) if not (v == 1 and c in WIDE)]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pibronic_gb300 import build, _native
    _native.load(build.build())


def _eval(c, precision, q=None, want_coef=False, variant=0):
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    q = c["q"] if q is None else q
    prep = prepared_from_case(c, q.shape[2])
    plan = DevicePlan(prep, precision=precision, variant=variant)
    out = evaluate_device(plan, q.shape[0], q=torch.as_tensor(q, device="cuda"), want_coef=want_coef)
    torch.cuda.synchronize()
    assert int(out["status"].item()) == 0
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("name,variant", FORMS)
def test_fused_fp64_matches_reference(runs, name, variant):
    c = case_of(runs, name)
    got = _eval(c, 64, variant=variant)
    assert np.allclose(got["s_rho"], c["s_rho"], rtol=1e-9, atol=0)
    assert np.allclose(got["s_g"], c["s_g"], rtol=1e-9, atol=0)
    if "s_gP" in c:
        assert np.allclose(got["s_gp"], c["s_gP"], rtol=1e-9, atol=0)
        assert np.allclose(got["s_gm"], c["s_gM"], rtol=1e-9, atol=0)


@pytest.mark.parametrize("name,variant", FORMS)
def test_fused_fp32_matches_reference(runs, name, variant):
    c = case_of(runs, name)
    got = _eval(c, 32, variant=variant)
    assert np.allclose(got["s_rho"], c["s_rho"], rtol=2e-4, atol=0)
    assert np.allclose(got["s_g"], c["s_g"], rtol=2e-4, atol=0)
    if "s_gP" in c:
        assert np.allclose(got["s_gp"], c["s_gP"], rtol=2e-4, atol=0)
        assert np.allclose(got["s_gm"], c["s_gM"], rtol=2e-4, atol=0)
        db = float(c["delta_beta"])
        s1r = (c["s_gP"] - c["s_gM"]) / (2 * db * c["s_rho"])
        s1 = (got["s_gp"] - got["s_gm"]) / (2 * db * got["s_rho"])
        assert np.allclose(s1, s1r, rtol=2e-3, atol=1e-6 * np.abs(s1r).max())
        s2r = (c["s_gP"] - 2 * c["s_g"] + c["s_gM"]) / (db ** 2 * c["s_rho"])
        s2 = (got["s_gp"] - 2 * got["s_g"] + got["s_gm"]) / (db ** 2 * got["s_rho"])
        err = np.max(np.abs(s2 - s2r)) / np.abs(s2r).max()
        print(f"{name} form {variant}: s2 max error {err:.2e} of max|s2|")
        assert err <= 2e-4, err


def test_fp32_q_input_matches_fp64_q_input(runs):
    c = case_of(runs, "cfg2")
    q32 = c["q"].astype(np.float32)
    a = _eval(c, 32, q=q32.astype(np.float64))
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    prep = prepared_from_case(c, 64)
    plan = DevicePlan(prep, precision=32)
    b = evaluate_device(plan, q32.shape[0], q=torch.as_tensor(q32, device="cuda"))
    for k in ("s_rho", "s_g", "s_gp", "s_gm"):
        assert np.allclose(b[k].cpu().numpy(), a[k], rtol=1e-5, atol=0), k


def test_stage_kernels_explicit_example(explicit, tmp_path):
    """test_pimc_explicit_example.py:168-211 through the package's stage functions."""
    import shutil
    from pibronic_gb300 import pimc, file_structure as fs
    FS = fs.FileStructure(str(tmp_path), 0, 0)
    with open(FS.path_vib_model, "w") as fh:
        fh.write(str(explicit["coupled_model_json"]))
    with open(FS.path_rho_model, "w") as fh:
        fh.write(str(explicit["sampling_model_json"]))
    data = pimc.BoxData.from_FileStructure(FS)
    data.samples, data.beads, data.temperature = 10, 5, 300.0
    data.block_size = 2
    data.blocks = 5
    data.preprocess()
    rho, vib = data.rho, data.vib
    y_rho, y_g = np.full(10, np.nan), np.full(10, np.nan)
    for blk in range(5):
        v = slice(2 * blk, 2 * blk + 2)
        data.qTensor = explicit["samples"][v]
        pimc.build_o_matrix(data, rho.const, rho.state_shift)
        assert np.allclose(rho.const.omatrix.cpu().numpy(), explicit["rho_oMat"][v], rtol=1e-5, atol=1e-8)
        pimc.build_o_matrix(data, vib.const, vib.state_shift)
        assert np.allclose(vib.const.omatrix.cpu().numpy(), explicit["vib_oMat"][v], rtol=1e-5, atol=1e-8)
        pimc.build_denominator(rho.const, y_rho, v)
        pimc.diagonalize_coupling_matrix(data)
        pimc.build_numerator(data, vib.const, y_g, v)
        assert np.allclose(data.M_matrix.cpu().numpy(), explicit["vib_mMat"][v], rtol=1e-5, atol=1e-8)
    assert np.allclose(y_rho, explicit["denominator_rho"], rtol=1e-5, atol=1e-8)
    assert np.allclose(y_g, explicit["numerator_g"], rtol=1e-5, atol=1e-8)
    shutil.rmtree(str(tmp_path), ignore_errors=True)


def test_stage_scaling_matches_oracle(runs):
    """build_scaling_factors + scale_o_matrices + numerator/denominator on the cfg2 q."""
    from pibronic_gb300 import pimc
    c = case_of(runs, "odd")
    box = oracle_box_from_case(c, c["q"].shape[2])
    ref = box.evaluate(c["q"], plus_minus=False)

    class D:
        pass
    data = D()
    A = box.A
    data.states = A
    data.qTensor = np.broadcast_to(c["q"][:, None], (c["q"].shape[0], A) + c["q"].shape[1:]).copy()
    data.qTempTensor = data.qTensor
    data.tau = box.tau

    class Const:
        pass

    def tdc(model):
        k = Const()
        k.d_coth = torch.as_tensor(model["const"]["coth"], device="cuda").contiguous()
        k.d_csch = torch.as_tensor(model["const"]["csch"], device="cuda").contiguous()
        k.d_prefactor = torch.as_tensor(model["const"]["prefactor"], device="cuda")
        return k
    rc, vc = tdc(box.rho), tdc(box.vib)
    pimc.build_o_matrix(data, rc, box.rho["state_shift"])
    pimc.build_o_matrix(data, vc, box.vib["state_shift"])
    S12 = torch.empty((c["q"].shape[0], c["q"].shape[2]), dtype=torch.float64, device="cuda")
    pimc.build_scaling_factors(S12, rc, vc)
    pimc.scale_o_matrices(S12, rc, vc)
    y_rho, y_g = np.empty(c["q"].shape[0]), np.empty(c["q"].shape[0])
    pimc.build_denominator(rc, y_rho, slice(None))

    class V:
        pass
    data.vib = V()
    data.vib.energy, data.vib.linear, data.vib.quadratic = box.vib["energy"], box.vib["linear"], box.vib["quadratic"]
    pimc.diagonalize_coupling_matrix(data)
    pimc.build_numerator(data, vc, y_g, slice(None))
    assert np.allclose(S12.cpu().numpy(), ref["S12"], rtol=1e-10)
    assert np.allclose(y_rho, ref["rho"], rtol=1e-9)
    assert np.allclose(y_g, ref["g"], rtol=1e-9)


@pytest.mark.parametrize("name", ["a12", "a16", "a8", "degen12", "degen7", "degen4"])
def test_tensor_core_form_matches_reference(runs, name):
    """The tensor-core form (V(q) by the tcgen05 GEMM; the wide kernel above 8 surfaces, the
    row-team kernel on the GEMM's V up to 8) on the reference's recorded q, against the
    reference's outputs at the FP32 production tolerance."""
    from pibronic_gb300.plan import DevicePlan
    c = case_of(runs, name)
    got = _eval(c, 32, variant=DevicePlan.VARIANT_TC)
    assert np.allclose(got["s_rho"], c["s_rho"], rtol=2e-4, atol=0)
    assert np.allclose(got["s_g"], c["s_g"], rtol=2e-4, atol=0)
    assert np.allclose(got["s_gp"], c["s_gP"], rtol=2e-4, atol=0)
    assert np.allclose(got["s_gm"], c["s_gM"], rtol=2e-4, atol=0)

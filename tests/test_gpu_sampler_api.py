"""GPU: the device sampler, the end-to-end API (BoxDataPM -> block_compute_pm -> result files ->
estimators), the device reductions against the oracle's estimators, a closed-form check on a
harmonic (uncoupled) model, and edge cases."""
import math
import os

import numpy as np
import pytest

from conftest import case_of

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pibronic_gb300 import build, _native
    _native.load(build.build())


def make_box(tmp_path, A=4, N=12, P=64, T=300.0, X=20000, seed=7, pm=True, model_seed=3,
             uncoupled=False, **kw):
    from pibronic_gb300 import constants, pimc, synthetic, vibronic_io
    from pibronic_gb300.file_structure import FileStructure
    FS = FileStructure(str(tmp_path), 0, 0)
    model = synthetic.make_coupled_model(A, N, model_seed, **kw)
    if uncoupled:
        VMK = vibronic_io.VMK
        off = ~np.eye(A, dtype=bool)
        model[VMK.E][off] = 0.0
        model[VMK.G1][:, off] = 0.0
        model[VMK.G2][...] = 0.0
    vibronic_io.save_model_to_JSON(FS.path_vib_model, model)
    vibronic_io.create_basic_diagonal_model(FS)
    FS.generate_model_hashes()
    beta = constants.beta(T)
    data = pimc.BoxDataPM(1e-4 * beta) if pm else pimc.BoxData()
    data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
    data.hash_vib, data.hash_rho = FS.hash_vib, FS.hash_rho
    data.states, data.modes, data.beads, data.temperature = A, N, P, T
    data.samples, data.block_size = X, min(X, 10000)
    data.blocks = X // data.block_size
    data.seed = seed
    data.preprocess()
    return FS, data


def test_sampler_distribution(tmp_path):
    """Normal-mode coordinates of the drawn q have the precision 2 coth - csch lambda_k
    (pimc.py:402-404) and the sources follow the state weights (pimc.py:343-350)."""
    from pibronic_gb300 import _native
    from pibronic_gb300.plan import ring_mode_basis, ring_mode_eigenvalues
    FS, data = make_box(tmp_path, A=3, N=4, P=16, X=200000)
    X, N, P = data.samples, data.modes, data.beads
    q = torch.empty((X, N, P), dtype=torch.float32, device="cuda")
    src = torch.empty(X, dtype=torch.int32, device="cuda")
    lib = _native.load()
    _native.check(lib.pbr_sample_q(data.plan.struct, 11, 0, X, _native.ptr(q), _native.ptr(src),
                                   _native.stream_handle()), "sample_q")
    q = q.double().cpu().numpy()
    src = src.cpu().numpy()
    w = data.rho.state_weight
    counts = np.bincount(src, minlength=len(w))
    sd = np.sqrt(X * w * (1 - w))
    assert np.all(np.abs(counts - X * w) < 5 * sd + 1)
    B = ring_mode_basis(P)
    lam = ring_mode_eigenvalues(P)
    prep = data.prepared
    coth = 1 / np.tanh(prep.tau * prep.rho_omega)
    csch = 1 / np.sinh(prep.tau * prep.rho_omega)
    var = 1.0 / (2 * coth[:, None] - csch[:, None] * lam[None, :])          # (N, P)
    for a in range(len(w)):
        sel = src == a
        n = sel.sum()
        if n < 1000:
            continue
        x = q[sel] - prep.rho_shift[a][None, :, None]
        cc = np.einsum("xjp,pk->xjk", x, B)
        m = cc.mean(axis=0)
        v = cc.var(axis=0)
        assert np.all(np.abs(m) < 6 * np.sqrt(var / n)), a
        assert np.all(np.abs(v / var - 1) < 6 * np.sqrt(2.0 / n)), a


def test_sampled_q_evaluates_like_oracle(tmp_path):
    """pbr_sample_eval's own q (returned) through the FP64 oracle gives the kernel's outputs."""
    from oracle import pimc_oracle as po
    from pibronic_gb300.pimc import evaluate_device
    FS, data = make_box(tmp_path, A=4, N=12, P=64, X=64)
    out = evaluate_device(data.plan, 64, seed=5, offset=1000, want_q=True)
    q = out["q"].double().cpu().numpy()
    box = po.OracleBox(po.model_from_file(FS.path_vib_model),
                       po.model_from_file(FS.path_rho_model, diagonal=True), 64, 64, 64,
                       data.temperature, delta_beta=data.delta_beta, draw_sources=False)
    ref = box.evaluate(q)
    for k, rk in (("s_rho", "rho"), ("s_g", "g"), ("s_gp", "gP"), ("s_gm", "gM")):
        assert np.allclose(out[k].cpu().numpy(), ref[rk], rtol=2e-4, atol=0), k
    # the sampler-only entry point draws the same q
    from pibronic_gb300 import _native
    q2 = torch.empty((64, 12, 64), dtype=torch.float32, device="cuda")
    _native.check(_native.load().pbr_sample_q(data.plan.struct, 5, 1000, 64, _native.ptr(q2), None,
                                              _native.stream_handle()), "sample_q")
    assert torch.equal(q2, out["q"])


def test_both_kernel_forms_draw_the_same_samples(tmp_path):
    """The register-chunk and row-team forms consume the same Philox stream: same q, and the
    same outputs up to FP32 rounding."""
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    FS, data = make_box(tmp_path, A=4, N=12, P=64, X=256)
    a = evaluate_device(DevicePlan(data.prepared, variant=1), 256, seed=4, offset=77, want_q=True)
    b = evaluate_device(DevicePlan(data.prepared, variant=2), 256, seed=4, offset=77, want_q=True)
    assert torch.equal(a["src"], b["src"])
    assert torch.allclose(a["q"], b["q"], rtol=1e-6, atol=1e-5)
    for k in ("s_rho", "s_g", "s_gp", "s_gm"):
        assert torch.allclose(a[k], b[k], rtol=2e-4, atol=0), k


def test_counter_based_stream_is_deterministic_and_splittable(tmp_path):
    from pibronic_gb300.pimc import evaluate_device
    FS, data = make_box(tmp_path, A=2, N=3, P=12, X=1000)
    a = evaluate_device(data.plan, 1000, seed=9, offset=0)
    b = evaluate_device(data.plan, 1000, seed=9, offset=0)
    c = evaluate_device(data.plan, 600, seed=9, offset=400)
    for k in ("s_rho", "s_g", "s_gp", "s_gm"):
        assert torch.equal(a[k], b[k])
        assert torch.equal(a[k][400:], c[k])


def test_block_compute_pm_files_and_estimators(tmp_path):
    """End to end through the public API: result file keys (pimc.py:954-963), merge of several
    job files (pimc.py:975-1040), device estimators vs the oracle's stats.py formulas."""
    from oracle import stats_oracle as so
    from pibronic_gb300 import pimc, stats
    FS, data = make_box(tmp_path, A=4, N=12, P=64, X=20000)
    for job in range(2):
        data.seed = 100 + job
        res = pimc.BoxResultPM(data=data)
        res.path_root = FS.path_rho_results
        res.id_job = job
        pimc.block_compute_pm(data, res)
        path = os.path.join(FS.path_rho_results, f"P64_T300.00_J{job}_data_points.npz")
        with np.load(path) as f:
            assert set(f.files) == {"hash_vib", "hash_rho", "number_of_samples", "s_rho", "s_g",
                                    "s_gP", "s_gM"}
            assert int(f["number_of_samples"]) == 20000
            assert np.all(np.isfinite(f["s_g"]))
        dev = stats.device_estimates(res.device["s_rho"], res.device["s_g"], res.device["s_gp"],
                                     res.device["s_gm"], data.temperature, data.delta_beta)
        terms = so.basic_terms(data.delta_beta, res.scaled_rho, res.scaled_g,
                               res.scaled_gofr_plus, res.scaled_gofr_minus)
        basic = so.estimate_basic(20000, data.temperature, *terms)
        jk = so.estimate_jackknife(20000, data.temperature, data.delta_beta, basic,
                                   *[so.jackknife_term(20000, t) for t in terms])
        assert math.isclose(dev["Z"], basic["Z"], rel_tol=1e-12)
        assert math.isclose(dev["Z error"], basic["Z error"], rel_tol=1e-9)
        assert math.isclose(dev["E"], basic["E"], rel_tol=1e-12)
        assert math.isclose(dev["Cv"], basic["Cv"], rel_tol=1e-9, abs_tol=1e-12)
        assert math.isclose(dev["jk_E"], jk["E"], rel_tol=1e-9)
        assert math.isclose(dev["jk_E error"], jk["E error"], rel_tol=1e-4)
        assert math.isclose(dev["jk_Cv"], jk["Cv"], rel_tol=1e-6, abs_tol=1e-9)
        assert math.isclose(dev["jk_Cv error"], jk["Cv error"], rel_tol=1e-3)
    merged = pimc.BoxResultPM()
    merged.load_multiple_results([os.path.join(FS.path_rho_results, f"P64_T300.00_J{j}_data_points.npz")
                                  for j in range(2)])
    assert merged.samples == 40000 and np.all(np.isfinite(merged.scaled_gofr_minus))


def test_reductions_match_reference_stats(runs):
    """Device reductions on the reference's own cfg1 outputs reproduce its stats.py numbers."""
    from pibronic_gb300 import stats
    c = case_of(runs, "cfg1")
    t = {k: torch.as_tensor(c[k], device="cuda") for k in ("s_rho", "s_g", "s_gP", "s_gM")}
    dev = stats.device_estimates(t["s_rho"], t["s_g"], t["s_gP"], t["s_gM"], 300.0, float(c["delta_beta"]))
    assert math.isclose(dev["Z"], float(runs["stats/basic/Z"]), rel_tol=1e-12)
    assert math.isclose(dev["Z error"], float(runs["stats/basic/Z error"]), rel_tol=1e-9)
    assert math.isclose(dev["E"], float(runs["stats/basic/E"]), rel_tol=1e-11)
    assert math.isclose(dev["Cv"], float(runs["stats/basic/Cv"]), rel_tol=1e-8)
    assert math.isclose(dev["jk_E"], float(runs["stats/jk/E"]), rel_tol=1e-9)
    assert math.isclose(dev["jk_E error"], float(runs["stats/jk/E error"]), rel_tol=1e-5)
    assert math.isclose(dev["jk_Cv"], float(runs["stats/jk/Cv"]), rel_tol=1e-7)
    assert math.isclose(dev["jk_Cv error"], float(runs["stats/jk/Cv error"]), rel_tol=1e-4)


def test_uncoupled_model_matches_closed_form(tmp_path):
    """Uncoupled model with rho = its diagonal: g/rho = 1 for every sample, and the sampled
    finite-difference E, Cv agree with the closed-form harmonic partition function
    Z(beta) ~ sum_a exp(-beta Etilde_a) prod_j 1/(2 sinh(beta w_j / 2)) within 5 sigma."""
    from pibronic_gb300 import stats
    from pibronic_gb300.constants import boltzman
    from pibronic_gb300.pimc import evaluate_device
    X = 400000
    FS, data = make_box(tmp_path, A=3, N=6, P=32, T=300.0, X=X, uncoupled=True)
    out = evaluate_device(data.plan, X, seed=21, offset=0)
    r = (out["s_g"] / out["s_rho"]).cpu().numpy()
    assert np.allclose(r, 1.0, rtol=1e-5, atol=0)
    est = stats.device_estimates(out["s_rho"], out["s_g"], out["s_gp"], out["s_gm"],
                                 data.temperature, data.delta_beta)
    prep = data.prepared
    w = prep.vib_omega

    def Z(b):
        return np.sum(np.exp(-b * prep.vib_tilde)) * np.prod(1.0 / (2 * np.sinh(b * w / 2)))
    b, db = prep.beta, data.delta_beta
    E_fd = -(Z(b + db) - Z(b - db)) / (2 * db * Z(b))
    Cv_fd = ((Z(b + db) - 2 * Z(b) + Z(b - db)) / (db ** 2 * Z(b)) - E_fd ** 2) / (boltzman * 300.0 ** 2)
    assert abs(est["jk_E"] - E_fd) < 5 * est["jk_E error"] + 1e-9 * abs(E_fd)
    assert abs(est["jk_Cv"] - Cv_fd) < 5 * est["jk_Cv error"] + 1e-6 * abs(Cv_fd)


@pytest.mark.parametrize("X", [1, 3, 127, 1001])
def test_ragged_sample_counts(tmp_path, X):
    from pibronic_gb300.pimc import evaluate_device
    FS, data = make_box(tmp_path, A=2, N=3, P=12, X=2000)
    full = evaluate_device(data.plan, 2000, seed=3, offset=0)
    part = evaluate_device(data.plan, X, seed=3, offset=0)
    for k in ("s_rho", "s_g", "s_gp", "s_gm"):
        assert torch.equal(full[k][:X], part[k])


SHAPES = [(1, 1, 3), (2, 2, 5), (3, 7, 33), (4, 20, 256), (2, 64, 8), (6, 20, 128), (8, 4, 17),
          (5, 9, 40)]


@pytest.mark.parametrize("A,N,P,variant", [s + (v,) for s in SHAPES for v in (1, 2) if v == 2 or s[0] <= 4])
def test_shapes_sample_eval_against_oracle(tmp_path, A, N, P, variant):
    from oracle import pimc_oracle as po
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    FS, data = make_box(tmp_path, A=A, N=N, P=P, X=32, sd_quadratic=0.0005)
    plan = DevicePlan(data.prepared, precision=32, variant=variant)
    out = evaluate_device(plan, 32, seed=1, offset=0, want_q=True)
    q = out["q"].double().cpu().numpy()
    box = po.OracleBox(po.model_from_file(FS.path_vib_model),
                       po.model_from_file(FS.path_rho_model, diagonal=True), 32, 32, P,
                       data.temperature, delta_beta=data.delta_beta, draw_sources=False)
    ref = box.evaluate(q)
    for k, rk in (("s_rho", "rho"), ("s_g", "g"), ("s_gp", "gP"), ("s_gm", "gM")):
        rel = np.max(np.abs(out[k].cpu().numpy() / ref[rk] - 1.0))
        assert rel <= 1e-4, (k, rel)


def test_eval_q_long_ring(tmp_path):
    """P = 512 on the caller-q path (chunks of 16 beads per thread), FP64 kernel vs oracle."""
    from oracle import pimc_oracle as po
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    FS, data = make_box(tmp_path, A=2, N=3, P=512, X=8, sd_quadratic=0.0005)
    box = po.OracleBox(po.model_from_file(FS.path_vib_model),
                       po.model_from_file(FS.path_rho_model, diagonal=True), 8, 8, 512,
                       data.temperature, delta_beta=data.delta_beta)
    q = box.draw_q(slice(0, 8))
    ref = box.evaluate(q)
    out = evaluate_device(DevicePlan(data.prepared, precision=64), 8, q=torch.as_tensor(q, device="cuda"))
    for k, rk in (("s_rho", "rho"), ("s_g", "g"), ("s_gp", "gP"), ("s_gm", "gM")):
        assert np.allclose(out[k].cpu().numpy(), ref[rk], rtol=1e-9, atol=0), k


def test_errors_are_reported_not_faulted(tmp_path):
    """Host-side failures: NaN coordinates raise (status flag), unsupported sizes raise
    AssertionError, a sampling model with fewer surfaces than the coupled one is rejected."""
    from pibronic_gb300 import _native
    from pibronic_gb300.pimc import evaluate_device
    FS, data = make_box(tmp_path, A=2, N=3, P=12, X=16)
    q = torch.zeros((16, 3, 12), dtype=torch.float64, device="cuda")
    q[3, 1, 5] = float("nan")
    out = evaluate_device(data.plan, 16, q=q)
    assert int(out["status"].item()) == _native.PBR_ERR_NONFINITE
    (tmp_path / "big").mkdir()
    FS2, data2 = make_box(tmp_path / "big", A=2, N=65, P=4, X=16, sd_quadratic=0.0)
    with pytest.raises(AssertionError):
        evaluate_device(data2.plan, 16, seed=1)        # the fused kernels support N <= 64
    from pibronic_gb300.plan import PreparedModels
    from pibronic_gb300 import vibronic_io
    vib = vibronic_io.load_model_from_JSON(FS.path_vib_model)
    rho = vibronic_io.load_diagonal_model_from_JSON(FS.path_rho_model)
    rho1 = {k: (v[..., :1] if isinstance(v, np.ndarray) and k != vibronic_io.VMK.w else v)
            for k, v in rho.items()}
    rho1[vibronic_io.VMK.A] = 1
    with pytest.raises(AssertionError):
        PreparedModels(vib, rho1, 12, temperature=300.0)


def test_pooled_reduction_on_one_process_equals_the_plain_one(tmp_path):
    """DeviceReducer.pooled (the multi-rank jackknife of shard.pooled_moments) without a process
    group runs the same two passes as DeviceReducer.launch."""
    from pibronic_gb300 import stats
    from pibronic_gb300.pimc import evaluate_device
    FS, data = make_box(tmp_path, A=3, N=5, P=16, X=50000)
    out = evaluate_device(data.plan, 50000, seed=3, offset=0)
    args = (out["s_rho"], out["s_g"], out["s_gp"], out["s_gm"], data.delta_beta, data.temperature)
    red = stats.DeviceReducer(50000)
    pooled = red.pooled(*args)
    plain = stats.device_estimates(out["s_rho"], out["s_g"], out["s_gp"], out["s_gm"], data.temperature,
                                   data.delta_beta)
    for k, v in plain.items():
        assert v == pooled[k], k

"""GPU: the quadratic part of V on the tensor cores inside the fused kernels (mma.sync m16n8k16,
FP16 hi/lo split of the pair products and of the power-of-two-scaled couplings, three MMAs per
tile): the register-chunk form at 3-4 surfaces and the row-team form's bead records at 5-8
surfaces (one block per SM), both from 16 modes on.

Checked against the FP64 oracle on the kernel's own samples and against the FP64 build on the same
q, at the FP32 production tolerance (rtol 2e-4 on rho, g, g(beta +- db)); and with one sample's
coordinate beyond the FP16-safe bound (|q| > 181), which sends its warp to the FP32 pair loop for
every bead, against the FP64 build on that q."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL = 2e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pibronic_gb300 import build, _native
    _native.load(build.build())


def _box(tmp_path, A, N, P, X, seed=5, **kw):
    from pibronic_gb300 import constants, pimc, synthetic, vibronic_io
    from pibronic_gb300.file_structure import FileStructure
    FS = FileStructure(str(tmp_path), 0, 0)
    model = synthetic.make_coupled_model(A, N, seed, **kw)
    vibronic_io.save_model_to_JSON(FS.path_vib_model, model)
    vibronic_io.create_basic_diagonal_model(FS)
    FS.generate_model_hashes()
    data = pimc.BoxDataPM(1e-4 * constants.beta(300.0))
    data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
    data.hash_vib, data.hash_rho = FS.hash_vib, FS.hash_rho
    data.states, data.modes, data.beads, data.temperature = A, N, P, 300.0
    data.samples, data.block_size, data.blocks, data.seed = X, X, 1, seed
    data.preprocess()
    return FS, data


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) / np.asarray(b) - 1.0)))


@pytest.mark.parametrize("A,N,P,X,variant", [(4, 20, 32, 40, 1), (3, 16, 24, 40, 1), (4, 24, 50, 33, 1),
                                               (6, 20, 128, 12, 2), (7, 16, 33, 21, 2), (8, 18, 20, 24, 2)])
def test_against_oracle(tmp_path, A, N, P, X, variant):
    """Register-chunk form (variant 1) and row teams (variant 2), device-drawn samples; X not a
    multiple of the warp's samples, P = 50 (ragged last chunk) and P = 33 (a partial last round of
    bead records) exercise the uniform loops' idle rows."""
    from oracle import pimc_oracle as po
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    FS, data = _box(tmp_path, A, N, P, X)
    out = evaluate_device(DevicePlan(data.prepared, precision=32, variant=variant), X, seed=3, offset=0,
                          want_q=True)
    assert int(out["status"].item()) == 0
    q = out["q"].double().cpu().numpy()
    box = po.OracleBox(po.model_from_file(FS.path_vib_model),
                       po.model_from_file(FS.path_rho_model, diagonal=True), X, X, P,
                       data.temperature, delta_beta=data.delta_beta, draw_sources=False)
    ref = box.evaluate(q)
    for k, rk in (("s_rho", "rho"), ("s_g", "g"), ("s_gp", "gP"), ("s_gm", "gM")):
        rel = _rel(out[k].cpu().numpy(), ref[rk])
        print(f"A={A} N={N} P={P} {k}: max rel {rel:.2e}")
        assert rel <= RTOL, (k, rel)


@pytest.mark.parametrize("A,N,P,variant", [(4, 20, 32, 1), (7, 16, 32, 2)])
def test_large_coordinate_takes_the_fp32_loop(tmp_path, A, N, P, variant):
    """Caller's q (FP32) with one sample's mode 3 at bead 5 set to 250: the records of that
    sample's warp use the FP32 pair loop; the warp's other samples (ordinary coordinates) match
    the FP64 build on the same q, as do all other samples.  The planted sample itself (an energy
    of thousands of eV at that bead) is left out of the comparison.  The quadratic couplings are
    N(0, 2e-5) so that sample's exp(-tau V) stays inside the FP32 range."""
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    X = 64
    FS, data = _box(tmp_path, A, N, P, X, sd_quadratic=2e-5)
    q = evaluate_device(DevicePlan(data.prepared, precision=32, variant=variant), X, seed=9, offset=0,
                        want_q=True)["q"]
    q[7, 3, 5] = 250.0
    o32 = evaluate_device(DevicePlan(data.prepared, precision=32, variant=variant), X, q=q)
    o64 = evaluate_device(DevicePlan(data.prepared, precision=64, variant=variant), X, q=q.double())
    assert int(o32["status"].item()) == 0 and int(o64["status"].item()) == 0
    keep = np.arange(X) != 7
    for k in ("s_rho", "s_g", "s_gp", "s_gm"):
        a, b = o32[k].cpu().numpy()[keep], o64[k].cpu().numpy()[keep]
        rel = _rel(a, b)
        print(f"{k}: max rel {rel:.2e}")
        assert rel <= RTOL, (k, rel)

"""GPU: the learned proposal's kernels against the numpy flow oracle (oracle/flow_oracle.py),
the tensor-core layers of the sampling direction against the FP32 ones, the exactness of the
density (unbiased estimates for any parameters, checked on a model with a closed-form answer, with
the tensor-core layers that sampling uses by default), and what training gains over plain rho."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pibronic_gb300 import build, _native
    _native.load(build.build())


def _box(tmp_path, **kw):
    from test_gpu_sampler_api import make_box
    return make_box(tmp_path, **kw)


def _flow(data, **kw):
    from pibronic_gb300.flow import FlowProposal
    return FlowProposal(data.prepared, data.plan, **kw)


def _draw(data, X, seed=3):
    from pibronic_gb300 import _native
    q = torch.empty((X, data.modes, data.beads), dtype=torch.float32, device="cuda")
    _native.check(_native.load().pbr_sample_q(data.plan.struct, seed, 0, X, _native.ptr(q), None,
                                              _native.stream_handle()), "sample_q")
    return q


@pytest.mark.parametrize("N,P,X", [(5, 16, 64), (20, 50, 37), (13, 128, 40), (64, 24, 11)])
def test_prepare_matches_numpy(tmp_path, N, P, X):
    """P = 50 and 24: bead counts that are not a multiple of the warp; X not a multiple of the
    block's whole samples; N = 64: four samples per block."""
    from pibronic_gb300.plan import ring_mode_basis
    FS, data = _box(tmp_path, A=3, N=N, P=P, X=X)
    fl = _flow(data, nsel=3, layers=2, hidden=32)
    q = _draw(data, X)
    y, U = fl.prepare(q)
    qh = q.double().cpu().numpy()
    B = ring_mode_basis(P)[:, :3]
    c = fl.t_center.cpu().numpy()
    sig = fl.t_sigma.cpu().numpy().reshape(N, 3)
    x = qh - c[None, :, None]
    yref = np.einsum("xjp,ps->xjs", x, B) / sig[None]
    assert np.allclose(y.cpu().numpy().reshape(X, N, 3), yref, rtol=1e-5, atol=1e-5)
    tau, w = data.prepared.tau, data.prepared.rho_omega
    lam_q = (2 / np.tanh(tau * w))[None, :] * (x ** 2).sum(axis=2) \
        - (1 / np.sinh(tau * w))[None, :] * 2 * (x * np.roll(x, -1, axis=2)).sum(axis=2)
    Uref = lam_q.sum(axis=1) - (yref ** 2).sum(axis=(1, 2))
    # FP32 within a mode, FP64 across modes: ~1e-7 relative per mode (a weight moves by e^(dU/2))
    assert np.allclose(U.cpu().numpy(), Uref, rtol=2e-6, atol=1e-6 * N)


@pytest.mark.parametrize("N,P,X,nsel", [(5, 16, 64, 3), (20, 50, 37, 3), (13, 128, 41, 2), (7, 33, 9, 5)])
def test_apply_matches_numpy(tmp_path, N, P, X, nsel):
    """x = q + sum_s B_s sigma_s (y' - y) against numpy; X N rows not a multiple of the kernel's
    four-row groups (13 x 41, 7 x 9)."""
    from pibronic_gb300 import _native
    from pibronic_gb300.plan import ring_mode_basis
    FS, data = _box(tmp_path, A=3, N=N, P=P, X=X)
    fl = _flow(data, nsel=nsel, layers=2, hidden=32)
    q = _draw(data, X)
    g = torch.Generator(device="cuda").manual_seed(3)
    y = torch.randn((X, N * nsel), generator=g, device="cuda")
    yn = y + 0.1 * torch.randn((X, N * nsel), generator=g, device="cuda")
    x = torch.empty_like(q)
    p = _native.ptr
    _native.check(_native.load().pbr_flow_apply(p(q), p(y), p(yn), X, N, P, nsel, p(fl.t_sigma), p(x),
                                                _native.stream_handle()), "flow apply")
    torch.cuda.synchronize()
    B = ring_mode_basis(P)[:, :nsel]
    sig = fl.t_sigma.cpu().numpy().reshape(N, nsel)
    d = (yn - y).double().cpu().numpy().reshape(X, N, nsel) * sig[None]
    xref = q.double().cpu().numpy() + np.einsum("xjs,ps->xjp", d, B)
    assert np.allclose(x.double().cpu().numpy(), xref, rtol=1e-6, atol=1e-5)


# (N, nsel, layers, hidden, X): sample-tiled layers at hidden 32 / 64 / 128 (ragged last tile, odd
# D with I != J, the learned configurations' D = 60 and D = 128), and D = 192 at hidden 128, whose
# padded weights exceed the tiled form's shared memory (the warp-per-sample layers run)
LAYER_CASES = [(4, 3, 4, 64, 300), (5, 3, 2, 128, 77), (20, 3, 2, 128, 1000), (64, 2, 2, 128, 130),
               (64, 3, 2, 128, 130), (4, 3, 2, 32, 65)]


@pytest.mark.parametrize("N,nsel,layers,hidden,X", LAYER_CASES)
def test_layers_match_oracle(tmp_path, N, nsel, layers, hidden, X):
    from oracle import flow_oracle as fo
    FS, data = _box(tmp_path, A=2, N=N, P=12, X=64)
    fl = _flow(data, nsel=nsel, layers=layers, hidden=hidden, init_scale=0.5, seed=2)
    y = torch.randn((X, fl.D), device="cuda")
    yf, ldf = fl.forward(y)
    ref_y, ref_ld = fo.forward(fl.params_host(), y.double().cpu().numpy())
    assert np.allclose(yf.cpu().numpy(), ref_y, rtol=1e-4, atol=1e-4)
    assert np.allclose(ldf.cpu().numpy(), ref_ld, rtol=1e-4, atol=1e-4)
    yi, ldi = fl.inverse(yf)
    assert np.allclose(yi.cpu().numpy(), y.cpu().numpy(), atol=1e-4)
    assert np.allclose(ldi.cpu().numpy(), -ldf.cpu().numpy(), atol=1e-4)


@pytest.mark.parametrize("N,nsel,layers,hidden,X", LAYER_CASES)
def test_tensor_core_layers_follow_the_fp32_layers(tmp_path, N, nsel, layers, hidden, X):
    """The BF16 tensor-core layers (sampling direction) against the FP32 layers on the same
    weights: BF16 rounds the weights and activations to 8 bits, so y' and the log-determinant
    follow the FP32 network to about 1e-2 of their scale, not to FP32 rounding.  With a zero head
    the layers are the identity exactly."""
    FS, data = _box(tmp_path, A=2, N=N, P=12, X=64)
    fl = _flow(data, nsel=nsel, layers=layers, hidden=hidden, init_scale=0.5, seed=2)
    # D = 192 at hidden 128: the weights and a 128-sample tile exceed the shared memory, and that
    # proposal samples with the FP32 layers
    assert fl.sample_tc == (fl.D <= 128)
    if not fl.sample_tc:
        return
    y = torch.randn((X, fl.D), device="cuda")
    yf, ldf = fl.forward(y)
    yt, ldt = fl.forward_tc(y)
    torch.cuda.synchronize()
    assert int(fl._tc_status.item()) == 0
    dy = float((yt - yf).abs().max() / (yf.abs().max() + 1.0))
    dl = float((ldt - ldf).abs().max() / (ldf.abs().max() + 1.0))
    print(f"N={N} nsel={nsel} layers={layers} H={hidden} X={X}: max |dy| {dy:.2e}, |dlogdet| {dl:.2e}")
    assert dy < 3e-2 and dl < 3e-2, (dy, dl)
    zero = _flow(data, nsel=nsel, layers=layers, hidden=hidden, init_scale=0.0, seed=2)
    yz, ldz = zero.forward_tc(y)
    assert torch.equal(yz, y) and not bool(ldz.abs().max() > 0)


@pytest.mark.parametrize("N,nsel,layers,hidden,X", [(4, 3, 4, 32, 4096), (5, 3, 2, 128, 1000),
                                                    (64, 2, 2, 128, 1000), (64, 3, 2, 128, 300)])
def test_gradients_match_oracle(tmp_path, N, nsel, layers, hidden, X):
    from oracle import flow_oracle as fo
    FS, data = _box(tmp_path, A=3, N=N, P=12, X=64)
    fl = _flow(data, nsel=nsel, layers=layers, hidden=hidden, init_scale=0.5, seed=5)
    fl.nu.copy_(torch.tensor([0.2, -0.1, 0.3], device="cuda"))
    y = torch.randn((X, fl.D), device="cuda")
    r = torch.exp(torch.randn(X, device="cuda", dtype=torch.float64))
    loss, grads, g_nu = fl.gradients(y, r)
    torch.cuda.synchronize()
    ref_loss, ref_grads, ref_gnu = fo.loss_and_grads(fl.params_host(), fl.nu.double().cpu().numpy(),
                                                     y.double().cpu().numpy(), r.cpu().numpy(),
                                                     fl.t_mu.double().cpu().numpy(), fl.log_w)
    assert math.isclose(float(loss), ref_loss, rel_tol=1e-4, abs_tol=1e-5)
    for l in range(layers):
        for k, v in grads[l].items():
            ref = ref_grads[l][k]
            scale = np.abs(ref).max() + 1e-12
            assert np.max(np.abs(v.double().cpu().numpy() - ref)) <= 2e-3 * scale, (l, k)
    assert np.allclose(g_nu.double().cpu().numpy(), ref_gnu, rtol=1e-3, atol=1e-5)


def test_flow_estimates_are_unbiased_for_any_parameters(tmp_path):
    """Uncoupled model (g = rho exactly): whatever the flow and the learned surface weights,
    mean(g/q_flow) must equal Z/Z_rho = 1 and E must equal the closed form within 5 sigma."""
    from pibronic_gb300 import stats
    from pibronic_gb300.constants import boltzman
    FS, data = _box(tmp_path, A=3, N=6, P=32, T=300.0, X=1000, uncoupled=True)
    fl = _flow(data, nsel=3, layers=4, hidden=32, init_scale=0.4, seed=7)
    fl.nu.copy_(torch.tensor([0.5, -0.5, 0.2], device="cuda"))
    X = 400_000
    out = fl.sample_and_evaluate(X, seed=11)
    assert int(out["status"].item()) == 0
    est = stats.device_estimates(out["s_q"], out["s_g"], out["s_gp"], out["s_gm"], 300.0, data.delta_beta)
    assert abs(est["Z"] - 1.0) < 5 * est["Z error"]
    assert est["ESS"] < 0.999 * X                         # the flow really moved the samples
    prep = data.prepared
    w = prep.vib_omega

    def Z(b):
        return np.sum(np.exp(-b * prep.vib_tilde)) * np.prod(1.0 / (2 * np.sinh(b * w / 2)))
    b, db = prep.beta, data.delta_beta
    E_fd = -(Z(b + db) - Z(b - db)) / (2 * db * Z(b))
    assert abs(est["jk_E"] - E_fd) < 5 * est["jk_E error"] + 1e-9


def test_training_gains_effective_samples(tmp_path):
    """Strongly coupled model: after training on rho's own weighted samples the proposal's ESS
    per sample beats plain rho's, and Z, E agree with plain rho within error bars."""
    from pibronic_gb300 import stats
    from pibronic_gb300.pimc import evaluate_device
    FS, data = _box(tmp_path, A=3, N=4, P=16, T=200.0, X=1000, sd_offdiag=0.1, model_seed=404)
    X = 200_000
    plain = evaluate_device(data.plan, X, seed=1, offset=0, want_q=True)
    ep = stats.device_estimates(plain["s_rho"], plain["s_g"], plain["s_gp"], plain["s_gm"], 200.0,
                                data.delta_beta)
    fl = _flow(data, nsel=3, layers=6, hidden=64, seed=1)
    y, _ = fl.prepare(plain["q"])
    r = plain["s_g"] / plain["s_rho"]
    fl.train(y, r, epochs=6, batch=8192, lr=2e-3)
    out = fl.sample_and_evaluate(X, seed=2)
    ef = stats.device_estimates(out["s_q"], out["s_g"], out["s_gp"], out["s_gm"], 200.0, data.delta_beta)
    assert ef["ESS"] / X > ep["ESS"] / X
    assert abs(ef["Z"] - ep["Z"]) < 5 * math.hypot(ef["Z error"], ep["Z error"])
    assert abs(ef["jk_E"] - ep["jk_E"]) < 5 * math.hypot(ef["jk_E error"], ep["jk_E error"])

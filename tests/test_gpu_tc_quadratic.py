"""GPU: the tensor-core quadratic coupling contraction (pbr_tc_quadratic) against an FP64 numpy
contraction, and the tensor-core block evaluation (pbr_sample_eval_tc) against the oracle, the
row-team form on the same samples, and itself under different chunkings.

Tolerances: the contraction keeps about 21 bits per product (TF32 hi/lo split, three MMAs) and
accumulates in FP32, so |vq - ref| <= 1e-5 * sum_k |q_d q_e| |Qp| per entry; the block
evaluation is held to the FP32 production tolerance (rtol 2e-4 on rho, g, g(beta +- db))."""
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


def _dims(N, A):
    import ctypes
    from pibronic_gb300 import _native
    n2p, a2p = ctypes.c_int32(), ctypes.c_int32()
    _native.check(_native.load().pbr_tc_quadratic_dims(N, A, ctypes.byref(n2p), ctypes.byref(a2p)), "dims")
    return n2p.value, a2p.value


@pytest.mark.parametrize("N,P,A,X,precision", [(12, 64, 4, 3, 32), (64, 8, 8, 41, 64), (1, 3, 1, 50, 32),
                                               (33, 17, 6, 9, 64), (20, 128, 5, 5, 32)])
def test_tc_quadratic_matches_fp64(N, P, A, X, precision):
    from pibronic_gb300 import _native
    lib = _native.load()
    rng = np.random.default_rng(N * 1000 + A)
    N2, A2 = N * (N + 1) // 2, A * (A + 1) // 2
    n2p, a2p = _dims(N, A)
    assert n2p >= N2 and n2p % 32 == 0 and a2p >= A2 and a2p % 16 == 0
    qq = rng.normal(0.0, 0.01, size=(N2, A2))
    q = rng.normal(0.0, 3.0, size=(X, N, P)).astype(np.float32)
    dt = torch.float32 if precision == 32 else torch.float64
    t_qq = torch.as_tensor(qq, dtype=dt).cuda().contiguous()
    t_q = torch.as_tensor(q).cuda().contiguous()
    bh = torch.empty((a2p, n2p), dtype=torch.float32, device="cuda")
    bl = torch.empty_like(bh)
    vq = torch.full((X * P, a2p), float("nan"), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    sh = _native.stream_handle()
    p = _native.ptr
    _native.check(lib.pbr_tc_pack_quadratic(p(t_qq), precision, N, A, p(bh), p(bl), sh), "pack")
    _native.check(lib.pbr_tc_quadratic(p(t_q), X, N, P, A, p(bh), p(bl), p(vq), p(st), sh), "tc_quadratic")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    # packed operands: hi + lo reproduce the FP32 couplings, padding is zero
    both = (bh + bl).double().cpu().numpy()
    assert np.allclose(both[:A2, :N2], qq.T.astype(np.float32), rtol=5e-7, atol=0)
    assert not both[A2:].any() and not both[:, N2:].any()
    d, e = np.tril_indices(N)                                   # row-major d >= e = pair_index order
    rows = q.astype(np.float64).transpose(0, 2, 1).reshape(X * P, N)
    prod = rows[:, d] * rows[:, e]
    ref = prod @ qq
    bound = np.abs(prod) @ np.abs(qq)
    got = vq.double().cpu().numpy()
    assert np.all(np.abs(got[:, :A2] - ref) <= 1e-5 * bound + 1e-30)


def _box(tmp_path, A, N, P, X, seed=7):
    from pibronic_gb300 import constants, pimc, synthetic, vibronic_io
    from pibronic_gb300.file_structure import FileStructure
    FS = FileStructure(str(tmp_path), 0, 0)
    model = synthetic.make_coupled_model(A, N, 3, sd_quadratic=0.0005)
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


@pytest.mark.parametrize("A,N,P", [(4, 12, 64), (8, 64, 16), (6, 48, 32), (2, 64, 8), (5, 33, 17), (1, 40, 12)])
def test_tc_form_against_oracle(tmp_path, A, N, P):
    from oracle import pimc_oracle as po
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    FS, data = _box(tmp_path, A, N, P, 32)
    plan = DevicePlan(data.prepared, precision=32, variant=DevicePlan.VARIANT_TC)
    assert plan.use_tc
    out = evaluate_device(plan, 32, seed=1, offset=0, want_q=True)
    assert int(out["status"].item()) == 0
    q = out["q"].double().cpu().numpy()
    box = po.OracleBox(po.model_from_file(FS.path_vib_model),
                       po.model_from_file(FS.path_rho_model, diagonal=True), 32, 32, P,
                       data.temperature, delta_beta=data.delta_beta, draw_sources=False)
    ref = box.evaluate(q)
    for k, rk in (("s_rho", "rho"), ("s_g", "g"), ("s_gp", "gP"), ("s_gm", "gM")):
        assert np.allclose(out[k].cpu().numpy(), ref[rk], rtol=2e-4, atol=0), k


def test_tc_form_draws_the_row_team_samples(tmp_path):
    """Same seed and offset: the same q and sources as the row-team form, rho identical, g within
    FP32 rounding."""
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    FS, data = _box(tmp_path, 6, 24, 32, 300)
    a = evaluate_device(DevicePlan(data.prepared, variant=2), 300, seed=4, offset=77, want_q=True)
    b = evaluate_device(DevicePlan(data.prepared, variant=3), 300, seed=4, offset=77, want_q=True)
    assert torch.equal(a["src"], b["src"])
    assert torch.equal(a["q"], b["q"])
    assert torch.equal(a["s_rho"], b["s_rho"])
    for k in ("s_g", "s_gp", "s_gm"):
        assert torch.allclose(a[k], b[k], rtol=2e-4, atol=0), k


def test_tc_form_chunking_and_capacity(tmp_path):
    """Outputs do not depend on the chunk the scratch allows; a scratch too small for one sample
    is a capacity error, not a launch."""
    from pibronic_gb300 import _native
    from pibronic_gb300.plan import DevicePlan
    FS, data = _box(tmp_path, 4, 40, 24, 1000)
    plan = DevicePlan(data.prepared, variant=3)
    lib = _native.load()
    X = 1000
    res = []
    for chunk in (7, 1000):
        nbytes = int(lib.pbr_sample_eval_tc_scratch(plan.struct, chunk))
        scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        outs = {k: torch.empty(X, dtype=torch.float64, device="cuda") for k in ("s_rho", "s_g", "s_gp", "s_gm")}
        o = _native.PbrOutputs()
        for k, v in outs.items():
            setattr(o, k, v.data_ptr())
        _native.check(lib.pbr_sample_eval_tc(plan.struct, 9, 5, X, o, scratch.data_ptr(), nbytes,
                                             _native.stream_handle()), "sample_eval_tc")
        res.append(outs)
    for k in res[0]:
        assert torch.equal(res[0][k], res[1][k]), k
    small = int(lib.pbr_sample_eval_tc_scratch(plan.struct, 1)) - 1
    scratch = torch.empty(small, dtype=torch.uint8, device="cuda")
    rc = lib.pbr_sample_eval_tc(plan.struct, 9, 5, X, o, scratch.data_ptr(), small, _native.stream_handle())
    assert rc == _native.PBR_ERR_CAPACITY

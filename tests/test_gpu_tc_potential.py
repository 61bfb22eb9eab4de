"""GPU: the tensor-core potential GEMM (pbr_tc_potential: energies, linear and quadratic
couplings) against an FP64 numpy contraction, and the tensor-core block evaluation
(pbr_sample_eval_tc) against the oracle, the row-team form on the same samples, and itself under
different chunkings.

Tolerances: the GEMM keeps about 22 bits per product (FP16 hi/lo split of both operands after
exact power-of-two scaling, three MMAs) and accumulates in FP32, so
|V - ref| <= 1e-5 * sum_k |a_k| |B_k| per entry; the block
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
    _native.check(_native.load().pbr_tc_potential_dims(N, A, ctypes.byref(n2p), ctypes.byref(a2p)), "dims")
    return n2p.value, a2p.value


def _quads(N):
    """K layout of the potential GEMM: quads (d, e0) over the slots [q, 0 .., 1 at NA, 0, 0, 0]."""
    na = (N + 3) // 4 * 4
    qs = [(d, e0) for d in range(N) for e0 in range(0, d + 1, 4)]
    qs += [(na, j0) for j0 in range(0, N, 4)] + [(na, na)]
    while len(qs) % 16:
        qs.append((na + 1, na))
    return qs, na


def _expected_operands(N, A2, qq, lin, en, q_rows):
    qs, na = _quads(N)
    K = 4 * len(qs)
    B = np.zeros((A2, K))
    slots = np.zeros((q_rows.shape[0], na + 4))
    slots[:, :N] = q_rows
    slots[:, na] = 1.0
    a = np.zeros((q_rows.shape[0], K))
    for i, (d, e0) in enumerate(qs):
        for u in range(4):
            k, e = 4 * i + u, e0 + u
            a[:, k] = slots[:, d] * slots[:, e] if d < na + 1 else 0.0
            if d < N and e <= d:
                B[:, k] = qq[d * (d + 1) // 2 + e]
            elif d == na and e0 < N and e < N and lin is not None:
                B[:, k] = lin[e]
            elif d == na and e0 == na and u == 0 and en is not None:
                B[:, k] = en
    return a, B


def _unpack(bp, mp, n2p):
    """b_packed (stages of 64 K columns, FP16 hi then lo, mp rows each, in the core layout; then
    the largest |coupling| and the FP32 scale 2^s_B) -> hi, lo [mp][n2p] (FP64) and the scale."""
    words = bp.cpu().numpy()
    h = words[:mp * n2p].view(np.float16).astype(np.float64)
    nst = n2p // 64
    hi, lo = np.zeros((mp, n2p)), np.zeros((mp, n2p))
    r = np.arange(mp)[:, None]
    k = np.arange(64)[None, :]
    idx = (((r // 8) * 8 + k // 8) * 8 + r % 8) * 8 + k % 8
    for st in range(nst):
        base = st * 2 * mp * 64
        for part, dst in ((0, hi), (1, lo)):
            blk = h[base + part * mp * 64: base + (part + 1) * mp * 64]
            dst[:, st * 64: (st + 1) * 64] = blk[idx]
    return hi, lo, float(words[mp * n2p + 1])


def _n_quads(N):
    """Quads before the padding: the energy quad is the last of them."""
    return sum((d + 4) // 4 for d in range(N)) + (N + 3) // 4 + 1


@pytest.mark.parametrize("N,P,A,X,precision,full", [(12, 64, 4, 3, 32, True), (64, 8, 8, 41, 64, True),
                                                    (1, 3, 1, 50, 32, True), (33, 17, 6, 9, 64, False),
                                                    (20, 128, 5, 5, 32, False), (64, 4, 12, 33, 32, True),
                                                    (30, 8, 16, 20, 64, True), (7, 40, 3, 300, 32, True)])
def test_tc_potential_matches_fp64(N, P, A, X, precision, full):
    from pibronic_gb300 import _native
    lib = _native.load()
    rng = np.random.default_rng(N * 1000 + A)
    N2, A2 = N * (N + 1) // 2, A * (A + 1) // 2
    n2p, a2p = _dims(N, A)
    assert n2p % 32 == 0 and a2p >= A2 and a2p % 16 == 0
    qq = rng.normal(0.0, 0.01, size=(N2, A2))
    lin = rng.normal(0.0, 0.05, size=(N, A2)) if full else None
    en = rng.normal(0.0, 0.3, size=A2) if full else None
    q = rng.normal(0.0, 3.0, size=(X, N, P)).astype(np.float32)
    dt = torch.float32 if precision == 32 else torch.float64
    dev = {k: (torch.as_tensor(v, dtype=dt).cuda().contiguous() if v is not None else None)
           for k, v in (("qq", qq), ("l", lin), ("e", en))}
    t_q = torch.as_tensor(q).cuda().contiguous()
    nbp = int(lib.pbr_tc_potential_packed_floats(N, A))
    mp = (nbp - 4) // n2p
    assert mp == a2p and nbp == a2p * n2p + 4
    bp = torch.full((nbp,), float("nan"), dtype=torch.float32, device="cuda")
    vq = torch.full((X * P, a2p), float("nan"), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    sh = _native.stream_handle()
    p = _native.ptr
    _native.check(lib.pbr_tc_pack_potential(p(dev["qq"]), p(dev["l"]) if full else None,
                                            p(dev["e"]) if full else None, precision, N, A, p(bp), sh), "pack")
    _native.check(lib.pbr_tc_potential(p(t_q), X, N, P, A, p(bp), p(vq), p(st), sh), "tc_potential")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    rows = q.astype(np.float64).transpose(0, 2, 1).reshape(X * P, N)
    a_op, B = _expected_operands(N, A2, qq, lin, en, rows)
    assert B.shape[1] == n2p
    # packed operands: (hi + lo) / 2^s_B reproduce the FP32 couplings in the documented layout;
    # the first padding row holds 1 at the energies' column, the rest of the padding is zero
    hi, lo, scale = _unpack(bp, mp, n2p)
    assert scale > 0 and np.log2(scale) == np.round(np.log2(scale))
    B32 = B.astype(np.float32).astype(np.float64)
    assert np.max(np.abs(B32) * scale) < 2.0 ** 14
    assert np.allclose((hi + lo)[:A2] / scale, B32, rtol=1e-6, atol=1e-7 * np.abs(B32).max())
    unit = np.zeros(n2p)
    unit[4 * (_n_quads(N) - 1)] = 1.0
    assert np.array_equal((hi + lo)[A2], unit)
    assert not (hi + lo)[A2 + 1:].any()
    ref = a_op @ B.T
    bound = np.abs(a_op) @ np.abs(B.T)
    got = vq.double().cpu().numpy()
    assert np.all(np.abs(got[:, :A2] - ref) <= 1e-5 * bound + 1e-30)
    if full:      # and the quadratic, linear, energy terms directly
        d, e = np.tril_indices(N)
        direct = (rows[:, d] * rows[:, e]) @ qq + rows @ lin + en[None, :]
        assert np.allclose(ref, direct, rtol=1e-10, atol=1e-12)


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


@pytest.mark.parametrize("A,N,P", [(4, 12, 64), (8, 64, 16), (6, 48, 32), (2, 64, 8), (5, 33, 17), (1, 40, 12),
                                   (12, 16, 16), (9, 10, 24), (16, 8, 12), (12, 64, 32), (13, 5, 3), (12, 20, 256),
                                   (12, 64, 256)])
def test_tc_form_against_oracle(tmp_path, A, N, P):
    """Row-team form for A <= 8, the wide form (exp(-tau V) by scaling and squaring) above."""
    from oracle import pimc_oracle as po
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    X = 4 if N * P > 8192 else 32          # the oracle's cost grows with N^2 P
    FS, data = _box(tmp_path, A, N, P, X)
    plan = DevicePlan(data.prepared, precision=32, variant=DevicePlan.VARIANT_TC)
    assert plan.use_tc
    out = evaluate_device(plan, X, seed=1, offset=0, want_q=True)
    assert int(out["status"].item()) == 0
    q = out["q"].double().cpu().numpy()
    box = po.OracleBox(po.model_from_file(FS.path_vib_model),
                       po.model_from_file(FS.path_rho_model, diagonal=True), X, X, P,
                       data.temperature, delta_beta=data.delta_beta, draw_sources=False)
    ref = box.evaluate(q)
    for k, rk in (("s_rho", "rho"), ("s_g", "g"), ("s_gp", "gP"), ("s_gm", "gM")):
        rel = np.max(np.abs(out[k].cpu().numpy() / ref[rk] - 1.0))
        print(f"A={A} N={N} P={P} {k}: max rel {rel:.2e}")
        assert rel <= 1e-4, (k, rel)


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


def test_sampler_row_streaming_form(tmp_path):
    """Samples too large to stage whole in shared memory (N = 64, P = 1024) are streamed by rows:
    finite bead coordinates, valid sources, and the counter-based stream splits by offset."""
    from pibronic_gb300 import _native
    lib = _native.load()
    FS, data = _box(tmp_path, 2, 64, 1024, 64)
    X, N, P = 64, 64, 1024
    q = torch.full((X, N, P), float("nan"), dtype=torch.float32, device="cuda")
    src = torch.full((X,), -1, dtype=torch.int32, device="cuda")
    _native.check(lib.pbr_sample_q(data.plan.struct, 3, 10, X, _native.ptr(q), _native.ptr(src),
                                   _native.stream_handle()), "sample_q rows")
    torch.cuda.synchronize()
    assert torch.isfinite(q).all()
    assert int(src.min()) >= 0 and int(src.max()) < 2
    # offsets split the stream: samples 10.. of seed 3 equal samples 0.. drawn at offset 10
    q2 = torch.empty((8, N, P), dtype=torch.float32, device="cuda")
    _native.check(lib.pbr_sample_q(data.plan.struct, 3, 14, 8, _native.ptr(q2), None, _native.stream_handle()),
                  "sample_q rows offset")
    torch.cuda.synchronize()
    assert torch.equal(q2, q[4:12])


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

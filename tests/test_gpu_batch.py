"""GPU: many independent models of uneven sizes and temperatures in one persistent launch per
surface count: each model's outputs match its own single-model evaluation on the same Philox
stream, the segmented reductions match per-model reductions, and a CUDA-graph replay reproduces
the direct run."""
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


def _models(seed, count):
    from pibronic_gb300 import constants, synthetic
    from pibronic_gb300.plan import PreparedModels
    rng = np.random.default_rng(seed)
    preps = []
    for i in range(count):
        A, N, P = int(rng.integers(2, 9)), int(rng.integers(3, 21)), int(rng.integers(8, 97))
        T = float(rng.uniform(100, 500))
        m = synthetic.make_coupled_model(A, N, 1000 + i, sd_quadratic=0.0005)
        beta = constants.beta(T)
        preps.append(PreparedModels(m, synthetic.diagonal_of(m), P, beta=beta, delta_beta=1e-4 * beta))
    return preps


def test_batch_matches_single_model_runs():
    from pibronic_gb300 import stats
    from pibronic_gb300.constants import boltzman
    from pibronic_gb300.batch import ModelBatch
    from pibronic_gb300.plan import DevicePlan
    from pibronic_gb300.pimc import evaluate_device
    preps = _models(3, 7)
    X = [300 + 37 * i for i in range(7)]
    seeds = [11 + i for i in range(7)]
    mb = ModelBatch(preps, X, seeds, offsets=[5 * i for i in range(7)])
    assert mb.groups >= 2
    mb.run()
    mb.reduce()
    torch.cuda.synchronize()
    assert int(mb.status.item()) == 0
    ests = mb.estimates()
    for i, prep in enumerate(preps):
        single = evaluate_device(DevicePlan(prep, precision=32, variant=2), X[i], seed=seeds[i], offset=5 * i)
        sl = slice(int(mb.seg[i]), int(mb.seg[i + 1]))
        for k in ("s_rho", "s_g", "s_gp", "s_gm"):
            assert torch.allclose(mb.out[k][sl], single[k], rtol=2e-4, atol=0), (i, k)
        ref = stats.device_estimates(mb.out["s_rho"][sl], mb.out["s_g"][sl], mb.out["s_gp"][sl],
                                     mb.out["s_gm"][sl], 1.0 / (prep.beta * boltzman), prep.delta_beta)
        for key in ("Z", "Z error", "E", "jk_E", "jk_E error"):
            assert np.isclose(ests[i][key], ref[key], rtol=1e-8), (i, key)


def test_batch_tensor_core_groups_match_single_model_runs():
    """Models with 5-8 surfaces and 16+ modes whose tiles need one block per SM form the
    tensor-core groups (bead records' quadratic part of V by mma.sync); each matches its own
    single-model evaluation."""
    from pibronic_gb300 import constants, synthetic
    from pibronic_gb300.batch import ModelBatch
    from pibronic_gb300.plan import DevicePlan, PreparedModels
    from pibronic_gb300.pimc import evaluate_device
    preps = []
    for i, (A, N, P) in enumerate([(7, 18, 24), (8, 16, 20), (6, 20, 128), (7, 9, 24), (3, 17, 40)]):
        m = synthetic.make_coupled_model(A, N, 2000 + i, sd_quadratic=0.0005)
        beta = constants.beta(250.0)
        preps.append(PreparedModels(m, synthetic.diagonal_of(m), P, beta=beta, delta_beta=1e-4 * beta))
    X = [257, 300, 64, 200, 333]
    seeds = [21 + i for i in range(5)]
    mb = ModelBatch(preps, X, seeds)
    mb.run()
    torch.cuda.synchronize()
    assert int(mb.status.item()) == 0
    for i, prep in enumerate(preps):
        single = evaluate_device(DevicePlan(prep, precision=32, variant=2), X[i], seed=seeds[i], offset=0)
        sl = slice(int(mb.seg[i]), int(mb.seg[i + 1]))
        for k in ("s_rho", "s_g", "s_gp", "s_gm"):
            assert torch.allclose(mb.out[k][sl], single[k], rtol=2e-4, atol=0), (i, k)


def test_batch_graph_replay_matches_direct_run():
    from pibronic_gb300.batch import ModelBatch
    preps = _models(5, 5)
    mb = ModelBatch(preps, [512] * 5, [7] * 5)
    mb.run()
    mb.reduce()
    torch.cuda.synchronize()
    direct = {k: v.clone() for k, v in mb.out.items()}
    mom = mb.moments.clone()
    for v in mb.out.values():
        v.zero_()
    mb.capture()
    mb.replay()
    torch.cuda.synchronize()
    for k in direct:
        assert torch.equal(mb.out[k], direct[k])
    assert torch.equal(mb.moments, mom)


def test_batch_dispatch_forms_match_single_model_runs():
    """One batch holding every dispatch path: register-chunk launches per model (up to 4
    surfaces), the two-block row-team build (5-6 surfaces whose tiles fit twice per SM), the
    one-block build (a 126 KB tile) and 8 surfaces -- each model against its own single-model run
    in the library's automatic form and in the row-team form."""
    from pibronic_gb300 import constants, synthetic
    from pibronic_gb300.batch import ModelBatch
    from pibronic_gb300.plan import DevicePlan, PreparedModels
    from pibronic_gb300.pimc import evaluate_device
    shapes = [(3, 6, 32), (4, 12, 64), (5, 16, 32), (6, 20, 128), (8, 8, 32), (6, 10, 32)]
    preps = []
    for i, (A, N, P) in enumerate(shapes):
        m = synthetic.make_coupled_model(A, N, 2000 + i, sd_quadratic=0.0005)
        beta = constants.beta(250.0 + 20 * i)
        preps.append(PreparedModels(m, synthetic.diagonal_of(m), P, beta=beta, delta_beta=1e-4 * beta))
    X = [700 + 13 * i for i in range(len(shapes))]
    seeds = [31 + i for i in range(len(shapes))]
    mb = ModelBatch(preps, X, seeds)
    assert mb.groups >= 5
    mb.run()
    torch.cuda.synchronize()
    assert int(mb.status.item()) == 0
    for i, prep in enumerate(preps):
        sl = slice(int(mb.seg[i]), int(mb.seg[i + 1]))
        for variant in (0, 2):
            single = evaluate_device(DevicePlan(prep, precision=32, variant=variant), X[i], seed=seeds[i], offset=0)
            for k in ("s_rho", "s_g", "s_gp", "s_gm"):
                assert torch.allclose(mb.out[k][sl], single[k], rtol=2e-4, atol=0), (shapes[i], variant, k)


def test_autotuner_times_every_candidate_per_surface_count_and_its_choice_is_exact():
    """autotune times each surface-count group under every candidate form / tile budget (at least
    three feasible per group), and a batch packed with its choices (and with every candidate
    forced on all groups) reproduces the single-model runs."""
    from pibronic_gb300 import constants, synthetic
    from pibronic_gb300.batch import ModelBatch, autotune, candidates
    from pibronic_gb300.plan import DevicePlan, PreparedModels
    from pibronic_gb300.pimc import evaluate_device
    shapes = [(2, 5, 24), (3, 6, 32), (5, 16, 48), (6, 20, 128), (7, 8, 40)]
    preps = []
    for i, (A, N, P) in enumerate(shapes):
        m = synthetic.make_coupled_model(A, N, 3000 + i, sd_quadratic=0.0005)
        beta = constants.beta(200.0 + 30 * i)
        preps.append(PreparedModels(m, synthetic.diagonal_of(m), P, beta=beta, delta_beta=1e-4 * beta))
    seeds = [41 + i for i in range(len(shapes))]
    budgets, times = autotune(preps, seeds, X_probe=512, reps=2)
    assert sorted(budgets) == sorted({s[0] for s in shapes})
    for A, tv in times.items():
        assert set(tv) == set(candidates(A))
        assert sum(v is not None for v in tv.values()) >= 3, (A, tv)
        assert budgets[A] in tv and tv[budgets[A]] is not None
    X = [400 + 11 * i for i in range(len(shapes))]
    singles = [evaluate_device(DevicePlan(p, precision=32, variant=2), X[i], seed=seeds[i], offset=0)
               for i, p in enumerate(preps)]
    tables = [budgets] + [{A: b for A in budgets} for b in (0, 72 * 1024, 48 * 1024)]
    for table in tables:
        mb = ModelBatch(preps, X, seeds, smem_budget=table)
        mb.run()
        torch.cuda.synchronize()
        assert int(mb.status.item()) == 0
        for i in range(len(preps)):
            sl = slice(int(mb.seg[i]), int(mb.seg[i + 1]))
            for k in ("s_rho", "s_g", "s_gp", "s_gm"):
                assert torch.allclose(mb.out[k][sl], singles[i][k], rtol=2e-4, atol=0), (table, shapes[i], k)

"""Multi-rank host path on CPU (gloo, world size 2): disjoint counter ranges and the moment merge
reproduce the single-process result exactly up to rounding, and the pooled jackknife of two ranks
(shard.pooled_moments with host restatements of the two reduction kernels) equals the reference's
jackknife (jackknife.py:60-105, in the oracle) over both ranks' samples together."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp


def _moments(r, s1, s2):
    out = [len(r)]
    for v in (r, s1, s2):
        out += [v.mean(), ((v - v.mean()) ** 2).sum()]
    return np.array(out, dtype=np.float64)


def _data(rank, world, X):
    from pibronic_gb300.shard import counter_offset
    start = counter_offset(3, rank, world, X)
    rng = np.random.default_rng(start)           # stands in for the rank's Philox range
    return rng.lognormal(size=X), rng.normal(1, 0.3, X), rng.normal(2, 0.5, X)


DB, T = 1e-2, 250.0


def _outputs(rank, world, X):
    """Per-sample rho, g, g(beta +- db) of a rank's shard (seeded stand-ins)."""
    from pibronic_gb300.shard import counter_offset
    rng = np.random.default_rng(counter_offset(5, rank, world, X) + 17)
    rho = rng.uniform(0.5, 1.5, X)
    g = rho * rng.lognormal(0.0, 0.3, X)
    e, c = rng.normal(0.2, 0.05, X), rng.normal(0.05, 0.02, X)
    return rho, g, g * np.exp(-DB * e + 0.5 * DB * DB * c), g * np.exp(DB * e + 0.5 * DB * DB * c)


def _terms(rho, g, gp, gm):
    return g / rho, (gp - gm) / (2 * DB * rho), (gp - 2 * g + gm) / (DB * DB * rho)


def _pass2(r, s1, s2, totals):
    """Host restatement of the jackknife kernel (pbr_reduce.cu jackknife_partial)."""
    from pibronic_gb300.constants import boltzman
    Sr, S1, S2 = totals
    E0 = -S1 / Sr
    inv_den = 1.0 / (Sr * (Sr - r))
    dE = (Sr * s1 - S1 * r) * inv_den
    dC = (-(Sr * s2 - S2 * r) * inv_den - dE * (2 * E0 + dE)) / (boltzman * T * T)
    return np.array([len(r), dE.mean(), ((dE - dE.mean()) ** 2).sum(), dC.mean(), ((dC - dC.mean()) ** 2).sum()])


def _pooled_worker(rank, world, port, X, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pibronic_gb300.shard import pooled_moments
    from pibronic_gb300.stats import estimates_from_moments
    t = _terms(*_outputs(rank, world, X))
    m, j = pooled_moments(lambda: _moments(*t), lambda totals: _pass2(*t, totals))
    q.put((rank, estimates_from_moments(m, j, T)))
    dist.barrier()
    dist.destroy_process_group()


def _worker(rank, world, port, X, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pibronic_gb300.shard import allgather_moments
    merged = allgather_moments(_moments(*_data(rank, world, X)))
    if rank == 0:
        q.put(merged)
    dist.barrier()
    dist.destroy_process_group()


def test_counter_ranges_are_disjoint_and_cover_the_stream():
    from pibronic_gb300.shard import counter_offset
    X, W = 1000, 4
    starts = sorted(counter_offset(s, r, W, X) for s in range(3) for r in range(W))
    assert starts == [i * X for i in range(3 * W)]


def test_merge_matches_single_pass():
    from pibronic_gb300.shard import merge_moments
    parts = [_data(r, 3, 5000) for r in range(3)]
    merged = merge_moments([_moments(*p) for p in parts])
    full = _moments(*[np.concatenate([p[k] for p in parts]) for k in range(3)])
    assert np.allclose(merged, full, rtol=1e-12)


@pytest.mark.timeout(120)
def test_two_rank_gloo_allgather():
    import socket
    from pibronic_gb300.shard import merge_moments
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, 4000, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=100)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = merge_moments([_moments(*_data(r, 2, 4000)) for r in range(2)])
    assert np.allclose(merged, ref, rtol=1e-14)


@pytest.mark.timeout(120)
def test_two_rank_pooled_jackknife_equals_the_reference_over_all_samples():
    import socket
    from oracle import stats_oracle as so
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    X, world = 3000, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_pooled_worker, args=(r, world, port, X, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=100) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    rho, g, gp, gm = (np.concatenate(a) for a in zip(*[_outputs(r, world, X) for r in range(world)]))
    terms = so.basic_terms(DB, rho, g, gp, gm)
    n = len(rho)
    basic = so.estimate_basic(n, T, *terms)
    jk = so.estimate_jackknife(n, T, DB, basic, *[so.jackknife_term(n, t) for t in terms])
    for est in got.values():                     # every rank holds the pooled estimates
        assert est["X"] == n
        assert np.isclose(est["Z"], basic["Z"], rtol=1e-12)
        assert np.isclose(est["Z error"], basic["Z error"], rtol=1e-9)
        for k in ("E", "Cv"):
            assert np.isclose(est["jk_" + k], jk[k], rtol=1e-8), (k, est["jk_" + k], jk[k])
            assert np.isclose(est["jk_" + k + " error"], jk[k + " error"], rtol=1e-6), k
    # a single rank's own jackknife is not the pooled one
    t0 = _terms(*_outputs(0, world, X))
    m0 = _moments(*t0)
    from pibronic_gb300.stats import estimates_from_moments
    own = estimates_from_moments(m0, _pass2(*t0, np.array([m0[1], m0[3], m0[5]]) * m0[0]), T)
    assert not np.isclose(own["jk_E error"], jk["E error"], rtol=1e-3)

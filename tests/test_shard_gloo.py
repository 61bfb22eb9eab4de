"""Multi-rank host path on CPU (gloo, world size 2): disjoint counter ranges and the moment merge
reproduce the single-process result exactly up to rounding."""
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

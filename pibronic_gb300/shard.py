"""Sharding the sample stream over ranks (one process per GPU).

Samples are independent: rank r of W takes the Philox counter range starting at
(step * W + r) * X for step ``step``, so the union of all ranks' samples is exactly the stream a
single GPU would draw for W times as many samples.  No collective touches the data path; the
only exchanges are merging the per-rank estimator moments (count, mean, M2 of r, s1, s2) with
Chan's pairwise formula, in rank order, after the work is done, and, for the jackknife errors of
all ranks' samples together, a second merge (``pooled_moments``): every rank runs the
jackknife's leave-one-out pass over its own samples against the totals of all samples, and the
(count, mean, M2) of the leave-one-out deviations are merged the same way (jackknife.py:60-105
over the union of the shards).
"""
from __future__ import annotations

import numpy as np


def counter_offset(step, rank, world, X):
    """First Philox sample counter of this rank's shard at this step."""
    return (int(step) * int(world) + int(rank)) * int(X)


def merge_moments(parts):
    """Merge [n, mean_r, M2_r, mean_s1, M2_s1, mean_s2, M2_s2] vectors (pbr_reduce_terms layout)
    in the given order."""
    parts = [np.asarray(p, dtype=np.float64) for p in parts]
    acc = parts[0].copy()
    for p in parts[1:]:
        na, nb = acc[0], p[0]
        if nb == 0:
            continue
        if na == 0:
            acc = p.copy()
            continue
        n = na + nb
        out = np.empty_like(acc)
        out[0] = n
        for k in range(1, len(acc), 2):
            d = p[k] - acc[k]
            out[k] = acc[k] + d * nb / n
            out[k + 1] = acc[k + 1] + p[k + 1] + d * d * na * nb / n
        acc = out
    return acc


def allgather_moments(moments, group=None):
    """Gather every rank's moment vector (torch.distributed, any backend) and merge in rank order."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    t = torch.as_tensor(np.asarray(moments, dtype=np.float64))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    out = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(out, t, group=group)
    return merge_moments([o.cpu().numpy() for o in out])


def pooled_moments(pass1, pass2, group=None):
    """Estimator moments and jackknife moments over every rank's samples.

    pass1() returns this rank's [n, mean, M2] x (r, s1, s2) vector; the vectors of all ranks are
    merged in rank order, so every rank holds the same global moments.  pass2(totals) runs the
    jackknife pass over this rank's samples with the global totals S_r, S_1, S_2 (the leave-one-out
    estimator of sample i is -(S_1 - s1_i) / (S_r - r_i), which needs only the totals) and returns
    [n, mean dE, M2 dE, mean dC, M2 dC]; those are merged in rank order as well.  Without an
    initialised process group (or with one rank) this is the single-process reduction."""
    import torch.distributed as dist
    distributed = dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1
    local = pass1()
    m = allgather_moments(local, group) if distributed else np.asarray(local, dtype=np.float64)
    totals = np.array([m[1], m[3], m[5]], dtype=np.float64) * m[0]
    jl = pass2(totals)
    j = allgather_moments(jl, group) if distributed else np.asarray(jl, dtype=np.float64)
    return m, j

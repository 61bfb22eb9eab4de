"""Sharding the sample stream over ranks (one process per GPU).

Samples are independent: rank r of W takes the Philox counter range starting at
(step * W + r) * X for step ``step``, so the union of all ranks' samples is exactly the stream a
single GPU would draw for W times as many samples.  No collective touches the data path; the
only exchange is merging the per-rank estimator moments (count, mean, M2 of r, s1, s2) with
Chan's pairwise formula, in rank order, after the work is done.
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

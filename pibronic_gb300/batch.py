"""Many independent models in one persistent launch per surface count.

Each model keeps its own sizes (A, N, P), temperature, seed, counter offset and sample count;
``ModelBatch.run`` evaluates all of them with ``pbr_sample_eval_batch`` (CTAs take the
concatenated sample tiles round-robin and reload a model's tables when the model changes) and
``reduce`` turns every model's samples into Z, E, Cv with jackknife errors by segmented device
reductions.  ``capture`` records both in a CUDA graph for replay.  ``autotune`` picks, per
surface count, the kernel form and the shared-memory budget that fixes the models' tile shape
(samples per tile, hence CTAs per SM and, at 5-6 surfaces, the two-block build) by timing each
surface-count group alone for every candidate on a small sample count.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _native
from .constants import boltzman
from .plan import DevicePlan
from .stats import estimates_from_moments


#: budget value that selects the per-model register-chunk launches (up to 4 surfaces)
CHUNKS = -1
MAX_A = 8


def budget_table(smem_budget):
    """Per-surface-count budgets (index = surface count) from None (register chunks up to 4
    surfaces, whole shared memory beyond), an int (that budget for the row-team groups, register
    chunks up to 4 surfaces) or a dict {A: budget} (missing entries as for None)."""
    table = [0] + [CHUNKS if a <= 4 else 0 for a in range(1, MAX_A + 1)]
    if isinstance(smem_budget, dict):
        for a, b in smem_budget.items():
            table[int(a)] = int(b)
    elif smem_budget:
        table = [0] + [CHUNKS if a <= 4 else int(smem_budget) for a in range(1, MAX_A + 1)]
    return table


class ModelBatch:
    def __init__(self, preps, X, seeds, offsets=None, smem_budget=None, grid_cap=0, plans=None):
        torch = _native.require_cuda()
        lib = _native.load()
        self.preps = list(preps)
        M = len(self.preps)
        self.X = np.asarray(X, dtype=np.int64).reshape(M)
        self.seeds = np.asarray(seeds, dtype=np.uint64).reshape(M)
        self.offsets = np.zeros(M, dtype=np.uint64) if offsets is None else np.asarray(offsets, dtype=np.uint64)
        assert all(p.K == self.preps[0].K for p in self.preps), "one series order per batch"
        self.K = self.preps[0].K
        self.plans = list(plans) if plans is not None else [DevicePlan(p, precision=32) for p in self.preps]
        dev = torch.device("cuda", torch.cuda.current_device())
        self.seg = np.concatenate([[0], np.cumsum(self.X)]).astype(np.int64)
        total = int(self.seg[-1])
        f64 = dict(dtype=torch.float64, device=dev)
        self.out = {k: torch.empty(total, **f64) for k in ("s_rho", "s_g")}
        if self.K > 0:
            self.out.update({k: torch.empty(total, **f64) for k in ("s_gp", "s_gm")})
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        outs = (_native.PbrOutputs * M)()
        models = (_native.PbrModel * M)()
        es = {k: v.element_size() for k, v in self.out.items()}
        for m in range(M):
            models[m] = self.plans[m].struct
            o = outs[m]
            for k, v in self.out.items():
                setattr(o, k, v.data_ptr() + int(self.seg[m]) * es[k])
            o.status = self.status.data_ptr()
        self._models, self._outs = models, outs
        self.smem_budget, self.grid_cap = smem_budget, grid_cap
        self._pack(smem_budget, grid_cap)
        # segmented reductions
        self.t_seg = torch.as_tensor(self.seg, dtype=torch.int64, device=dev)
        self.t_db = torch.as_tensor([p.delta_beta for p in self.preps], **f64)
        self.T = np.array([1.0 / (p.beta * boltzman) for p in self.preps])
        self.t_kT2 = torch.as_tensor(boltzman * self.T ** 2, **f64)
        self.scratch = torch.empty(int(lib.pbr_reduce_segments_scratch(M)) + 16, **f64)
        self.moments = torch.empty((M, 7), **f64)
        self.jk = torch.empty((M, 5), **f64)
        self.graph = None

    def _pack(self, smem_budget, grid_cap):
        torch = _native.require_cuda()
        lib = _native.load()
        M = len(self.preps)
        nbytes = int(lib.pbr_batch_blob_bytes(M))
        self._host_blob = ctypes.create_string_buffer(nbytes)
        X = (ctypes.c_int64 * M)(*[int(v) for v in self.X])
        seeds = (ctypes.c_uint64 * M)(*[int(v) for v in self.seeds])
        offs = (ctypes.c_uint64 * M)(*[int(v) for v in self.offsets])
        self.budgets = budget_table(smem_budget)
        table = (ctypes.c_int32 * len(self.budgets))(*self.budgets)
        rc = lib.pbr_batch_pack(self._models, seeds, offs, X, self._outs, M, table, int(grid_cap),
                                self._host_blob)
        _native.check(rc, "pbr_batch_pack")
        host = torch.frombuffer(bytearray(self._host_blob.raw), dtype=torch.uint8)
        self._dev_blob = host.to("cuda")
        self.groups = int(lib.pbr_batch_groups(self._host_blob))

    def run(self, stream=None):
        lib = _native.load()
        _native.check(lib.pbr_sample_eval_batch(self._host_blob, ctypes.c_void_p(self._dev_blob.data_ptr()),
                                                _native.stream_handle(stream)), "pbr_sample_eval_batch")

    def reduce(self, stream=None):
        lib = _native.load()
        p = _native.ptr
        sh = _native.stream_handle(stream)
        M = len(self.preps)
        o = self.out
        _native.check(lib.pbr_reduce_terms_segments(p(o["s_rho"]), p(o["s_g"]), p(o.get("s_gp")), p(o.get("s_gm")),
                                                    p(self.t_seg), M, p(self.t_db), p(self.scratch),
                                                    p(self.moments), sh), "segment reduction")
        if self.K > 0:
            _native.check(lib.pbr_reduce_jackknife_segments(p(o["s_rho"]), p(o["s_g"]), p(o["s_gp"]), p(o["s_gm"]),
                                                            p(self.t_seg), M, p(self.t_db), p(self.t_kT2),
                                                            p(self.moments), p(self.scratch), p(self.jk), sh),
                          "segment jackknife")

    def capture(self):
        """Record run + reduce in a CUDA graph (warmed up first on a side stream)."""
        torch = _native.require_cuda()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run(s)
            self.reduce(s)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.run(s)
            self.reduce(s)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def estimates(self):
        m = self.moments.cpu().numpy()
        j = self.jk.cpu().numpy() if self.K > 0 else [None] * len(self.preps)
        return [estimates_from_moments(m[i], j[i], self.T[i]) for i in range(len(self.preps))]


def candidates(A):
    """Kernel forms and shared-memory budgets tried for a surface count: up to 4 surfaces the
    register-chunk launches and three row-team tile budgets, beyond that five row-team budgets
    (at 5-6 surfaces the smaller ones let two tiles share an SM)."""
    if A <= 4:
        return (CHUNKS, 0, 110 * 1024, 72 * 1024)
    return (0, 150 * 1024, 110 * 1024, 72 * 1024, 48 * 1024)


def autotune(preps, seeds, X_probe=2048, reps=3):
    """For each surface count of the batch, time that group's models alone (X_probe samples each)
    under every candidate of ``candidates`` and keep the fastest.  Returns (budgets {A: budget},
    times {A: {budget: seconds}}); a candidate the library refuses is recorded as None."""
    torch = _native.require_cuda()
    plans = [DevicePlan(p, precision=32) for p in preps]
    budgets, times = {}, {}
    for A in sorted({p.A for p in preps}):
        idx = [i for i, p in enumerate(preps) if p.A == A]
        sub = [preps[i] for i in idx]
        subp = [plans[i] for i in idx]
        subs = [seeds[i] for i in idx]
        times[A] = {}
        for b in candidates(A):
            try:
                mb = ModelBatch(sub, [X_probe] * len(sub), subs, smem_budget={A: b}, plans=subp)
                mb.run()
            except AssertionError:
                times[A][b] = None
                continue
            torch.cuda.synchronize()
            best = float("inf")
            for _ in range(reps):
                t0 = time.perf_counter()
                mb.run()
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t0)
            times[A][b] = best
        ok = {b: t for b, t in times[A].items() if t is not None}
        budgets[A] = min(ok, key=ok.get)
    return budgets, times

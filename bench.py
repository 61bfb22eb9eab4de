#!/usr/bin/env python
"""Benchmark: effective samples per second of the PIMC block evaluation on GB300.

Workload (the headline configuration): synthetic seeded vibronic model A=4 surfaces, N=12 modes,
P=64 beads, T=300 K, delta_beta = 1e-4 beta, X = 1e6 samples per step per GPU, plain rho
proposal.  One step = one fused launch that draws and evaluates X samples (rho, g, g(beta+-db))
plus the two FP64 reduction passes that turn them into Z, E, Cv with jackknife errors.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  value = ESS/s summed over ranks, ESS = (sum w)^2 / sum w^2 of w = g/rho.
--impl reference times the CPU restatement of the reference engine (the oracle port of
pibronic/pimc/pimc.py block_compute_pm) on all host cores on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

METRIC = "ESS/sec for Z,E,Cv at 1e-3 rel err: learned vs plain rho, 1 GB300"
A_, N_, P_, T_ = 4, 12, 64, 300.0
MODEL_SEED = 20240


def flops_per_sample(A, N, P):
    """Algorithmic work per sample: ring transform 2NP^2, four O sets 24ANP, V P(2N^2A^2 + 2NA^2),
    eigh 10PA^3, M 2PA^3, three ring products 3P(2A^3 + A^2)."""
    return (2 * N * P * P + 24 * A * N * P + P * (2 * N * N * A * A + 2 * N * A * A)
            + 10 * P * A ** 3 + 2 * P * A ** 3 + 3 * P * (2 * A ** 3 + A * A))


# ---------------------------------------------------------------------------------------------
# CPU side: the oracle port (reference arm and cpu_baseline)
# ---------------------------------------------------------------------------------------------
def _cpu_worker(args):
    vib_text, rho_text, X, P, T, db_rel, seed = args
    import numpy as np
    from oracle import pimc_oracle as po
    np.random.seed(seed)
    vib = po.model_from_text(vib_text)
    rho = po.model_from_text(rho_text, diagonal=True)
    beta = po.beta_of(T)
    box = po.OracleBox(vib, rho, X, min(X, 10_000), P, T, delta_beta=db_rel * beta)
    t0 = time.perf_counter()
    res = box.block_compute(plus_minus=True)
    el = time.perf_counter() - t0
    return el, res["s_rho"], res["s_g"], res["s_gP"], res["s_gM"]


def cpu_port_run(vib_text, rho_text, samples_per_worker, workers, seed0=0):
    """One bounded sample of the workload on `workers` processes (spawned); returns
    (samples/s, ESS/s, ESS/X, wall seconds, cpu seconds)."""
    import multiprocessing as mp
    import numpy as np
    for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"          # one BLAS thread per spawned process
    ctx = mp.get_context("spawn")
    jobs = [(vib_text, rho_text, samples_per_worker, P_, T_, 1e-4, 1000 + seed0 + i)
            for i in range(workers)]
    with ctx.Pool(workers) as pool:
        t0 = time.perf_counter()
        outs = pool.map(_cpu_worker, jobs)
        wall = time.perf_counter() - t0
    busy = max(o[0] for o in outs)
    r = np.concatenate([o[2] / o[1] for o in outs])
    ess_frac = r.sum() ** 2 / (r * r).sum() / len(r)
    sps = len(r) / busy
    return sps, sps * ess_frac, ess_frac, wall, sum(o[0] for o in outs)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def model_texts():
    from pibronic_gb300 import synthetic, vibronic_io
    root = tempfile.mkdtemp(prefix="pbr_bench_")
    from pibronic_gb300.file_structure import FileStructure
    FS = FileStructure(root, 0, 0)
    synthetic.write_model_pair(FS, A_, N_, MODEL_SEED)
    with open(FS.path_vib_model) as fh:
        vt = fh.read()
    with open(FS.path_rho_model) as fh:
        rt = fh.read()
    return FS, vt, rt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    _, vt, rt = model_texts()
    cores = host_cores()
    per_worker = args.cpu_samples
    for w in range(args.warmup):
        cpu_port_run(vt, rt, max(20, per_worker // 4), cores, seed0=10_000 * (w + 1))
    vals, sps_l, fr = [], [], []
    t_all = time.perf_counter()
    for s in range(args.steps):
        sps, ess_s, ess_frac, wall, cpu = cpu_port_run(vt, rt, per_worker, cores, seed0=100 * s)
        vals.append(ess_s)
        sps_l.append(sps)
        fr.append(ess_frac)
    elapsed = time.perf_counter() - t_all
    value = statistics.mean(vals)
    sample = (f"{args.steps} steps x {cores} spawned processes x {per_worker} samples of the "
              f"workload (oracle port of block_compute_pm, FP64 numpy), preprocess excluded")
    line = {
        "metric": METRIC, "value": value, "unit": "ESS/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * elapsed / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(),
        "samples_per_s": statistics.mean(sps_l), "ess_per_sample": statistics.mean(fr),
        "cpu_baseline": {"value": value, "unit": "ESS/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "ESS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_config():
    return {"workload": f"plain-rho PIMC block evaluation (block_compute_pm): A={A_} N={N_} P={P_} "
                        f"T={T_:.0f}K dbeta=1e-4*beta, 1e6 samples per step per GPU",
            "A": A_, "N": N_, "P": P_, "T": T_, "X_per_gpu": 1_000_000, "model_seed": MODEL_SEED,
            "proposal": "rho (plain)", "l2": "flushed between timed steps (256 MB write)"}


# ---------------------------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms.  start() returns once the first
    sample is on file (nvidia-smi takes a moment to come up); mark() at the start of the timed
    region sets aside the samples taken before it, so the median is of samples under load."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 100

    def __init__(self, index):
        self.index, self.proc, self.path, self.skip = index, None, None, 0

    def _lines(self):
        with open(self.path) as fh:
            return [ln for ln in fh.read().split("\n")[:-1] if ln.strip()]

    def start(self, wait_s=5.0):
        try:
            fd, self.path = tempfile.mkstemp(prefix="pbr_clk_", suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t_end = time.monotonic() + wait_s
        while time.monotonic() < t_end and self.proc.poll() is None and not self._lines():
            time.sleep(0.02)

    def mark(self):
        """Samples on file now were taken before the timed region."""
        if self.proc is not None:
            self.skip = len(self._lines())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for i, line in enumerate(self._lines()):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                try:
                    rows.append((i, float(parts[0]), float(parts[1]), parts[3:7]))
                except ValueError:
                    pass
        os.unlink(self.path)
        inside = [r for r in rows if r[0] >= self.skip]
        # a timed region shorter than the period may hold no sample: report the last one before
        # it, with samples = 0
        use = inside if inside else rows[-1:]
        if not use:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, _, f in use for i, v in enumerate(f) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in use), "sm_max_mhz": max(r[2] for r in use),
                "reasons": reasons, "samples": len(inside), "period_ms": self.PERIOD_MS}


def fp32_peak(torch, lib, stream):
    """Measured FP32 FMA peak (TFLOP/s) of this GPU with the library's FFMA probe."""
    from pibronic_gb300 import _native
    import ctypes
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    out = torch.empty(sms * 8, dtype=torch.float32, device="cuda")
    fl = ctypes.c_double()
    best = 0.0
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _native.check(lib.pbr_fma_probe(_native.ptr(out), sms * 8, 4096, ctypes.byref(fl),
                                        _native.stream_handle(stream)), "fma probe")
        e1.record(stream)
        e1.synchronize()
        best = max(best, fl.value / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def measured_hbm_gbs():
    """(HBM copy bandwidth in GB/s, where it came from): the pool's measured figure when
    MEASURED_PEAKS.json is present, else the fallback of one earlier GB300 measurement."""
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def read_traffic():
    """DRAM bytes (read + write) of one 1e6-sample fused launch, measured by ncu on this bench's
    own command (the launch list in profiles/fused_config2_ncu.md), if that summary is present."""
    path = os.path.join(HERE, "profiles", "fused_config2_ncu.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def run_ours(args):
    import numpy as np
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from pibronic_gb300 import _native, pimc, stats
    from pibronic_gb300.build import build
    lib = _native.load(build() if rank == 0 and world == 1 else None)
    X = args.samples
    FS, vt, rt = model_texts() if rank == 0 else (None, None, None)
    if world > 1:
        obj = [vt, rt]
        dist.broadcast_object_list(obj, src=0)
        vt, rt = obj
        root = tempfile.mkdtemp(prefix=f"pbr_bench_r{rank}_")
        from pibronic_gb300.file_structure import FileStructure
        FS = FileStructure(root, 0, 0)
        open(FS.path_vib_model, "w").write(vt)
        open(FS.path_rho_model, "w").write(rt)
    # the public API: BoxDataPM from the model files, preprocess builds the device plan
    from pibronic_gb300 import constants
    beta = constants.beta(T_)
    data = pimc.BoxDataPM(1e-4 * beta)
    data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
    data.states, data.modes, data.beads, data.temperature = A_, N_, P_, T_
    data.samples, data.block_size = X, 10_000
    data.blocks = X // data.block_size
    data.seed = 0x5EED + rank
    data.preprocess()
    from pibronic_gb300.plan import DevicePlan
    plan = DevicePlan(data.prepared, precision=32, variant=args.variant) if args.variant else data.plan
    stream = torch.cuda.current_stream()
    dev = torch.device("cuda", local)
    bufs = {k: torch.empty(X, dtype=torch.float64, device=dev) for k in ("s_rho", "s_g", "s_gp", "s_gm")}
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    o = _native.PbrOutputs()
    o.s_rho, o.s_g = bufs["s_rho"].data_ptr(), bufs["s_g"].data_ptr()
    o.s_gp, o.s_gm = bufs["s_gp"].data_ptr(), bufs["s_gm"].data_ptr()
    o.status = status.data_ptr()
    red = stats.DeviceReducer(X)
    sh = _native.stream_handle(stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    hist = torch.empty((args.steps + args.warmup, 12), dtype=torch.float64, device=dev)

    from pibronic_gb300.shard import allgather_moments, counter_offset

    def step(i, e_k0=None, e_k1=None):
        offset = counter_offset(i, rank, world, X)
        if e_k0 is not None:
            e_k0.record(stream)
        _native.check(lib.pbr_sample_eval(plan.struct, data.seed, offset, X, o, sh), "sample_eval")
        if e_k1 is not None:
            e_k1.record(stream)
        red.launch(bufs["s_rho"], bufs["s_g"], bufs["s_gp"], bufs["s_gm"], data.delta_beta, T_, stream)
        hist[i, :7].copy_(red.moments)
        hist[i, 7:].copy_(red.jk)

    for w in range(args.warmup):
        step(w)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    clocks.mark()
    for s in range(args.steps):
        flush.fill_(float(s))                      # L2 flush between timed steps (untimed)
        e0, e1, e2 = ev[s]
        step(args.warmup + s, e0, e1)
        e2.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    step_ms = [e0.elapsed_time(e2) for e0, _, e2 in ev]
    kern_ms = [e0.elapsed_time(e1) for e0, e1, _ in ev]
    ms_step = sum(step_ms) / len(step_ms)
    ms_kern = sum(kern_ms) / len(kern_ms)
    if int(status.item()) != 0:
        raise RuntimeError("non-finite results in the timed steps")
    H = hist.cpu().numpy()[args.warmup:]
    ests = [stats.estimates_from_moments(h[:7], h[7:], T_) for h in H]
    if dist:
        # per step, the ESS of all ranks' samples together: merge the moments in rank order
        ess_total = statistics.mean(
            stats.estimates_from_moments(allgather_moments(h[:7]), None, T_)["ESS"] for h in H)
        tmax = torch.tensor([ms_step], dtype=torch.float64, device=dev)
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        ms_step = float(tmax[0])
    else:
        ess_total = statistics.mean(e["ESS"] for e in ests)
    value = ess_total / (ms_step * 1e-3)
    sps = X * world / (ms_step * 1e-3)
    # the last step's estimates over all ranks' samples: moments merged in rank order and the
    # jackknife pass of every rank against the global totals (after the timed region)
    e = red.pooled(bufs["s_rho"], bufs["s_g"], bufs["s_gp"], bufs["s_gm"], data.delta_beta, T_) if dist \
        else ests[-1]
    rel = {"Z": e["Z error"] / abs(e["Z"]), "E": e["jk_E error"] / abs(e["jk_E"]),
           "Cv": e["jk_Cv error"] / abs(e["jk_Cv"])}
    t_1e3 = {k: X * world * (v / 1e-3) ** 2 / sps for k, v in rel.items()}

    # ---- e2e through the public API with host buffers ----
    # Every step copies its inputs (the model tables) from pinned host memory, evaluates, reduces,
    # and copies its four per-sample arrays and its moments back to pinned host memory.  Two
    # output sets alternate, so step s's device->host copies (on a copy stream) overlap step s+1's
    # evaluation; the host clock runs from the first step's input copy to the last step's results
    # on the host.
    e2e_val, h2d, d2h = None, 0, 0
    tab_host = {k: v.cpu().pin_memory() for k, v in plan.tensors.items()}
    h2d = sum(v.numel() * v.element_size() for v in tab_host.values())
    copy_stream = torch.cuda.Stream(device=dev)
    sets = []
    for b in range(2):
        bb = bufs if b == 0 else {k: torch.empty_like(v) for k, v in bufs.items()}
        ob = o if b == 0 else _native.PbrOutputs()
        if b:
            ob.s_rho, ob.s_g = bb["s_rho"].data_ptr(), bb["s_g"].data_ptr()
            ob.s_gp, ob.s_gm = bb["s_gp"].data_ptr(), bb["s_gm"].data_ptr()
            ob.status = status.data_ptr()
        sets.append({"bufs": bb, "out": ob, "red": red if b == 0 else stats.DeviceReducer(X),
                     "host": {k: torch.empty(X, dtype=torch.float64, pin_memory=True) for k in bufs},
                     "mom": torch.empty(7, dtype=torch.float64, pin_memory=True),
                     "jk": torch.empty(5, dtype=torch.float64, pin_memory=True),
                     "done": torch.cuda.Event(), "copied": torch.cuda.Event(), "used": False})
    d2h = sum(v.numel() * v.element_size() for v in sets[0]["host"].values()) + 12 * 8
    n_e2e = max(2, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(n_e2e):
        S = sets[s % 2]
        if S["used"]:
            stream.wait_event(S["copied"])            # this set's previous results are on the host
        for k, v in tab_host.items():                 # the step's inputs: model tables
            plan.tensors[k].copy_(v, non_blocking=True)
        _native.check(lib.pbr_sample_eval(plan.struct, data.seed + 1, counter_offset(s, rank, world, X), X,
                                          S["out"], sh), "sample_eval")
        b = S["bufs"]
        S["red"].launch(b["s_rho"], b["s_g"], b["s_gp"], b["s_gm"], data.delta_beta, T_, stream)
        S["done"].record(stream)
        copy_stream.wait_event(S["done"])
        with torch.cuda.stream(copy_stream):
            for k in b:
                S["host"][k].copy_(b[k], non_blocking=True)
            S["mom"].copy_(S["red"].moments, non_blocking=True)
            S["jk"].copy_(S["red"].jk, non_blocking=True)
            S["copied"].record(copy_stream)
        S["used"] = True
    copy_stream.synchronize()
    torch.cuda.synchronize()
    e2e_t = (time.perf_counter() - t0) / n_e2e
    last = sets[(n_e2e - 1) % 2]
    ee = stats.estimates_from_moments(last["mom"].numpy(), last["jk"].numpy(), T_)
    if not (ee["Z"] > 0):
        raise RuntimeError("e2e results not finite")
    if dist:
        tt = torch.tensor([e2e_t], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_t = float(tt[0])
    e2e_val = ess_total / e2e_t

    # ---- roofline of the fused kernel ----
    W = flops_per_sample(A_, N_, P_)
    achieved = W * X / (ms_kern * 1e-3) / 1e12
    peak = fp32_peak(torch, lib, stream)
    traffic = read_traffic()
    hbm = measured_hbm_gbs()
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 1e6-sample launch "
                              "of this command (profiles/fused_config2_ncu.md); the outputs stay in L2",
            "algorithmic_bytes": 32 * X,
            "peak_source": "FP32 FFMA probe (pbr_fma_probe) measured in this run; "
                           "MEASURED_PEAKS.json has only HBM copy and bf16 tensor peaks",
            "flops_per_sample": W, "kernel_ms": ms_kern,
            "hbm_frac_of_measured": (32.0 * X / (ms_kern * 1e-3) / 1e9) / hbm[0], "hbm_peak_source": hbm[1]}
    line = {
        "metric": METRIC, "value": value, "unit": "ESS/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(),
        "samples_per_s": sps, "ess_per_sample": ess_total / (X * world),
        "rel_err": rel, "time_to_1e-3_s": t_1e3, "estimates_over": f"{world} rank(s), {X * world} samples",
        "estimates": {k: e[k] for k in ("Z", "Z error", "E", "jk_E", "jk_E error", "Cv", "jk_Cv", "jk_Cv error")},
        "roofline": roof,
        "e2e": {"value": e2e_val, "unit": "ESS/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1e3 * e2e_t},
        "clocks": clk, "gpu_launches": 5 * args.steps,
    }
    # ---- FP32 against the FP64 build on identical q at 100, 300, 500 K ----
    if rank == 0 and not args.no_precision:
        line["precision"] = precision_leg(args)
    # ---- learned proposal vs plain rho (A=6, N=20, P=128, T=200 K, strong couplings) ----
    if rank == 0 and not args.no_learned:
        line["learned"] = learned_leg(args)
    # ---- batched uneven models in one graph-captured launch per surface count ----
    if rank == 0 and not args.no_batched:
        line["batched"] = batched_leg(args)
    # ---- large dense configuration on the tensor-core form (A=12, N=64, P=256) ----
    if rank == 0 and not args.no_large:
        line["large"] = large_leg(args)
    # ---- CPU baseline: the oracle port on the host cores, rank 0 at N=1 only ----
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = host_cores()
        sps_c, ess_c, frac_c, wall, cpu = cpu_port_run(vt, rt, args.cpu_samples, cores)
        line["cpu_baseline"] = {
            "value": ess_c, "unit": "ESS/s", "cores": cores, "kind": "port",
            "samples_per_s": sps_c,
            "sample": f"{cores} spawned processes x {args.cpu_samples} samples of the same workload "
                      f"(oracle port of block_compute_pm, FP64 numpy), {cpu:.1f} s of CPU work"}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def _timed(torch, fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, time.perf_counter() - t0


def _warm_training(torch, FlowProposal, prepared, plan, nsel, y, r):
    """A throwaway proposal of the same shapes through both training rounds (two steps each) and
    its own sampling: on a fresh box the first use of some PyTorch kernels compiles them (seconds),
    which would otherwise land in train_s."""
    n = min(y.shape[0], 2 * 16384)
    warm = FlowProposal(prepared, plan, nsel=nsel, layers=8, hidden=128, seed=1)
    warm.train(y[:n].contiguous(), r[:n].contiguous(), epochs=1, batch=min(16384, n), lr=1e-3)
    own = warm.sample_and_evaluate(n, seed=3, keep=True)
    warm.train(own["y"], own["s_g"] / own["s_q"], epochs=1, batch=min(16384, n), lr=1e-3)
    torch.cuda.synchronize()


def rate_summary(e, t, X, train_s=0.0):
    """ESS/s, samples/s, estimates and the wall time to 1e-3 relative error of Z, E and Cv at the
    measured rate (X (rel / 1e-3)^2 samples), plus train_s when given.  A quantity within 3 of its
    statistical errors of zero has no meaningful relative error: its time is None."""
    out = {"samples": X, "ess_per_sample": e["ESS"] / X, "ess_per_s": e["ESS"] / t, "samples_per_s": X / t,
           "Z": e["Z"], "Z error": e["Z error"], "E": e["jk_E"], "E error": e["jk_E error"],
           "Cv": e["jk_Cv"], "Cv error": e["jk_Cv error"]}
    times = {}
    for k, v, err in (("Z", e["Z"], e["Z error"]), ("E", e["jk_E"], e["jk_E error"]),
                      ("Cv", e["jk_Cv"], e["jk_Cv error"])):
        times[k] = None if abs(v) < 3.0 * err else train_s + X * (err / abs(v) / 1e-3) ** 2 / (X / t)
    out["time_to_1e-3_s"] = times
    return out


def _chunked(torch, fn, X, chunk):
    """Run fn(n, offset) over X samples in chunks; returns (concatenated outputs, seconds)."""
    outs = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for off in range(0, X, chunk):
        outs.append(fn(min(chunk, X - off), off))
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    keys = ("s_rho", "s_q", "s_g", "s_gp", "s_gm")
    return {k: torch.cat([o[k] for o in outs]) for k in keys if k in outs[0]}, t


#: epochs of each training round of the learned configuration: measured on GB300, 3 epochs per
#: round give the same ESS/sample as 6 (0.886 against 0.883 on the strongly coupled model, 0.936
#: against 0.927 on seed 44) in half the time, 2 epochs 1-2 % less; the second round (on the flow's
#: own samples) is what lifts ESS/sample from ~0.6 to ~0.88 on the strongly coupled model
LEARNED_EPOCHS = 3


def learned_leg(args):
    """The learned-proposal configuration: plain rho vs the affine-coupling flow, each evaluated on
    args.learned_samples samples (1e7).  The flow is trained on 2e6 of rho's own weighted samples
    plus one round on 1e6 of its own; its training cost (drawing those samples and the two training
    rounds) is reported and added to its wall time to 1e-3."""
    import torch
    from pibronic_gb300 import constants, pimc, stats, synthetic
    from pibronic_gb300.file_structure import FileStructure
    from pibronic_gb300.flow import FlowProposal
    from pibronic_gb300.pimc import evaluate_device
    A, N, P, T = 6, 20, 128, 200.0
    X, C = args.learned_samples, 1_000_000
    out = {"workload": f"A={A} N={N} P={P} T={T:.0f}K off-diagonal couplings N(0,0.1) eV, dbeta=1e-4 beta, "
                       f"{X} samples per estimate; flow: 8 coupling layers, hidden 128, 3 ring slots per mode, "
                       f"trained on 2e6 rho samples + 1e6 of its own ({LEARNED_EPOCHS} epochs each, batch 16384)",
           "models": []}
    for seed in args.learned_seeds:
        root = tempfile.mkdtemp(prefix="pbr_learned_")
        FS = FileStructure(root, 0, 0)
        synthetic.write_model_pair(FS, A, N, seed, sd_offdiag=0.1)
        data = pimc.BoxDataPM(1e-4 * constants.beta(T))
        data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
        data.states, data.modes, data.beads, data.temperature = A, N, P, T
        data.samples = data.block_size = 1000
        data.blocks = 1
        data.preprocess()
        evaluate_device(data.plan, 10_000, seed=99, offset=0)
        fl = FlowProposal(data.prepared, data.plan, nsel=3, layers=8, hidden=128, seed=0)
        # ---- training cost: rho's samples with their q, two training rounds ----
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ys, rs = [], []
        for k in range(2):
            pl = evaluate_device(data.plan, C, seed=1001, offset=k * C, want_q=True)
            y, _ = fl.prepare(pl["q"])
            ys.append(y)
            rs.append(pl["s_g"] / pl["s_rho"])
            del pl
        torch.cuda.synchronize()
        t_draw = time.perf_counter() - t0
        if not out["models"]:
            _warm_training(torch, FlowProposal, data.prepared, data.plan, 3, ys[0], rs[0])
        _, t_train1 = _timed(torch, lambda: fl.train(torch.cat(ys), torch.cat(rs), epochs=LEARNED_EPOCHS,
                                                     batch=16384, lr=1e-3))
        del ys, rs
        first, t_own = _timed(torch, lambda: fl.sample_and_evaluate(C, seed=7, keep=True))
        _, t_train2 = _timed(torch, lambda: fl.train(first["y"], first["s_g"] / first["s_q"],
                                                     epochs=LEARNED_EPOCHS, batch=16384, lr=1e-3))
        del first
        train_s = t_draw + t_train1 + t_own + t_train2
        # ---- the two estimates, X samples each ----
        fl.sample_and_evaluate(10_000, seed=5)
        plain, tp = _chunked(torch, lambda n, off: evaluate_device(data.plan, n, seed=1, offset=off), X, C)
        ep = stats.device_estimates(plain["s_rho"], plain["s_g"], plain["s_gp"], plain["s_gm"], T, data.delta_beta)
        del plain
        res, tf = _chunked(torch, lambda n, off: fl.sample_and_evaluate(n, seed=8, offset=off), X, C)
        ef = stats.device_estimates(res["s_q"], res["s_g"], res["s_gp"], res["s_gm"], T, data.delta_beta)
        del res
        sp, sl = rate_summary(ep, tp, X), rate_summary(ef, tf, X, train_s)
        ratio = {k: (sp["time_to_1e-3_s"][k] / sl["time_to_1e-3_s"][k]
                     if sp["time_to_1e-3_s"][k] and sl["time_to_1e-3_s"][k] else None) for k in ("Z", "E", "Cv")}
        agree = {k: abs(sl[k] - sp[k]) / math.hypot(sl[k + " error"], sp[k + " error"]) for k in ("Z", "E", "Cv")}
        out["models"].append({"model_seed": seed, "plain": sp, "learned": sl,
                              "train_s": train_s,
                              "train_parts_s": {"rho_samples_2e6": t_draw, "round1": t_train1,
                                                "own_samples_1e6": t_own, "round2": t_train2},
                              "ess_per_s_ratio": sl["ess_per_s"] / sp["ess_per_s"],
                              "proposal_overhead": sp["samples_per_s"] / sl["samples_per_s"] - 1.0,
                              "wall_to_1e-3_ratio_incl_training": ratio,
                              "agreement_sigma": agree})
    out["median_ess_per_s_ratio"] = statistics.median(m["ess_per_s_ratio"] for m in out["models"])
    return out


def cublas_peak(torch, dtype):
    """cuBLAS dense GEMM throughput measured in this run (8192^3, best of 5, CUDA events), FP32
    inputs with TF32 math or 16-bit inputs: the denominators for the tcgen05 kernels (the pool's
    MEASURED_PEAKS.json holds a bf16 figure measured outside this run)."""
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    n = 8192
    a = torch.randn(n, n, device="cuda").to(dtype)
    b = torch.randn(n, n, device="cuda").to(dtype)
    c = a @ b
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    torch.backends.cuda.matmul.allow_tf32 = old
    del a, b, c
    return 2.0 * n ** 3 / best / 1e12


def large_leg(args):
    """The large dense configuration: A=12, N=64, P=256, dense Q ~ N(0, 0.001) eV, T=300 K.  V is
    built by the tcgen05 TF32 GEMM (pbr_sample_eval_tc), exp(-tau V) by the wide form; the
    learned proposal (flow over 2 ring slots per mode) is trained on the method's own samples."""
    import ctypes
    import torch
    from pibronic_gb300 import _native, stats
    from pibronic_gb300.flow import FlowProposal
    from pibronic_gb300.pimc import evaluate_device
    A, N, P, T = 12, 64, 256, 300.0
    X, Ct = args.large_samples, 400_000
    data = large_model_data(T)
    plan = data.plan
    assert plan.use_tc
    evaluate_device(plan, 1000, seed=9, offset=0)
    # the flow's training samples (rho's own, with their q: 26 GB at 4e5 samples)
    train_pl, t_draw = _timed(torch, lambda: evaluate_device(plan, Ct, seed=1001, offset=0, want_q=True))
    plain, tp = _chunked(torch, lambda n, off: evaluate_device(plan, n, seed=1, offset=off), X, 2_000_000)
    ep = stats.device_estimates(plain["s_rho"], plain["s_g"], plain["s_gp"], plain["s_gm"], T, data.delta_beta)
    del plain
    # the tcgen05 GEMM alone on one L2-sized chunk of this run's q
    lib = _native.load()
    n2p, a2p = ctypes.c_int32(), ctypes.c_int32()
    _native.check(lib.pbr_tc_potential_dims(N, A, ctypes.byref(n2p), ctypes.byref(a2p)), "dims")
    n2p, a2p = n2p.value, a2p.value
    Xc = min(X, max(1, (64 << 20) // (4 * P * (N + a2p))))
    bp = torch.empty(int(lib.pbr_tc_potential_packed_floats(N, A)), dtype=torch.float32, device="cuda")
    vq = torch.empty((Xc * P, a2p), dtype=torch.float32, device="cuda")
    t_ = plan.tensors
    sh = _native.stream_handle()
    _native.check(lib.pbr_tc_pack_potential(t_["vib_qq"].data_ptr(), t_["vib_l"].data_ptr(), t_["vib_e"].data_ptr(),
                                            32, N, A, _native.ptr(bp), sh), "pack")
    qc = train_pl["q"][:Xc]
    ts = []
    for i in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _native.check(lib.pbr_tc_potential(_native.ptr(qc), Xc, N, P, A, _native.ptr(bp), _native.ptr(vq), None, sh),
                      "tc potential")
        e1.record()
        e1.synchronize()
        if i:
            ts.append(e0.elapsed_time(e1) * 1e-3)
    t_tc = min(ts)
    mp = a2p                                                             # pair columns incl. padding
    issued = 6.0 * Xc * P * mp * n2p / t_tc / 1e12
    useful = 2.0 * Xc * P * (A * (A + 1) // 2) * (N * (N + 1) // 2 + N + 1) / t_tc / 1e12
    peak16 = cublas_peak(torch, torch.float16)
    probe = torch.empty(2, dtype=torch.float64, device="cuda")

    def mma_rate(fmt, n_cols):
        # A in TMEM, as the potential GEMM issues them
        rate, cyc = ctypes.c_double(), ctypes.c_double()
        _native.check(lib.pbr_tc_mma_rate(fmt, 128, n_cols, 1, 1, 4096, _native.ptr(probe), ctypes.byref(rate),
                                          ctypes.byref(cyc), sh), "mma rate")
        return rate.value, cyc.value
    r256, c256 = mma_rate(1, 256)
    rN, cN = mma_rate(1, mp)

    out = {"workload": f"A={A} N={N} P={P} T={T:.0f}K dense Q N(0,0.001) eV, dbeta=1e-4 beta, {X} samples per "
                       f"estimate; flow over 2 ring slots per mode trained on {Ct} rho samples",
           "plain": rate_summary(ep, tp, X),
           "tc_gemm": {"chunk_samples": Xc, "ms": 1e3 * t_tc, "issued_tflops": issued, "useful_tflops": useful,
                       "fp16_cublas_tflops_measured": peak16, "frac_of_measured_fp16": issued / peak16,
                       "f16_mma_128x256x16_tflops_measured": r256, "cycles_per_mma_n256": c256,
                       f"f16_mma_128x{mp}x16_tflops_measured": rN, f"cycles_per_mma_n{mp}": cN,
                       "frac_of_mma_rate_at_its_n": issued / rN,
                       "note": "issued = 3 FP16 passes (hi/lo split) x padded K x padded pair columns; "
                               "a kind::f16 MMA costs the same cycles for every N up to 128, so at "
                               f"N = {mp} the tensor pipe's ceiling is the rate at that N"}}
    if not args.no_learned:
        fl = FlowProposal(data.prepared, plan, nsel=2, layers=8, hidden=128, seed=0)
        y, _ = fl.prepare(train_pl["q"])
        r = train_pl["s_g"] / train_pl["s_rho"]
        del train_pl
        _warm_training(torch, FlowProposal, data.prepared, plan, 2, y, r)
        _, t_train = _timed(torch, lambda: fl.train(y, r, epochs=6, batch=16384, lr=1e-3))
        del y
        fl.sample_and_evaluate(1000, seed=5)
        res, tf = _chunked(torch, lambda n, off: fl.sample_and_evaluate(n, seed=8, offset=off), X, Ct)
        ef = stats.device_estimates(res["s_q"], res["s_g"], res["s_gp"], res["s_gm"], T, data.delta_beta)
        del res
        train_s = t_draw + t_train
        sl = rate_summary(ef, tf, X, train_s)
        sp = out["plain"]
        out["learned"] = sl
        out["train_s"] = train_s
        out["ess_per_s_ratio"] = sl["ess_per_s"] / sp["ess_per_s"]
        out["wall_to_1e-3_ratio_incl_training"] = {
            k: (sp["time_to_1e-3_s"][k] / sl["time_to_1e-3_s"][k]
                if sp["time_to_1e-3_s"][k] and sl["time_to_1e-3_s"][k] else None) for k in ("Z", "E", "Cv")}
        out["agreement_sigma"] = {k: abs(sl[k] - sp[k]) / math.hypot(sl[k + " error"], sp[k + " error"])
                                  for k in ("Z", "E", "Cv")}
    return out


def large_model_data(T=300.0):
    """The large dense configuration's model pair and BoxDataPM (A=12, N=64, P=256, dense Q)."""
    from pibronic_gb300 import constants, pimc, synthetic, vibronic_io
    from pibronic_gb300.file_structure import FileStructure
    A, N, P = 12, 64, 256
    FS = FileStructure(tempfile.mkdtemp(prefix="pbr_large_"), 0, 0)
    model = synthetic.make_coupled_model(A, N, 5, sd_quadratic=0.001)
    vibronic_io.save_model_to_JSON(FS.path_vib_model, model)
    vibronic_io.create_basic_diagonal_model(FS)
    data = pimc.BoxDataPM(1e-4 * constants.beta(T))
    data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
    data.states, data.modes, data.beads, data.temperature = A, N, P, T
    data.samples = data.block_size = 1000
    data.blocks = 1
    data.preprocess()
    return data


def precision_leg(args):
    """The precision configuration: the main workload's model (A=4, N=12, P=64) at T = 100, 300 and
    500 K, args.precision_samples device-drawn samples each, evaluated by the FP32 production
    kernel and by the FP64 build of the same kernel on identical q (pibronic_gb300.precision):
    per-sample relative errors of rho, g, g(beta +- dbeta) and the FP32 - FP64 differences of Z, E
    and Cv in units of their statistical errors."""
    from pibronic_gb300 import constants, synthetic
    from pibronic_gb300.plan import PreparedModels
    from pibronic_gb300.precision import compare
    m = synthetic.make_coupled_model(A_, N_, MODEL_SEED)
    out = {"workload": f"A={A_} N={N_} P={P_}, {args.precision_samples} samples per temperature, "
                       f"FP32 kernel vs FP64 build on identical q", "temperatures": []}
    for T in (100.0, 300.0, 500.0):
        b = constants.beta(T)
        prep = PreparedModels(m, synthetic.diagonal_of(m), P_, beta=b, delta_beta=1e-4 * b)
        res = compare(prep, args.precision_samples, seed=77, temperature=T)
        out["temperatures"].append({"T": T, "per_sample": res["per_sample"], "estimates": res["estimates"],
                                    "ess_per_sample": res["ess_per_sample"]})
    out["max_per_sample_rel"] = max(v["max_rel"] for t in out["temperatures"]
                                    for k, v in t["per_sample"].items() if k.startswith("s_"))
    out["max_abs_delta_over_sigma"] = max(abs(v["delta_over_sigma"]) for t in out["temperatures"]
                                          for v in t["estimates"].values())
    return out


def profile_large(args):
    """Profiling helper (no timing, no JSON line): two evaluations of args.profile_large samples of
    the large dense configuration through the tensor-core form, for an ncu capture."""
    import torch
    from pibronic_gb300.pimc import evaluate_device
    data = large_model_data()
    for i in range(2):
        out = evaluate_device(data.plan, args.profile_large, seed=1 + i, offset=0)
    torch.cuda.synchronize()
    assert int(out["status"].item()) == 0
    print("profile-large done", args.profile_large)
    return 0


def profile_batched(args):
    """Profiling helper (no timing, no JSON line): the batched configuration's 256 models, two
    passes of args.profile_batched samples each, with the kernel form and tile budget the autotuner
    chose on this part (register chunks up to 4 surfaces, whole-memory row-team tiles from 5), for
    an ncu capture."""
    import torch
    from pibronic_gb300 import synthetic
    from pibronic_gb300.batch import ModelBatch
    count, X = args.batch_models, args.profile_batched
    preps = synthetic.batch_models(count=count, seed=3)
    mb = ModelBatch(preps, [X] * count, list(range(1, count + 1)),
                    smem_budget={2: -1, 3: -1, 4: -1, 5: 0, 6: 0, 7: 0, 8: 0})
    for _ in range(2):
        mb.run()
    torch.cuda.synchronize()
    assert int(mb.status.item()) == 0
    print("profile-batched done", X, "groups", mb.groups)
    return 0


def profile_learned(args):
    """Profiling helper (no timing, no JSON line): two plain-rho evaluations of args.profile_learned
    samples of the learned-proposal configuration's model (A=6, N=20, P=128, T=200 K, strong
    couplings; the row-team form), for an ncu capture."""
    import torch
    from pibronic_gb300 import constants, pimc, synthetic
    from pibronic_gb300.file_structure import FileStructure
    from pibronic_gb300.pimc import evaluate_device
    A, N, P, T = 6, 20, 128, 200.0
    FS = FileStructure(tempfile.mkdtemp(prefix="pbr_plearn_"), 0, 0)
    synthetic.write_model_pair(FS, A, N, args.learned_seeds[0], sd_offdiag=0.1)
    data = pimc.BoxDataPM(1e-4 * constants.beta(T))
    data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
    data.states, data.modes, data.beads, data.temperature = A, N, P, T
    data.samples = data.block_size = 1000
    data.blocks = 1
    data.preprocess()
    for i in range(2):
        out = evaluate_device(data.plan, args.profile_learned, seed=1 + i, offset=0)
    torch.cuda.synchronize()
    assert int(out["status"].item()) == 0
    print("profile-learned done", args.profile_learned)
    return 0


def mma_rates(args):
    """Profiling helper (no JSON line): the library's tcgen05 rate probe over operand type, M, N,
    independent accumulators and the A operand's home, one row per shape (cycles per MMA of the
    issuing thread and whole-GPU TF/s)."""
    import ctypes
    import torch
    from pibronic_gb300 import _native
    from pibronic_gb300.build import build
    lib = _native.load(build())
    probe = torch.empty(2, dtype=torch.float64, device="cuda")
    sh = _native.stream_handle()
    print("kind  M    N  accumulators  A_in_tmem  cycles_per_mma  TF/s")
    for fmt, kind in ((2, "tf32"), (1, "f16")):
        for M in (128, 64):
            for N in (16, 32, 64, 80, 96, 128, 160, 256):
                for nacc in (1, 2, 4):
                    for at in ((0, 1) if M == 128 else (0,)):
                        if nacc * N + (16 if at else 0) > 512:
                            continue
                        r, c = ctypes.c_double(), ctypes.c_double()
                        _native.check(lib.pbr_tc_mma_rate(fmt, M, N, nacc, at, 4096, _native.ptr(probe),
                                                          ctypes.byref(r), ctypes.byref(c), sh), "mma rate")
                        print(f"{kind:5s} {M:3d} {N:4d} {nacc:13d} {at:10d} {c.value:15.1f} {r.value:7.1f}")
    return 0


def profile_flow(args):
    """Profiling helper (no JSON line): the learned configuration's flow (A=6, N=20, P=128,
    hidden 128, 8 layers): 20 training steps at batch 16384 on rho's weighted samples, then one
    args.profile_flow-sample draw through the tensor-core sampling layers, for an ncu capture."""
    import torch
    from pibronic_gb300 import constants, pimc, synthetic
    from pibronic_gb300.file_structure import FileStructure
    from pibronic_gb300.flow import FlowProposal
    from pibronic_gb300.pimc import evaluate_device
    A, N, P, T = 6, 20, 128, 200.0
    FS = FileStructure(tempfile.mkdtemp(prefix="pbr_pflow_"), 0, 0)
    synthetic.write_model_pair(FS, A, N, args.learned_seeds[0], sd_offdiag=0.1)
    data = pimc.BoxDataPM(1e-4 * constants.beta(T))
    data.path_vib_model, data.path_rho_model = FS.path_vib_model, FS.path_rho_model
    data.states, data.modes, data.beads, data.temperature = A, N, P, T
    data.samples = data.block_size = 1000
    data.blocks = 1
    data.preprocess()
    pl = evaluate_device(data.plan, 20 * 16384, seed=1, offset=0, want_q=True)
    fl = FlowProposal(data.prepared, data.plan, nsel=3, layers=8, hidden=128, seed=0)
    y, _ = fl.prepare(pl["q"])
    fl.train(y, pl["s_g"] / pl["s_rho"], epochs=1, batch=16384, lr=1e-3)
    out = fl.sample_and_evaluate(args.profile_flow, seed=5)
    torch.cuda.synchronize()
    assert int(out["status"].item()) == 0
    print("profile-flow done", args.profile_flow)
    return 0


def batched_leg(args):
    """256 seeded models, A ~ U{2..8}, N ~ U{3..20}, P ~ U{8..256}, T ~ U[100, 500] K, 1e5 samples
    each, one persistent launch per row-team group or register-chunk launches per model, the form
    and tile budget autotuned per surface count, captured in a CUDA graph."""
    import torch
    from pibronic_gb300 import synthetic
    from pibronic_gb300.batch import ModelBatch, autotune
    count, X = args.batch_models, args.batch_samples
    preps = synthetic.batch_models(count=count, seed=3)
    seeds = list(range(1, count + 1))
    budgets, times = autotune(preps, seeds, X_probe=16384)
    mb = ModelBatch(preps, [X] * count, seeds, smem_budget=budgets)
    mb.capture()
    mb.replay()
    ts = []
    for _ in range(3):
        _, t = _timed(torch, mb.replay)
        ts.append(t)
    t = min(ts)
    ests = mb.estimates()
    W = sum(flops_per_sample(p.A, p.N, p.P) for p in preps) * X
    return {"workload": f"{count} models, A~U{{2..8}}, N~U{{3..20}}, P~U{{8..256}}, T~U[100,500]K, {X} samples each",
            "samples_per_s": count * X / t, "ms_per_pass": 1e3 * t, "launch_groups": mb.groups,
            "chosen_budget_bytes": {str(a): ("register chunks" if b < 0 else b) for a, b in budgets.items()},
            "autotune_ms": {str(a): {("register chunks" if b < 0 else str(b)): (None if v is None else 1e3 * v)
                                     for b, v in tv.items()} for a, tv in times.items()},
            "autotune_feasible_per_group": {str(a): sum(v is not None for v in tv.values()) for a, tv in times.items()},
            "algorithmic_tflops": W / t / 1e12,
            "median_ess_per_sample": statistics.median(e["ESS"] / X for e in ests),
            "finite": bool(int(mb.status.item()) == 0)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--samples", type=int, default=1_000_000, help="samples per step per GPU")
    ap.add_argument("--cpu-samples", type=int, default=400, help="samples per host process (CPU legs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--variant", type=int, default=0, help="fused-kernel form: 0 auto, 1 chunks, 2 teams")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--precision-samples", type=int, default=1_000_000)
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--learned-samples", type=int, default=10_000_000)
    ap.add_argument("--learned-seeds", type=int, nargs="+", default=[404, 44, 4])
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-models", type=int, default=256)
    ap.add_argument("--batch-samples", type=int, default=100_000)
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--large-samples", type=int, default=10_000_000)
    ap.add_argument("--profile-large", type=int, default=0,
                    help="profiling helper: evaluate this many samples of the large configuration twice, exit")
    ap.add_argument("--profile-learned", type=int, default=0,
                    help="profiling helper: evaluate this many plain-rho samples of the learned "
                         "configuration's model twice, exit")
    ap.add_argument("--profile-flow", type=int, default=0,
                    help="profiling helper: 20 flow training steps, then this many tensor-core flow samples, exit")
    ap.add_argument("--profile-batched", type=int, default=0,
                    help="profiling helper: two passes of the batched models with this many samples each, exit")
    ap.add_argument("--mma-rates", action="store_true",
                    help="profiling helper: sweep the tcgen05 rate probe, print a table, exit")
    args = ap.parse_args()
    if args.mma_rates:
        return mma_rates(args)
    if args.profile_flow > 0:
        return profile_flow(args)
    if args.profile_large > 0:
        return profile_large(args)
    if args.profile_learned > 0:
        return profile_learned(args)
    if args.profile_batched > 0:
        return profile_batched(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python3
"""Benchmark of the GB300-native electrostatic placement loop.

A "step" is one Placement::step (src/placement.rs:180-228) of the plain FP32
path on the 1,000,000-cell synthetic workload (1,050,000 nets, 16 macros,
4,000 IO pins, 1024x1024 bins, target density 1.0), replayed from the
context's captured CUDA graph.  `value` is Nesterov iterations/s with the
design resident in HBM; `e2e` is the same metric through the drop-in
host-coordinate call erp_step_host (pinned host x/y copied in and out every
step).  `--impl reference` times the CPU restatement of the reference loop
(the oracle, reference FP32 mode) on the machine's host cores; that arm builds
its input with the generator compiled on its own (oracle/_build/
liberp_synth.so) and never loads the product library.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "iters/s @1M cells, jobs/h, p99 latency: mixed/batched vs plain FP32 @HPWL±0.5%"
UNIT = "iters/s"
L2_BYTES = 129 * 2 ** 20

# Algorithmic bytes per launch of each stage (FP32 = 4 B, index = 4 B,
# int64 = 8 B; each array counted once): N movable cells, P pins, E nets,
# B = m*n bins.  wirelength (k_wa): per pin the cell index (4), the pin offset
# (8), the gathered (x, y) (8) and the pin gradient written (8); per net its
# HPWL (4) (the net_ptr reads of the ~1 % of nets above 8 pins are left out).
# wl_gather: per pin its slot index (4) and gradient (8); per cell the range
# (4) and the gradient pair written (8).
ALG_BYTES = {
    "wirelength": lambda N, P, E, B: 28 * P + 4 * E,
    "wl_gather": lambda N, P, E, B: 12 * P + 12 * N,
    "density": lambda N, P, E, B: 28 * N + 8 * B,
    "spectral": lambda N, P, E, B: 44 * B,   # R1 12 + 4, C1 4 + 8, R2 8 + 8 (read + write per bin)
    "force": lambda N, P, E, B: 36 * N + 8 * B,
    "nesterov": lambda N, P, E, B: 76 * N,
    "scheduler": lambda N, P, E, B: 0,
}
# DRAM bytes per launch from ncu (dram__bytes_read.sum + dram__bytes_write.sum)
# of one --set full capture of the kernel on this workload (cold L2, the
# profiler's default cache control), taken with the command
#   ncu --set full --clock-control none -k regex:k_wa -s 3 -c 1 -o k_wa \
#       python bench.py --steps 20 --warmup 3 --no-cpu --batch-count 0 --quick
# A bench run cannot count DRAM bytes itself, so the line labels this figure
# as coming from that capture, not from the run.
NCU_TRAFFIC = {("large", "wirelength"): 69.074176e6 + 15.063040e6}

# The workloads: the synthetic generator's arguments and the run's
# configuration.  The same data as reda_erplacer_gb300.design.WORKLOADS, kept
# here so that the reference arm builds its input without importing the
# package (tests/test_bench_fp64.py checks that the two agree).
WORKLOADS = {
    "small": (dict(num_cells=20000, num_nets=21000, num_io=400, num_macros=0, utilization=0.70, seed=1),
              dict(bins=(256, 256), target_density=1.0, iterations=450)),
    "large": (dict(num_cells=1000000, num_nets=1050000, num_io=4000, num_macros=16, macro_area_frac=0.015,
                   utilization=0.65, seed=2),
              dict(bins=(1024, 1024), target_density=1.0, iterations=1000)),
}
DESCS = {
    "small": "plain FP32, 20,000 movable cells / 21,000 nets / 400 IO, 256x256 bins",
    "large": "plain FP32, 1,000,000 movable cells / 1,050,000 nets / 16 macros / 4,000 IO, 1024x1024 bins",
}


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi SM clock / throttle-reason samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                  "sw_power_cap"), parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def allreduce_max(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_sum(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_items(items, world):
    """Concatenate every rank's list (rank order); the only cross-rank step of
    the sharded batch and serving sections besides the max of their times."""
    if world == 1:
        return list(items)
    import torch.distributed as dist
    out = [None] * world
    dist.all_gather_object(out, list(items))
    return [x for part in out for x in part]


def make_workload(name, generator):
    """The named workload's design from `generator` (the package's synth, or the
    oracle's copy of the same generator), its run configuration and label."""
    args, cfg = WORKLOADS[name]
    return generator(**args), dict(cfg), DESCS[name]


def workload_config(d, cfg, desc):
    """The line's `config`: the workload only, identical in both arms."""
    m, n = cfg["bins"]
    return {"workload": desc, "cells": int(d.num_movable), "nets": int(d.num_nets), "pins": int(d.num_pins),
            "bins": [m, n], "target_density": cfg["target_density"], "iterations": cfg["iterations"],
            "start": "die centre + Gaussian jitter (sigma 0.1% of die width)",
            "parallelism": "replicas (one design per GPU)",
            "l2": ("inputs larger than L2 (per-step working set > 129 MiB), no flush" if m * n >= 1 << 20
                   else "working set smaller than L2, no flush (a step reuses the last step's data)")}


def cpu_sample(d, cfg, iters, literal, warmup=1, trace=False):
    """Time `iters` oracle steps (all host threads) after `warmup` untimed steps.
    literal: the reference's own FP32 rules (sequential density below
    iteration 200, then per-bin atomic adds; FP32 sums), else the fixed-point /
    FP64 form.  trace: also return every step's (hpwl, overflow), warm-up
    steps included, in iteration order."""
    from oracle import erp_oracle as O
    m, n = cfg["bins"]
    o = O.Oracle(d, m, n, target_density=cfg["target_density"], start_mode=O.START_DB,
                 density_mode=O.DENSITY_REFERENCE if literal else O.DENSITY_FIXED,
                 reduce_fp64=0 if literal else 1, num_threads=0)
    hist = []
    for _ in range(max(1, warmup)):
        s = o.step()
        hist.append((s["hpwl"], s["overflow"]))
    t0 = time.perf_counter()
    for _ in range(iters):
        s = o.step()
        if trace:
            hist.append((s["hpwl"], s["overflow"]))
    dt = time.perf_counter() - t0
    o.close()
    return (iters / dt, dt, hist) if trace else (iters / dt, dt)


def parity_summary(gpu, ref, tto_iteration):
    """HPWL / overflow of the GPU run against the reference CPU loop, both from
    the same start over the same iteration count: at the iteration where the
    GPU run first reaches overflow 0.10, at each run's overflow minimum (the
    converged state; past it the loop diverges and two summation orders of the
    reference itself part), and at the last iteration."""
    def at(k):
        (hg, og), (hr, orf) = gpu[k], ref[k]
        return {"iteration": k + 1, "hpwl_gpu": hg, "hpwl_ref": hr, "hpwl_rel": (hg - hr) / hr,
                "overflow_gpu": og, "overflow_ref": orf, "overflow_abs": og - orf}
    kg = min(range(len(gpu)), key=lambda k: gpu[k][1])
    kr = min(range(len(ref)), key=lambda k: ref[k][1])
    out = {"iterations": len(gpu), "last": at(len(gpu) - 1),
           "overflow_min": {"iteration_gpu": kg + 1, "iteration_ref": kr + 1,
                            "overflow_gpu": gpu[kg][1], "overflow_ref": ref[kr][1],
                            "overflow_abs": gpu[kg][1] - ref[kr][1],
                            "hpwl_gpu": gpu[kg][0], "hpwl_ref": ref[kr][0],
                            "hpwl_rel": (gpu[kg][0] - ref[kr][0]) / ref[kr][0]}}
    if tto_iteration:
        out["at_overflow_0.10"] = at(tto_iteration - 1)
    return out


def batch_section(args, device, world=1, rank=0):
    """Batched workload: 64 instances (cells log-uniform 2k-200k, nets 1.05x,
    macros 0-16, bins = pow2 nearest sqrt(cells)/2 in 64..1024), each to 600
    iterations or overflow <= 0.10.  Jobs/hour of the batched graph (all
    instances in one CUDA graph) against running the same jobs one at a time
    through erp_run; both include context creation.  With several ranks the
    instances are sharded over the GPUs (host-side dispatch, no collective) and
    each time is the maximum over the ranks."""
    import torch
    import reda_erplacer_gb300 as R
    from reda_erplacer_gb300.dispatch import job_cost, rank_jobs
    full = R.workload_batch(count=args.batch_count)
    mine = rank_jobs([job_cost(d.num_movable, args.batch_iters) for d, _ in full], world, rank)
    mix = [full[i] for i in mine]
    designs = [d for d, _ in mix]
    bins = [b for _, b in mix]
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bt = R.Batch(designs, bins, 1.0, start_mode=1, device=device)
    t_bcreate = time.perf_counter() - t0
    tune_chosen, tune_ms = bt.tuning()
    spec_chosen, spec_ms = bt.spectral_tuning()
    its, lasts = bt.run(args.batch_iters, stop_overflow=0.10)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    packed_n = bt.packed_instances()
    bt.close()
    # the same mix with a graph branch per instance instead of the packed launches,
    # and a mix of many tiny instances (2,000-4,000 cells, 64^2 bins), where the
    # launches rather than the work set the pace, in both forms
    forms = {}
    tiny = R.workload_batch(count=64 if world == 1 else 64 // world, seed=4100, min_cells=2000, max_cells=4000)
    for name, jobs_ in (("mix", mix), ("tiny_mix", tiny)):
        for form in ("packed", "branches"):
            if name == "mix" and form == "packed":
                forms["mix_packed_s"] = t_batch
                continue
            os.environ["ERP_BATCH_FORM"] = form
            try:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                b2 = R.Batch([d for d, _ in jobs_], [b for _, b in jobs_], 1.0, start_mode=1, device=device)
                b2.run(args.batch_iters, stop_overflow=0.10)
                torch.cuda.synchronize()
                forms[f"{name}_{form}_s"] = time.perf_counter() - t0
                b2.close()
            finally:
                del os.environ["ERP_BATCH_FORM"]
    forms = {k: allreduce_max(v, world) for k, v in forms.items()}
    n_tiny = len(tiny) * world
    del tiny
    seq_lat = []
    t0 = time.perf_counter()
    seq_its = []
    t_screate = 0.0
    for d, b in mix:
        t1 = time.perf_counter()
        pl = R.Placement(d, b, 1.0, start_mode=1, device=device)
        t_screate += time.perf_counter() - t1
        it, last = pl.run(args.batch_iters, stop_overflow=0.10)
        pl.close()
        seq_its.append(it)
        seq_lat.append(time.perf_counter() - t1)
    t_seq = time.perf_counter() - t0
    K = len(mix)
    # mixed form: the spectral solve in BF16 hi/lo x3 on the tensor cores for every
    # instance whose bin grid allows it (multiples of 128), FP32 FFT for the 64^2 ones
    precs = [R.lib.PREC_BF16X3_GEMM if b[0] >= 128 else R.lib.PREC_FP32 for b in bins]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bm = R.Batch(designs, bins, 1.0, start_mode=1, device=device, precision=precs)
    its_m, lasts_m = bm.run(args.batch_iters, stop_overflow=0.10)
    torch.cuda.synchronize()
    t_mixed = time.perf_counter() - t0
    bm.close()
    # across ranks: times are the slowest rank's, counts and lists are gathered
    t_batch, t_seq, t_mixed = (allreduce_max(t, world) for t in (t_batch, t_seq, t_mixed))
    t_bcreate, t_screate = allreduce_max(t_bcreate, world), allreduce_max(t_screate, world)
    rows = sorted(gather_items([(i, int(a), int(b), int(c), la["overflow"], la["hpwl"], lm["overflow"], lm["hpwl"], q)
                                for i, a, b, c, la, lm, q in zip(mine, its, seq_its, its_m, lasts, lasts_m, seq_lat)],
                               world))
    precs_all = gather_items([int(p != R.lib.PREC_FP32) for p in precs], world)
    K = len(full)
    its, seq_its, its_m = [r[1] for r in rows], [r[2] for r in rows], [r[3] for r in rows]
    lasts = [{"overflow": r[4], "hpwl": r[5]} for r in rows]
    lasts_m = [{"overflow": r[6], "hpwl": r[7]} for r in rows]
    seq_lat = [r[8] for r in rows]
    designs = [d for d, _ in full]
    bins = [b for _, b in full]
    return {
        "instances": K, "ranks": world, "cells": [int(d.num_movable) for d in designs],
        "bins": [int(b[0]) for b in bins], "max_iterations": args.batch_iters, "stop_overflow": 0.10,
        "iterations_total": int(sum(its)), "retired_at_overflow": int(sum(1 for l in lasts if l["overflow"] <= 0.10)),
        "batched_s": t_batch, "sequential_s": t_seq,
        "batched_create_s": t_bcreate, "sequential_create_s": t_screate,
        "jobs_per_hour_batched": K / t_batch * 3600.0, "jobs_per_hour_sequential": K / t_seq * 3600.0,
        "speedup": t_seq / t_batch, "same_iterations": its == seq_its,
        "sequential_latency_p50_s": float(statistics.median(seq_lat)),
        "spectral": "FP32 FFT (batched and sequential)",
        "scatter_autotune": {"cells_per_block": tune_chosen,
                             "candidates_ms": {str(c): round(t, 4) for c, t in tune_ms},
                             "note": "0 = the rule of a context run alone; timed at creation, all instances' "
                                     "scatters together; included in batched_s"},
        "packed_instances": packed_n,
        "forms": {
            "mix_packed_jobs_per_hour": K / forms["mix_packed_s"] * 3600.0,
            "mix_branches_jobs_per_hour": K / forms["mix_branches_s"] * 3600.0,
            "tiny_mix_instances": n_tiny,
            "tiny_mix_packed_jobs_per_hour": n_tiny / forms["tiny_mix_packed_s"] * 3600.0,
            "tiny_mix_branches_jobs_per_hour": n_tiny / forms["tiny_mix_branches_s"] * 3600.0,
            "note": "packed: the FP32 instances with bins <= 256 advance in one launch per stage over a table of "
                    "all of them; branches: a graph branch of ten kernels per instance. Same bits either way; "
                    "times include context creation"},
        "spectral_autotune": {"seqs_per_block": spec_chosen,
                              "candidates_ms": {str(c): round(t, 4) for c, t in spec_ms},
                              "note": "rows / columns per block of the FP32 passes at sides 64-256 (0 = the "
                                      "fixed four); timed at creation, all FP32 instances' passes together; "
                                      "included in batched_s"},
        "mixed_batched": {
            "spectral": "BF16 hi/lo x3 tensor-core contractions (bins >= 128), FP32 FFT (64^2 bins)",
            "instances_bf16x3": int(sum(precs_all)),
            "batched_s": t_mixed, "jobs_per_hour": K / t_mixed * 3600.0,
            "speedup_vs_fp32_one_at_a_time": t_seq / t_mixed,
            "iterations_total": int(sum(its_m)),
            "retired_at_overflow": int(sum(1 for l in lasts_m if l["overflow"] <= 0.10)),
            "hpwl_rel_diff_median": float(statistics.median(
                [(a["hpwl"] - b["hpwl"]) / b["hpwl"] for a, b in zip(lasts_m, lasts)])),
        },
    }


def poisson_fp64(rho, bw, bh):
    """FP64 closed form of the Poisson solve (the per-axis transforms of the
    reference pipelines): A = (2/m)(2/n) DCT-II_m DCT-II_n(rho);
    field_x = IDXST_m IDCT_n(A wu / 2k^2), field_y = IDCT_m IDXST_n(A wv / 2k^2),
    psi = IDCT_m IDCT_n(A / k^2), k^2 = wu^2 + wv^2, [0,0] -> 0."""
    import numpy as np
    from scipy.fft import dct
    m, n = rho.shape
    a = dct(dct(rho.astype(np.float64), type=2, axis=0), type=2, axis=1) / (m * n)
    wu = 2.0 * np.pi * np.arange(m) / m
    wv = 2.0 * np.pi * np.arange(n) / n * (bw / bh)
    k2 = wu[:, None] ** 2 + wv[None, :] ** 2
    k2[0, 0] = 1.0
    inv = 1.0 / k2
    inv[0, 0] = 0.0

    def idct(x, ax):   # y_i = X_0 + 2 sum_{u>=1} X_u cos(pi u (2i+1) / 2N)
        return dct(x, type=3, axis=ax)

    def idxst(x, ax):  # y_i = (-1)^i IDCT(X')_i, X'_0 = 0, X'_u = X_(N-u)
        xp = np.zeros_like(x)
        if ax == 0:
            xp[1:] = x[1:][::-1]
        else:
            xp[:, 1:] = x[:, 1:][:, ::-1]
        y = idct(xp, ax)
        sgn = np.where(np.arange(x.shape[ax]) % 2 == 0, 1.0, -1.0)
        return y * (sgn[:, None] if ax == 0 else sgn[None, :])

    fx = idxst(idct(a * (0.5 * wu[:, None] * inv), 1), 0)
    fy = idct(idxst(a * (0.5 * wv[None, :] * inv), 1), 0)
    psi = idct(idct(a * inv, 1), 0)
    return fx, fy, psi


def measured_peak_tflops():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def spectral_section(args, device):
    """Isolated Poisson solve on the seeded density maps (0.7 background, 2,000
    Gaussian blobs, 10 macro blocks) at 512^2, 1024^2 and 2048^2 bins, in the
    three forms: FP32 FFT, TF32 DCT-GEMM and BF16 hi/lo DCT-GEMM (tcgen05).
    Time per solve (CUDA events, L2 flushed before each solve), the relative L2
    error of each output against the FP64 closed form, and the roofline: the
    FFT on 16 B per bin (rho in; field_x, field_y, psi out) against HBM, the
    contractions on 16 s^3 FLOP (x3 tensor products for BF16 hi/lo) against the
    measured bf16 tensor peak (TF32: half of it, the nominal ratio)."""
    import numpy as np
    import torch
    import reda_erplacer_gb300 as R
    peak, peak_kind = measured_peak_gbs()
    tpeak, tpeak_kind = measured_peak_tflops()
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device=f"cuda:{device}")
    forms = (("fp32_fft", R.lib.PREC_FP32), ("tf32_dct_gemm", R.lib.PREC_TF32_GEMM),
             ("bf16x3_dct_gemm", R.lib.PREC_BF16X3_GEMM))
    out = {}
    for side in (512, 1024, 2048):
        rho = R.workload_spectral(side, seed=3000 + side)
        ref = poisson_fp64(rho, 1.0, 1.0)
        r = torch.tensor(rho, device=f"cuda:{device}")
        row = {}
        for name, prec in forms:
            s = torch.cuda.Stream(device=device)
            sol = R.SpectralSolver(side, side, 1.0, 1.0, stream=s.cuda_stream, precision=prec)
            outs = [torch.empty_like(r) for _ in range(3)]
            ptrs = [t.data_ptr() for t in outs]
            with torch.cuda.stream(s):
                for _ in range(3):
                    sol.solve(r.data_ptr(), *ptrs)
                ts = []
                for _ in range(args.spectral_reps):
                    flush.fill_(1.0)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(s)
                    sol.solve(r.data_ptr(), *ptrs)
                    e1.record(s)
                    e1.synchronize()
                    ts.append(e0.elapsed_time(e1))
            torch.cuda.synchronize()
            got = [t.cpu().numpy().astype(np.float64) for t in outs]
            err = [float(np.linalg.norm(g - w) / np.linalg.norm(w)) for g, w in zip(got, ref)]
            us = 1000.0 * float(np.median(ts))
            entry = {"us_per_solve": us, "err_field_x": err[0], "err_field_y": err[1], "err_potential": err[2]}
            if prec == R.lib.PREC_FP32:
                achieved = 16.0 * side * side / (us * 1e-6) / 1e9
                entry.update({"bound": "hbm", "achieved_gbs": achieved, "frac": achieved / peak,
                              "peak_kind": peak_kind})
            else:
                flops = 16.0 * float(side) ** 3 * (3 if prec == R.lib.PREC_BF16X3_GEMM else 1)
                tfs = flops / (us * 1e-6) / 1e12
                pk = tpeak if prec == R.lib.PREC_BF16X3_GEMM else tpeak / 2.0
                entry.update({"bound": "tensor", "tensor_tflops": tfs, "peak_tflops": pk, "frac": tfs / pk,
                              "peak_kind": tpeak_kind if prec == R.lib.PREC_BF16X3_GEMM
                              else tpeak_kind + " bf16 / 2 (tf32 nominal ratio)"})
            row[name] = entry
            sol.close()
        out[f"{side}x{side}"] = row
    return out


def mixed_section(args, device, d, cfg, sc_fp32, tto_fp32):
    """The 1M-cell design end to end with the spectral solve on the tensor cores
    (TF32; BF16 hi/lo x3), against the plain FP32 path: iterations/s over the
    same number of iterations as the timed FP32 run (plus its warm-up); HPWL and
    overflow at the FP32 path's time-to-overflow-0.10 iteration count (the end
    of the run lies in the reference loop's diverging phase, where any
    perturbation grows); and the time to overflow 0.10 from a fresh context."""
    import torch
    import reda_erplacer_gb300 as R
    m, n = cfg["bins"]
    iters = int(sc_fp32["iteration"])
    ref_it = tto_fp32["iterations"] if tto_fp32 else None
    out = {"iterations": iters, "compare_at_iteration": ref_it,
           "fp32": {"hpwl": tto_fp32["hpwl"] if tto_fp32 else None,
                    "overflow": tto_fp32["overflow"] if tto_fp32 else None}}
    for name, prec in (("tf32_dct_gemm", R.lib.PREC_TF32_GEMM), ("bf16x3_dct_gemm", R.lib.PREC_BF16X3_GEMM)):
        entry = {}
        pl = R.Placement(d, (m, n), cfg["target_density"], start_mode=1, device=device, precision=prec)
        pl.synchronize()
        t0 = time.perf_counter()
        it, _ = pl.run(iters, stop_overflow=0.0)
        pl.synchronize()
        entry["iters_per_s"] = it / (time.perf_counter() - t0)
        pl.close()
        if ref_it:
            pc = R.Placement(d, (m, n), cfg["target_density"], start_mode=1, device=device, precision=prec)
            _, lc = pc.run(ref_it, stop_overflow=0.0)
            pc.close()
            entry.update({"hpwl": lc["hpwl"], "overflow": lc["overflow"],
                          "hpwl_rel_diff": (lc["hpwl"] - tto_fp32["hpwl"]) / tto_fp32["hpwl"],
                          "overflow_abs_diff": lc["overflow"] - tto_fp32["overflow"]})
        pt = R.Placement(d, (m, n), cfg["target_density"], start_mode=1, device=device, precision=prec)
        pt.synchronize()
        t0 = time.perf_counter()
        it_t, last_t = pt.run(cfg["iterations"], stop_overflow=0.10)
        pt.synchronize()
        entry["time_to_overflow"] = {"reached": bool(last_t["overflow"] <= 0.10), "iterations": it_t,
                                     "seconds": time.perf_counter() - t0}
        pt.close()
        out[name] = entry
    torch.cuda.synchronize()
    return out


class LazyJobs:
    """The serving stream's jobs, generated on a thread pool just ahead of use
    (at most `ahead` outstanding); the server copies a design when it is
    submitted, so each one is dropped once taken."""

    def __init__(self, specs, ahead=256):
        from concurrent.futures import ThreadPoolExecutor
        import reda_erplacer_gb300 as R
        self.make = R.design.batch_job
        self.specs = specs
        self.ex = ThreadPoolExecutor(max(1, os.cpu_count() or 1))
        self.fut = {}
        self.next = 0
        self.ahead = ahead

    def __len__(self):
        return len(self.specs)

    def __getitem__(self, i):
        while self.next < len(self.specs) and self.next <= i + self.ahead:
            self.fut[self.next] = self.ex.submit(self.make, *self.specs[self.next])
            self.next += 1
        return self.fut.pop(i).result()

    def close(self):
        self.ex.shutdown(wait=False, cancel_futures=True)


def serve_section(args, device, world=1, rank=0):
    """Serving workload: an open-loop stream of jobs (cells log-uniform 5k-500k,
    each its own seed) with Poisson arrivals at 80 % of the server's measured
    capacity; admission under a 150 GB HBM budget, retire at overflow <= 0.10 or
    600 iterations.  p50/p99 completion latency and jobs/hour of the
    continuous-batching server, and of the same stream served one job at a
    time.  The capacity is that of the same server (same limits) overloaded by
    the stream's first 256 jobs arriving at 200 per second: its steady completion
    rate, the middle half of the completions over the time they took (the ramp
    and the tail, where the GPU is not full, left out); set-up and admission are
    inside it.  With several ranks each GPU runs
    its own server, the capacity is the sum of the ranks' pilots and each
    arriving job is routed to the rank with the least assigned work (host-side
    dispatch, no collective)."""
    import numpy as np
    import reda_erplacer_gb300 as R
    from reda_erplacer_gb300.dispatch import job_cost, route_stream
    from reda_erplacer_gb300.serving import Server, run_stream
    specs = R.design.batch_specs(count=args.serve_jobs, seed=9000, min_cells=5000, max_cells=500000)
    n_pilot = min(256, len(specs))
    pilot = LazyJobs(specs[:n_pilot])
    sv = Server(max_active=64, hbm_budget_gb=150.0, max_iterations=args.batch_iters, stop_overflow=0.10, chunk=8,
                device=device)
    res = run_stream(sv, pilot, np.arange(n_pilot) / 200.0)
    sv.close()
    pilot.close()
    fin = np.sort([r["finish_s"] for r in res])
    q1, q3 = len(fin) // 4, (3 * len(fin)) // 4
    cap = allreduce_sum((q3 - q1) / max(fin[q3] - fin[q1], 1e-9), world)
    rate = 0.8 * cap
    rng = np.random.default_rng(17)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(specs)))
    route = route_stream([job_cost(sp[0]) for sp in specs], world)
    mine = [i for i, r in enumerate(route) if r == rank]
    out = {"jobs": len(specs), "ranks": world, "capacity_jobs_per_s": cap, "arrival_rate_jobs_per_s": rate,
           "hbm_budget_gb": 150.0, "max_iterations": args.batch_iters, "stop_overflow": 0.10}
    for name, max_active in (("continuous_batching", 64), ("one_at_a_time", 1)):
        jobs = LazyJobs([specs[i] for i in mine])
        sv = Server(max_active=max_active, hbm_budget_gb=150.0, max_iterations=args.batch_iters,
                    stop_overflow=0.10, chunk=8, device=device)
        barrier(world)
        res = run_stream(sv, jobs, arrivals[mine])
        sv.close()
        jobs.close()
        span = allreduce_max(max(r["finish_s"] for r in res) - min(r["submit_s"] for r in res) if res else 0.0,
                             world)
        res = gather_items([{"latency_s": r["latency_s"], "status": r["status"],
                             "last": {"overflow": r["last"]["overflow"]}} for r in res], world)
        lat = np.array([r["latency_s"] for r in res])
        at_ovf = np.array([r["last"]["overflow"] <= 0.10 for r in res], bool)

        def pct(a, q):
            return float(np.percentile(a, q)) if len(a) else None
        out[name] = {"p50_latency_s": pct(lat, 50), "p99_latency_s": pct(lat, 99),
                     "jobs_per_hour": len(res) / span * 3600.0, "makespan_s": span,
                     "failed": int(sum(1 for r in res if r["status"] != 0)),
                     "retired_at_overflow": int(at_ovf.sum()),
                     # the jobs that reached overflow 0.10 and those that ran into the
                     # iteration cap, apart (the loop's overflow minimum lies above
                     # 0.10 for some designs, alone as in the mix)
                     "retired_at_overflow_p50_s": pct(lat[at_ovf], 50),
                     "retired_at_overflow_p99_s": pct(lat[at_ovf], 99),
                     "capped_p50_s": pct(lat[~at_ovf], 50), "capped_p99_s": pct(lat[~at_ovf], 99)}
    return out


def run_reference(args):
    """The reference arm: the CPU restatement of the reference loop in its own
    FP32 rules, on all host threads, on the same workload and config as the
    GPU arm.  Its input comes from the generator compiled on its own
    (oracle/_build/liberp_synth.so); the product library is never loaded."""
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    from oracle import erp_oracle as O
    d, cfg, desc = make_workload(args.workload, O.synth)
    iters = args.ref_steps if args.ref_steps > 0 else args.steps
    warm = max(3, args.warmup)
    v, dt = cpu_sample(d, cfg, iters, literal=True, warmup=warm)
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
        "steps": iters, "warmup": warm, "ms_per_step": 1000.0 * dt / iters,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(d, cfg, desc),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{iters} full iterations of the workload after {warm} untimed "
                                   f"iterations, rank 0 only; oracle in the reference's FP32 rules "
                                   f"(sequential density below iteration 200, then atomic adds)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def phase_state(args):
    """--save-state / --profile-state: a checkpoint of the workload at one
    iteration, written by one process and profiled by another, so that a
    profiler attached to the second sees the stage launches of that phase without
    the hundreds of launches that led to it."""
    import torch
    import __graft_entry__ as G
    G.build_product()
    import reda_erplacer_gb300 as R
    d, cfg, _ = make_workload(args.workload, R.synth)
    m, n = cfg["bins"]
    pl = R.Placement(d, (m, n), cfg["target_density"], start_mode=1)
    if args.save_state:
        its, path = int(args.save_state[0]), args.save_state[1]
        pl.run(its)
        pl.synchronize()
        with open(path, "wb") as f:
            f.write(pl.checkpoint())
        print(json.dumps({"saved": path, "iteration": pl.scalars()["iteration"]}), flush=True)
    else:
        with open(args.profile_state, "rb") as f:
            pl.restore(f.read())
        for _ in range(16):
            pl.step(stats=False)
        pl.synchronize()
        ms = pl.profile_stages(reps=1)
        print(json.dumps({"iteration": pl.scalars()["iteration"], "stage_ms": ms}), flush=True)
    pl.close()
    torch.cuda.synchronize()
    return 0


def batch_only(args):
    """--batch-only NAME: build one batch (NAME "mix": the 64-design mix; "tiny_mix":
    64 designs of 2,000-4,000 cells on 64^2 bins) in the form the environment
    variable ERP_BATCH_FORM names, run it to 600 iterations or overflow <= 0.10,
    print its time and exit: a profiler's view of the batched launches alone."""
    import torch
    import __graft_entry__ as G
    G.build_product()
    import reda_erplacer_gb300 as R
    if args.batch_only == "mix":
        jobs = R.workload_batch(count=64)
    else:
        jobs = R.workload_batch(count=64, seed=4100, min_cells=2000, max_cells=4000)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = R.Batch([d for d, _ in jobs], [x for _, x in jobs], 1.0, start_mode=1)
    its, _ = b.run(args.batch_iters, stop_overflow=0.10)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    print(json.dumps({"batch": args.batch_only, "form": os.environ.get("ERP_BATCH_FORM", "packed"),
                      "instances": len(jobs), "packed_instances": b.packed_instances(),
                      "scatter_cells_per_block": b.tuning()[0], "spectral_seqs_per_block": b.spectral_tuning()[0],
                      "iterations_total": int(sum(its)), "s": dt}), flush=True)
    b.close()
    return 0


def run_ours(args):
    world, rank, local = dist_setup()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    import __graft_entry__ as G
    G.build_product()
    import reda_erplacer_gb300 as R

    d, cfg, desc = make_workload(args.workload, R.synth)
    m, n = cfg["bins"]
    stream = torch.cuda.Stream()
    pl = R.Placement(d, (m, n), cfg["target_density"], start_mode=1, device=local,
                     stream=stream.cuda_stream)
    for _ in range(args.warmup):
        pl.step(stats=False)
    pl.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        pl.step(stats=False)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms_local = e0.elapsed_time(e1)
    clk = clocks.stop()
    ms = allreduce_max(ms_local, world)
    sc = pl.scalars()
    st = pl.scalars()
    x_h, y_h = pl.positions()
    value = world * args.steps / (ms / 1000.0)
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms / args.steps,
                              "graph_kernels": st["graph_kernels"], "quick": True}), flush=True)
        pl.close()
        return 0

    # end to end through the drop-in host-coordinate call, pinned buffers
    N = d.num_nodes
    xp = torch.from_numpy(x_h).pin_memory()
    yp = torch.from_numpy(y_h).pin_memory()
    xa, ya = xp.numpy(), yp.numpy()
    e2e_steps = max(3, min(args.steps, 50))
    pl.step_host(xa, ya)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        last = pl.step_host(xa, ya)
    torch.cuda.synchronize()
    e2e_s = allreduce_max(time.perf_counter() - t0, world)
    e2e_value = world * e2e_steps / e2e_s
    h2d = 8 * N
    d2h = 8 * N + 256

    # roofline of the dominant stage (isolated launches, L2 flushed)
    stages = pl.profile_stages(reps=args.profile_reps)
    # the roofline's kernel: k_wa (the "wirelength" stage is that one kernel),
    # the largest single kernel of the step's launch list
    dom = "wirelength"
    B = m * n
    alg = {k: ALG_BYTES[k](d.num_movable, d.num_pins, d.num_nets, B) for k in stages}
    peak, peak_kind = measured_peak_gbs()
    achieved = alg[dom] / (stages[dom] * 1e-3) / 1e9
    traffic = NCU_TRAFFIC.get((args.workload, dom))
    per_stage = {k: {"ms": stages[k], "alg_bytes": alg[k],
                     "gbs": (alg[k] / (stages[k] * 1e-3) / 1e9) if stages[k] > 0 else None}
                 for k in stages}
    pl.close()

    # time to overflow 0.10 from the same start: a fresh context, erp_run with
    # the stop threshold, wall clock up to the run's return (it synchronises)
    tto = None
    if not args.no_tto:
        pt = R.Placement(d, (m, n), cfg["target_density"], start_mode=1, device=local)
        pt.synchronize()
        t0 = time.perf_counter()
        it_t, last_t = pt.run(cfg["iterations"], stop_overflow=0.10)
        pt.synchronize()
        tto = {"target_overflow": 0.10, "reached": bool(last_t["overflow"] <= 0.10),
               "iterations": it_t, "seconds": time.perf_counter() - t0,
               "overflow": last_t["overflow"], "hpwl": last_t["hpwl"],
               "call": "erp_run(max_iterations, stop_overflow=0.10), context created beforehand"}
        pt.close()

    # the workload's whole run (its configured iteration count) from a fresh
    # context: the device-resident rate over every phase of the run (CUDA
    # events, no per-step host sync), then the same run again with each step's
    # HPWL and overflow read back, for the comparison with the reference loop
    full = None
    gpu_trace = []
    if not args.no_full:
        pf = R.Placement(d, (m, n), cfg["target_density"], start_mode=1, device=local,
                         stream=stream.cuda_stream)
        pf.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(cfg["iterations"]):
            pf.step(stats=False)
        f1.record(stream)
        torch.cuda.synchronize()
        fms = f0.elapsed_time(f1)
        pf.close()
        full = {"iterations": cfg["iterations"], "iters_per_s": cfg["iterations"] / (fms / 1000.0),
                "ms_per_step": fms / cfg["iterations"],
                "note": "fresh context, every iteration of the workload (spreading, converged and "
                        "diverging phases); CUDA events on the context's stream"}
        pg = R.Placement(d, (m, n), cfg["target_density"], start_mode=1, device=local)
        for _ in range(cfg["iterations"]):
            pg.step()
            gpu_trace.append((pg.last_stats["hpwl"], pg.last_stats["overflow"]))
        pg.close()

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(d, cfg, desc),
        "timed_window": {"first_iteration": args.warmup, "iterations": args.steps,
                         "iteration_after": sc["iteration"], "hpwl_after": sc["hpwl_current"],
                         "overflow_after": sc["overflow_current"]},
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps, "call": "erp_step_host"},
        "gpu_launches": int(st["graph_kernels"]) * args.steps,
        "roofline": {"kernel": "k_wa", "stage": dom, "bound": "hbm", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "traffic_source": "ncu capture of k_wa on this workload (dram read + write per "
                                       "launch), not measured by this run",
                     "alg_bytes": alg[dom], "ms": stages[dom]},
        "stages": per_stage,
        "time_to_overflow": tto,
        "full_run": full,
    }
    if args.batch_count > 0:
        line["batched"] = batch_section(args, local, world, rank)
    if not args.no_spectral:
        line["spectral_solve"] = spectral_section(args, local)
    if not args.no_mixed:
        line["mixed_form"] = mixed_section(args, local, d, cfg, sc, tto)
    if args.serve_jobs > 0:
        line["serving"] = serve_section(args, local, world, rank)
    if rank == 0 and world == 1 and not args.no_cpu:
        # the reference loop on the host cores: the oracle in the reference's own
        # FP32 rules over the workload's whole run from the same start (one
        # untimed first step); its trajectory is the CPU result the GPU run is
        # compared with
        iters = args.cpu_iters if args.cpu_iters > 0 else cfg["iterations"]
        v, dt, ref_trace = cpu_sample(d, cfg, iters - 1, literal=True, warmup=1, trace=True)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": f"iterations 2-{iters} of the same workload from the same start "
                                          f"(oracle in the reference's FP32 rules, OpenMP on all host "
                                          f"threads), {dt:.1f} s"}
        if gpu_trace and len(ref_trace) == len(gpu_trace):
            tto_it = tto["iterations"] if tto and tto["reached"] else None
            line["parity_vs_reference"] = parity_summary(gpu_trace, ref_trace, tto_it)
            # The FP32 rules are not deterministic past iteration 200 (per-bin
            # atomic adds in thread order, as the reference's Mutex-guarded bins):
            # the same loop in its deterministic FP64 form, through the converged
            # state, shows how much of the difference is the reference's own noise.
            k64 = min(len(gpu_trace), max(tto_it or 0, 520) + 40)
            _, dt64, ref64 = cpu_sample(d, cfg, k64 - 1, literal=False, warmup=1, trace=True)
            line["parity_vs_reference_fp64_form"] = parity_summary(gpu_trace[:k64], ref64, tto_it)
            line["parity_vs_reference_fp64_form"]["note"] = (
                f"oracle in the reference loop's FP64 form (fixed-point map, FP64 sums), iterations 1-{k64}, "
                f"{dt64:.1f} s; the FP32-rules run above differs from it by the reference's own rounding")
            if tto_it:
                a32, a64 = ref_trace[tto_it - 1][0], ref64[tto_it - 1][0]
                line["parity_vs_reference_fp64_form"]["fp32_rules_vs_fp64_form_hpwl_rel_at_0.10"] = (a32 - a64) / a64
    if rank == 0:
        line["summary"] = summary(line)
        print(json.dumps(line), flush=True)
    return 0


def summary(line):
    """The headline figures of every section in a few short keys; printed last
    in the line, so that a reader who sees only its tail still has them."""
    out = {"iters_per_s": round(line["value"], 1), "e2e_iters_per_s": round(line["e2e"]["value"], 1)}
    if line.get("full_run"):
        out["full_run_iters_per_s"] = round(line["full_run"]["iters_per_s"], 1)
    t = line.get("time_to_overflow")
    if t:
        out["time_to_overflow_0.10_s"] = round(t["seconds"], 4)
        out["time_to_overflow_0.10_iterations"] = t["iterations"]
    cb = line.get("cpu_baseline")
    if cb:
        out["cpu_reference_iters_per_s"] = round(cb["value"], 2)
    pv = line.get("parity_vs_reference")
    if pv:
        k = pv.get("at_overflow_0.10", pv["last"])
        out["parity_at_iteration"] = k["iteration"]
        out["parity_hpwl_rel"] = round(k["hpwl_rel"], 5)
        out["parity_overflow_abs"] = round(k["overflow_abs"], 5)
        out["parity_min_overflow_abs"] = round(pv["overflow_min"]["overflow_abs"], 5)
        out["parity_hpwl_rel_at_min_overflow"] = round(pv["overflow_min"]["hpwl_rel"], 5)
    p64 = line.get("parity_vs_reference_fp64_form")
    if p64 and "at_overflow_0.10" in p64:
        out["parity_hpwl_rel_fp64_form"] = round(p64["at_overflow_0.10"]["hpwl_rel"], 5)
        out["parity_overflow_abs_fp64_form"] = round(p64["at_overflow_0.10"]["overflow_abs"], 5)
        out["reference_fp32_vs_fp64_form_hpwl_rel"] = round(p64["fp32_rules_vs_fp64_form_hpwl_rel_at_0.10"], 5)
    b = line.get("batched")
    if b:
        out["batched_jobs_per_hour"] = round(b["jobs_per_hour_batched"])
        out["one_at_a_time_jobs_per_hour"] = round(b["jobs_per_hour_sequential"])
        out["batched_speedup"] = round(b["speedup"], 3)
        f = b.get("forms")
        if f:
            out["batched_branches_jobs_per_hour"] = round(f["mix_branches_jobs_per_hour"])
            out["tiny_mix_packed_jobs_per_hour"] = round(f["tiny_mix_packed_jobs_per_hour"])
            out["tiny_mix_branches_jobs_per_hour"] = round(f["tiny_mix_branches_jobs_per_hour"])
        out["mixed_batched_speedup"] = round(b["mixed_batched"]["speedup_vs_fp32_one_at_a_time"], 3)
    sv = line.get("serving")
    if sv:
        cb_ = sv["continuous_batching"]
        out["serving_p50_s"] = round(cb_["p50_latency_s"], 3)
        out["serving_p99_s"] = round(cb_["p99_latency_s"], 3)
        out["serving_jobs_per_hour"] = round(cb_["jobs_per_hour"])
        out["serving_retired_at_overflow"] = cb_["retired_at_overflow"]
    sp = line.get("spectral_solve", {}).get("1024x1024")
    if sp:
        out["solve_1024_us"] = {k: round(v["us_per_solve"], 1) for k, v in sp.items()}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["large", "small"], default="large")
    ap.add_argument("--profile-reps", type=int, default=10)
    ap.add_argument("--cpu-iters", type=int, default=0,
                    help="iterations of the CPU reference run beside the GPU arm (0: the workload's count)")
    ap.add_argument("--ref-steps", type=int, default=0,
                    help="timed iterations of the reference arm (0: the same as --steps)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true", help="timed steps only (for profiler runs)")
    ap.add_argument("--batch-count", type=int, default=64, help="instances of the batched section (0: skip)")
    ap.add_argument("--batch-iters", type=int, default=600)
    ap.add_argument("--no-tto", action="store_true", help="skip the time-to-overflow-0.10 run")
    ap.add_argument("--no-full", action="store_true", help="skip the whole-run rate and trajectory")
    ap.add_argument("--no-spectral", action="store_true", help="skip the isolated-solve section")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision end-to-end runs")
    ap.add_argument("--spectral-reps", type=int, default=20)
    ap.add_argument("--serve-jobs", type=int, default=2000, help="jobs of the serving stream (0: skip)")
    ap.add_argument("--save-state", nargs=2, metavar=("ITERATIONS", "PATH"),
                    help="run the workload ITERATIONS iterations, write its checkpoint to PATH and exit")
    ap.add_argument("--profile-state", metavar="PATH",
                    help="restore the workload from the checkpoint at PATH, run 16 steps (the scatter order "
                         "follows the cells), launch every stage alone twice (erp_profile_stages, one timed "
                         "launch after one untimed) and exit: a profiler's view of one phase of the run")
    ap.add_argument("--batch-only", choices=["mix", "tiny_mix"], default=None,
                    help="run one batch (the 64-design mix or 64 tiny designs) in the form "
                         "ERP_BATCH_FORM names and exit: a profiler's view of the batched launches")
    args = ap.parse_args()
    if args.save_state or args.profile_state:
        return phase_state(args)
    if args.batch_only:
        return batch_only(args)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python
"""Benchmark of one NICAM NSW6 microphysics step on GB300.

Workload (N=1): gall = 16900 (130 x 130 points), kall = 42, lall = 10 regions
(7.1 M cells), dt = 60 s, FP64, seeded synthetic states (the NICAM snapshot the
reference ships without is replaced by nicam_kokkos_microphysics_gb300.state).
A step is one mp_driver call over all regions, in place, as the reference
harness loops over SET_iteration (src/main.cpp:261-319).  The working set
(about 3 GB) is far larger than the 129 MB L2, so no flush is needed between
steps.

Metric: cells per second per NSW6 step (gall * kall * lall / step time).  The
default line also carries the other two parts of the metric: the
mixed-precision step on the same workload (its rate, end to end, and its
per-field errors against the FP64 step), the adjoint / forward time ratio of
one FP64 step (4096 x 42) and of the 12-step checkpointed window (5 regions of
16900 x 42, forward FP64 and mixed-precision).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

For N > 1 (torchrun, one process per GPU) the N * lall regions are split into
one block of lall regions per rank (shard_regions; weak scaling, no collective
on the data path); rank 0 prints the line with value = all cells / max step
time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from nicam_kokkos_microphysics_gb300.state import (ARG_NAMES, MP_DRIVER_ARGS, StateSpec, batched_shape,  # noqa: E402
                                                   make_state, region_view, shard_regions)

METRIC = "cells/sec per NSW6 step (FP64)"
METRIC_MIXED = "cells/sec per NSW6 step (mixed precision)"
UNIT = "cells/s"
# Algorithmic bytes of one step per cell: 21 FP64 fields read and 28 written
# (the minimum the step must touch, without read-for-ownership) plus ~3 B of
# per-column outputs at kall = 42.
ALGO_BYTES_PER_CELL = 49 * 8 + 3
# Algorithmic bytes of the cell kernel per interior cell: it reads rhog,
# rhogq(6), q(QV), tem, gsgam2 and writes rhog, rhoge, tem, rhogq(6), q(5),
# re_liquid, re_cld.
CELL_KERNEL_BYTES_PER_CELL = (10 + 17) * 8
# Per launch of each kernel, from ncu captures of one 16900 x 42 region
# (profiles/fp64_work_16900x42.md; every figure grows in proportion to the
# cells): DRAM bytes read + written, and the FP64 thread instructions the
# kernel executes -- DFMA, DADD, DMUL and all instructions of the FP64 pipe
# (compares, min/max and conversions included) -- per interior cell (cell
# kernel) or per cell (column phase).  The column phase is nsw6_column_kernel
# and nsw6_satadj_kernel (the saturated cells), timed together as one
# interval; its figures are the two kernels' sums.
CELL_KERNEL_TRAFFIC_PER_CELL = {"fp64": 229.0, "mixed": 172.4}
COLUMN_KERNEL_TRAFFIC_PER_CELL = {"fp64": 379.8 + 30.0, "mixed": 386.4 + 30.0}
FP64_EXECUTED = {
    "nsw6_cell_kernel": {"fp64": {"dfma": 353.9, "dadd": 258.8, "dmul": 273.0, "pipe": 901.5},
                         "mixed": {"dfma": 5.0, "dadd": 43.0, "dmul": 20.1, "pipe": 91.9}},
    "nsw6_column_kernel": {"fp64": {"dfma": 113.8 + 9.9, "dadd": 137.4 + 6.0, "dmul": 144.8 + 5.4,
                                    "pipe": 403.0 + 21.6},
                           "mixed": {"dfma": 37.3 + 9.0, "dadd": 69.0 + 5.8, "dmul": 55.8 + 6.2,
                                     "pipe": 208.5 + 21.4}},
}
# FP64-pipe activity (fraction of active cycles) of each kernel in the same
# captures (cold, serialised launches; the column kernel alone).
FP64_PIPE_ACTIVE = {"nsw6_cell_kernel": {"fp64": 0.839, "mixed": 0.656},
                    "nsw6_column_kernel": {"fp64": 0.732, "mixed": 0.585}}
# FP64 op weights in flop equivalents (an FMA counts 2): the cost of CUDA's FP64
# divide, sqrt, exp, log and pow relative to DFMA, measured once on a GB300 with
# the throughput probe (probe/nsw6_probe.cu) and frozen here.
OP_WEIGHTS = {"add": 1.0, "mul": 1.0, "cmp": 1.0, "div": 15.0, "sqrt": 15.2, "exp": 30.0, "log": 58.4,
              "pow": 173.8}
ADJOINT_LAUNCHES = 12   # kernels of one mp_driver_adjoint call (hand-written sweeps)


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x: float, dist=None, device: str = "cuda") -> float:
    """The slowest rank's time (the job's time); x itself without a process group."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cells_per_rank: int, world: int, seconds: float) -> float:
    """Cells of all ranks per second of the slowest rank."""
    return cells_per_rank * world / seconds


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def workload_config(spec: StateSpec, precision: str, world: int) -> dict:
    """The `config` of both arms' lines (identical on the same workload)."""
    return {"workload": f"NSW6 {'mixed-precision' if precision == 'mixed' else 'FP64'} step, gall={spec.gall} "
                        f"kall={spec.kall} lall={spec.lall} per GPU ({spec.cells} cells), dt={spec.dt}",
            "variant": spec.variant, "precision": precision, "l2": "working set >> L2 (no flush needed)",
            "parallelism": f"regions x{world}"}


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def fp64_rates():
    """Measured FP64 rates of this GPU (throughput probe): DFMA per second and
    the op weights of the CUDA FP64 functions in FP64 flop equivalents (an FMA
    counts 2, so weight = 2 x DFMA rate / function rate, less the additions
    and multiplications the probe loop wraps around each call)."""
    import ctypes
    from probe import build as probe_build
    if not probe_build.LIB.exists():
        return None
    lib = ctypes.CDLL(str(probe_build.LIB))
    lib.nsw6_probe_rate.restype = ctypes.c_double
    lib.nsw6_probe_rate.argtypes = [ctypes.c_int, ctypes.c_int]
    r = {n: lib.nsw6_probe_rate(i, it) for i, (n, it) in
         enumerate([("dfma", 4000), ("dadd", 4000), ("dmul", 4000), ("div", 1000), ("sqrt", 1000),
                    ("exp", 500), ("log", 500), ("pow", 250)])}
    if min(r.values()) <= 0:
        return None
    extra = {"div": 0, "sqrt": 1, "exp": 2, "log": 1, "pow": 1}
    w = {"add": 1.0, "mul": 1.0, "cmp": 1.0}
    for k, e in extra.items():
        w[k] = 2.0 * (r["dfma"] / r[k] - e)
    return {"dfma_per_s": r["dfma"], "peak_tflops": 2.0 * r["dfma"] / 1e12, "weights": w, "rates": r}


def algorithmic_work(spec: StateSpec, st: dict, weights: dict) -> dict:
    """FP64 work per cell of the reference algorithm on region 0 of the state,
    counted by the operation-counting build of the oracle (integer powers as
    products), weighted with the measured op weights."""
    from oracle import restatement
    reg = region_view(st, 0)
    c = restatement.count_ops(reg, st["_gz"], st["_gzh"], spec.dt)
    n_int = spec.gall * (spec.kall - 2)
    n_all = spec.gall * spec.kall

    def work(ph):
        return sum(c[ph][k] * weights[k] for k in c[ph])

    return {"cell_per_interior_cell": (work("cell") + work("zdis")) / n_int,
            "column_per_cell": work("column") / n_all}


# ----------------------------------------------------------------- CPU side
def cpu_reference_sample(spec: StateSpec, steps: int, use_port: bool = False):
    """Time the reference's CPU implementation on one region per step.

    Uses the reference's own sources built with the OpenMP Kokkos shim
    (oracle/_ref) when they are available, else the OpenMP build of the C
    restatement.  Returns (cells/s, kind, threads, seconds per step list)."""
    one = StateSpec(gall=spec.gall, kall=spec.kall, lall=1, seed=spec.seed, variant=spec.variant, dt=spec.dt)
    st = make_state(one, out_fill=0.0)
    step, kind, threads = _reference_stepper(one, st)
    regs = [region_view(st, 0)]
    step(regs)  # warm-up
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        step(regs)
        times.append(time.perf_counter() - t0)
    return one.gall * one.kall / statistics.median(times), kind, threads, times


def _reference_stepper(spec: StateSpec, st: dict):
    """A function stepping a list of per-region argument sets in place with
    the reference's CPU build (oracle/_ref, OpenMP shim) or, where the
    reference sources are absent, the OpenMP build of the C restatement."""
    from oracle import build_ref, restatement
    if build_ref.sources_available():
        from oracle import ref
        lib = ref.load(spec.gall, spec.kall, st["_gz"], st["_gzh"], variant="omp")

        def step(regs):
            for r in regs:
                if ref.mp_driver(lib, r, spec.dt) != 0:
                    raise RuntimeError("reference step failed")
        return step, "reference", os.cpu_count()
    lib = restatement.load("omp")

    def step(regs):
        for r in regs:
            rc, status = restatement.mp_driver(r, st["_gz"], st["_gzh"], spec.dt, variant="omp")
            if rc != 0:
                raise RuntimeError(f"restatement step failed: {status}")
    return step, "port", lib.nsw6o_max_threads()


def run_reference_arm(args):
    """The reference's CPU implementation on the GPU arm's workload: every
    step is one mp_driver call per region over all lall regions (the
    reference harness's loop, src/main.cpp:261-319), the state evolving in
    place; W warm-up steps, then the mean of K timed steps."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    spec = StateSpec(gall=args.gall, kall=args.kall, lall=args.lall, seed=args.seed, variant=args.variant)
    st = make_state(spec, out_fill=0.0)
    step, kind, threads = _reference_stepper(spec, st)
    regs = [region_view(st, l) for l in range(spec.lall)]
    for _ in range(args.warmup):
        step(regs)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(regs)
    ms = (time.perf_counter() - t0) / args.steps * 1e3
    v = spec.cells / (ms * 1e-3)
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded NICAM-like state)",
        "impl": "reference",
        "config": workload_config(spec, "fp64", 1),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"all {spec.lall} regions of {spec.gall}x{spec.kall} cells per step, "
                                   f"{args.warmup} warm-up + {args.steps} timed steps (mean), OpenMP"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# Fields whose error the mixed path reports, and the reduction that gives it:
# per field, max |mixed - fp64| / max |fp64| (field-normalised maximum) and
# the mean over cells with |fp64| >= 1e-3 max |fp64| of the per-cell relative
# error; tracers per species.
MIXED_FIELDS = ["rhog", "rhogvx", "rhogvy", "rhogvz", "rhogw", "rhoge", "rhogq", "q", "tem", "precip",
                "precip_rhoe", "precip_lh_heat", "GPREC"]
SPECIES = ["QV", "QC", "QR", "QI", "QS", "QG"]


def field_errors(a, b) -> dict:
    d = (a - b).abs()
    bmax = b.abs().max()
    sig = (b.abs() >= 1e-3 * bmax) & (b.abs() > 0)   # a field that is zero everywhere has no relative error
    rel = d[sig] / b.abs()[sig]
    return {"max_rel_field": float(d.max() / bmax) if bmax > 0 else 0.0,
            "mean_rel": float(rel.mean()) if rel.numel() else 0.0,
            "max_rel_cell": float(rel.max()) if rel.numel() else 0.0}


def mixed_vs_fp64(drv, spec: StateSpec, st0: dict) -> dict:
    """One step of the FP64 path and one of the mixed path from the same state."""
    import torch
    ref = {n: torch.from_numpy(st0[n]).cuda() for n in ARG_NAMES}
    mix = {n: t.clone() for n, t in ref.items()}
    drv.set_precision("fp64")
    drv.mp_driver_batched(spec.lall, *[ref[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    drv.set_precision("mixed")
    drv.mp_driver_batched(spec.lall, *[mix[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    torch.cuda.synchronize()
    out = {}
    for n in MIXED_FIELDS:
        a, b = mix[n], ref[n]
        if n in ("rhogq", "q"):
            for s, sp in enumerate(SPECIES):
                out[f"{n}[{sp}]"] = field_errors(a[:, s], b[:, s])
        else:
            out[n] = field_errors(a, b)
    return out


# ----------------------------------------------------------------- GPU side
def time_device_steps(drv, lall: int, dev: dict, dt: float, steps: int, dist=None):
    """Mean time of `steps` steps on device-resident arrays (CUDA events on the
    library's stream, a synchronize on both sides), and the mean time of its
    cell and column kernels (events inside the library)."""
    import torch
    args_dev = [dev[n] for n in ARG_NAMES]
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    drv.set_timing(True)
    drv.read_timing()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        drv.mp_driver_batched(lall, *args_dev, dt=dt, ct=0.0)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t_cell, t_col, n = drv.read_timing()
    drv.set_timing(False)
    rc, cell = drv.last_error()
    if rc != 0:
        raise RuntimeError(f"timed steps failed with status {rc} at {cell}")
    return e0.elapsed_time(e1) / steps, t_cell / max(n, 1), t_col / max(n, 1)


def time_end_to_end(drv, spec: StateSpec, st: dict, steps: int, world: int, dist=None) -> dict:
    """The same step through the public host-memory entry point
    (mp_driver_argv with host = 1, via MPDriver.run on pinned numpy arrays):
    every step copies what it reads of the arguments to the device and the
    arguments it writes back inside the call; the byte counts are the
    library's own (nsw6_host_copy_bytes)."""
    import torch
    host = {}
    for n in ARG_NAMES:
        t = torch.empty(st[n].shape, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = st[n]
        host[n] = t.numpy()
    h2d, d2h = drv.host_copy_bytes(spec.lall)
    drv.run(host, dt=spec.dt)  # warm-up (allocates the staging buffers)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        drv.run(host, dt=spec.dt)
    dt_e2e = max_over_ranks((time.perf_counter() - t0) / steps, dist)
    return {"value": whole_job_rate(spec.cells, world, dt_e2e), "unit": UNIT,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": dt_e2e * 1e3}


def roofline_of(kernel_ms: dict, spec: StateSpec, precision: str, rates, aw) -> dict:
    """FP64 roofline of the dominant kernel.  Both kernels are bound by the
    FP64 pipe, which issues one DFMA, DADD, DMUL, compare, min/max or
    conversion per thread and slot.  achieved = the FP64-pipe thread
    instructions the kernel executes per launch (ncu, per cell, times the
    cells of a launch) / its mean CUDA-event duration, counted at 2 flops each
    as the peak counts a DFMA; peak = 2 x the DFMA rate the throughput probe
    measures in this run (MEASURED_PEAKS.json has no FP64 figure); frac is the
    share of the FP64 pipe's issue rate the kernel uses.  executed_flops
    counts the arithmetic alone (2 per DFMA, 1 per DADD or DMUL)."""
    peaks, src = measured_peaks()
    n_int = spec.gall * (spec.kall - 2) * spec.lall
    units = {"nsw6_cell_kernel": n_int, "nsw6_column_kernel": spec.cells}
    traffic = {"nsw6_cell_kernel": CELL_KERNEL_TRAFFIC_PER_CELL[precision] * n_int,
               "nsw6_column_kernel": COLUMN_KERNEL_TRAFFIC_PER_CELL[precision] * spec.cells}
    top = max(kernel_ms, key=kernel_ms.get)
    per = {}
    for k, ms in kernel_ms.items():
        d = {"ms": ms, "traffic": traffic[k], "fp64_pipe_active_ncu": FP64_PIPE_ACTIVE[k][precision]}
        ex = FP64_EXECUTED[k][precision]
        if rates and ex:
            d["achieved"] = 2.0 * ex["pipe"] * units[k] / (ms * 1e-3) / 1e12
            d["frac"] = d["achieved"] / rates["peak_tflops"]
            flops = (2.0 * ex["dfma"] + ex["dadd"] + ex["dmul"]) * units[k]
            d["executed_flops_tflops"] = flops / (ms * 1e-3) / 1e12
            d["executed_flops_frac"] = d["executed_flops_tflops"] / rates["peak_tflops"]
        if rates and aw:
            ref_work = aw["cell_per_interior_cell" if k == "nsw6_cell_kernel" else "column_per_cell"] * units[k]
            d["reference_work_rate_over_fp64_peak"] = ref_work / (ms * 1e-3) / 1e12 / rates["peak_tflops"]
        per[k] = d
    hbm_cell = CELL_KERNEL_BYTES_PER_CELL * n_int / (kernel_ms["nsw6_cell_kernel"] * 1e-3) / 1e9
    out = {"kernel": top, "bound": "fp64", "unit": "TFLOP/s", "achieved": per[top].get("achieved"),
           "peak": rates["peak_tflops"] if rates else None, "frac": per[top].get("frac"),
           "traffic": per[top]["traffic"],
           "executed_flops_tflops": per[top].get("executed_flops_tflops"),
           "executed_flops_frac": per[top].get("executed_flops_frac"),
           "peak_source": "measured in this run: FP64 FMA throughput probe, 2 flops per DFMA "
                          "(MEASURED_PEAKS.json has no FP64 peak)",
           "work_definition": "FP64-pipe thread instructions the kernel executes (ncu "
                              "sm__thread_inst_executed_pipe_fp64_pred_on per cell on one 16900 x 42 region, "
                              "profiles/fp64_work_16900x42.md, times the cells of the launch), 2 flops each",
           "kernels": per,
           "column_phase": "nsw6_column_kernel above times the column phase: nsw6_column_kernel and "
                           "nsw6_satadj_kernel (the saturated cells' Newton iteration), one CUDA-event interval",
           "hbm": {"cell_kernel_gbs": hbm_cell, "cell_kernel_frac": hbm_cell / peaks["hbm_gbs"],
                   "peak": peaks["hbm_gbs"], "unit": "GB/s", "peak_source": f"{src} copy bandwidth"}}
    if aw:
        out["reference_work"] = {
            "definition": "the reference algorithm's FP64 operations on this state (oracle op count, integer "
                          "powers as products) weighted add/mul/cmp 1, FMA 2, div/sqrt/exp/log/pow by their "
                          "frozen measured cost; rate / FP64 peak above 1 means the kernel does that work in less "
                          "time than the FP64 pipe needs for it as written",
            "per_interior_cell": aw["cell_per_interior_cell"], "column_per_cell": aw["column_per_cell"],
            "op_weights": OP_WEIGHTS, "op_weights_this_run": rates["weights"] if rates else None}
    return out


def adjoint_ratio(seed: int, variant: str, steps: int, warmup: int) -> dict:
    """Config 4: adjoint / forward time of one FP64 step on 4096 x 42 (one
    region), both timed with CUDA events on the library's stream; the adjoint
    seeded with the loss sum (precip)^2 + column QC."""
    import torch
    from nicam_kokkos_microphysics_gb300 import mp_init
    spec = StateSpec(gall=4096, kall=42, lall=1, seed=seed, variant=variant)
    st = make_state(spec, out_fill=0.0)
    drv = mp_init("NSW6", spec.gall, spec.kall, st["_gz"], st["_gzh"], lall_max=1)
    x0 = {n: torch.from_numpy(st[n]).cuda() for n in ARG_NAMES}
    kinds = {n: k for n, k, _ in MP_DRIVER_ARGS}
    y = {n: t.clone() for n, t in x0.items()}
    for _ in range(warmup):
        drv.mp_driver_batched(1, *[y[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        drv.mp_driver_batched(1, *[y[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    e1.record()
    torch.cuda.synchronize()
    t_fwd = e0.elapsed_time(e1) / steps
    bar0 = {n: torch.zeros(batched_shape(kinds[n], 1, spec.kall, spec.gall), dtype=torch.float64, device="cuda")
            for n in ARG_NAMES}
    seeds = []
    for _ in range(steps + warmup):
        b = {n: t.clone() for n, t in bar0.items()}
        b["precip"].fill_(1.0)
        b["rhogq"][:, 1] = 1.0
        seeds.append(b)
    for b in seeds[:warmup]:
        drv.adjoint(1, x0, b, dt=spec.dt)
    torch.cuda.synchronize()
    e0.record()
    for b in seeds[warmup:]:
        drv.adjoint(1, x0, b, dt=spec.dt)
    e1.record()
    torch.cuda.synchronize()
    t_adj = e0.elapsed_time(e1) / steps
    drv.close()
    return {"ratio": t_adj / t_fwd, "forward_ms": t_fwd, "adjoint_ms": t_adj,
            "workload": f"adjoint of one FP64 step, gall={spec.gall} kall={spec.kall} lall=1, dt={spec.dt}",
            "timing": "CUDA events on the library's stream, both sides", "steps": steps, "warmup": warmup}


def window_ratio(seed: int, variant: str, nsteps: int = 12, lall: int = 5) -> dict:
    """Config 5: gradient of the window-accumulated surface precipitation over
    `nsteps` steps with per-step checkpoints, against the plain forward window:
    the FP64 window (FP64 forward and adjoint), the mixed-precision window
    (mixed forward; its adjoint linearises the mixed step with FP32 rate
    adjoints and FP64 budgets, column stages and accumulation) and, beside it,
    the mixed forward with the FP64 adjoint."""
    import torch
    from nicam_kokkos_microphysics_gb300 import mp_init
    from nicam_kokkos_microphysics_gb300.window import window_forward, window_gradient
    spec = StateSpec(gall=16900, kall=42, lall=lall, seed=seed, variant=variant)
    st = make_state(spec, out_fill=0.0)
    x0 = {n: torch.from_numpy(st[n]).cuda() for n in ARG_NAMES}
    out = {"workload": f"{nsteps}-step window, gall={spec.gall} kall={spec.kall} lall={spec.lall}, dt={spec.dt}, "
                       f"per-step checkpoints, adjoint accumulation in FP64",
           "peak_device_bytes": "device memory in use at the window's peak beyond that before the handle was "
                                "created: the handle's workspaces, the checkpoints and the adjoint arrays"}
    for precision, adjoint, key in (("fp64", "fp64", "forward_fp64"), ("mixed", "mixed", "forward_mixed"),
                                    ("mixed", "fp64", "forward_mixed_adjoint_fp64")):
        # a handle per case, so that each peak includes the workspaces its calls allocate
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        free0 = torch.cuda.mem_get_info()[0]
        drv = mp_init("NSW6", spec.gall, spec.kall, st["_gz"], st["_gzh"], lall_max=spec.lall)
        res = window_gradient(drv, spec.lall, x0, nsteps, spec.dt, precision=precision, adjoint=adjoint,
                              free0=free0)
        peak = res["peak_bytes"]
        torch.cuda.empty_cache()
        res = window_gradient(drv, spec.lall, x0, nsteps, spec.dt, precision=precision, adjoint=adjoint)
        xs = {n: t.clone() for n, t in x0.items()}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        window_forward(drv, spec.lall, xs, nsteps, spec.dt, precision)
        torch.cuda.synchronize()
        t_plain = time.perf_counter() - t0
        out[key] = {
            "ratio": res["t_adjoint"] / t_plain, "forward_ms": t_plain * 1e3,
            "forward_with_checkpoints_ms": res["t_forward"] * 1e3, "adjoint_ms": res["t_adjoint"] * 1e3,
            "peak_device_bytes": peak, "J": res["J"]}
        drv.close()
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="NSW6 step benchmark")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--gall", type=int, default=16900)
    ap.add_argument("--kall", type=int, default=42)
    ap.add_argument("--lall", type=int, default=10)
    ap.add_argument("--variant", default="standard", choices=["standard", "convective", "cold"])
    ap.add_argument("--seed", type=int, default=1002)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="FP64 line only: no mixed-precision, adjoint or window sections")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="precision of the headline step: plain FP64, or FP32 process rates with FP64 budgets, "
                         "flux sums and Newton")
    ap.add_argument("--only", choices=["adjoint", "window"], default=None,
                    help="run one section alone and print its JSON (for profiling): the adjoint of one FP64 step "
                         "on 4096 x 42, or the checkpointed window (--window-steps steps on --lall regions)")
    ap.add_argument("--window-steps", type=int, default=12)
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.only == "adjoint":
        print(json.dumps(adjoint_ratio(args.seed, args.variant, args.steps, args.warmup)), flush=True)
        return 0
    if args.only == "window":
        print(json.dumps(window_ratio(args.seed, args.variant, args.window_steps, args.lall)), flush=True)
        return 0

    import torch
    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from nicam_kokkos_microphysics_gb300 import mp_init

    # this rank's block of the job's world * lall regions
    job = StateSpec(gall=args.gall, kall=args.kall, lall=args.lall * world, seed=args.seed, variant=args.variant)
    st = make_state(job, out_fill=0.0, regions=shard_regions(job.lall, rank, world))
    spec = StateSpec(gall=args.gall, kall=args.kall, lall=args.lall, seed=args.seed, variant=args.variant)
    st0 = {k: v.copy() for k, v in st.items()}
    drv = mp_init("NSW6", spec.gall, spec.kall, st["_gz"], st["_gzh"], lall_max=spec.lall)
    drv.set_sync_check(False)

    def device_run(precision: str, with_clocks: bool):
        drv.set_precision(precision)
        dev = {n: torch.from_numpy(st0[n]).cuda() for n in ARG_NAMES}
        for _ in range(args.warmup):
            drv.mp_driver_batched(spec.lall, *[dev[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
        rc, cell = drv.last_error()
        if rc != 0:
            raise RuntimeError(f"warm-up step failed with status {rc} at {cell}")
        sampler = ClockSampler(local) if with_clocks else None
        if sampler:
            sampler.start()
            time.sleep(0.3)
        ms, cell_ms, col_ms = time_device_steps(drv, spec.lall, dev, spec.dt, args.steps, dist)
        clocks = sampler.stop() if sampler else None
        del dev
        return max_over_ranks(ms, dist), {"nsw6_cell_kernel": cell_ms, "nsw6_column_kernel": col_ms}, clocks

    ms, kernel_ms, clocks = device_run(args.precision, True)
    value = whole_job_rate(spec.cells, world, ms * 1e-3)
    e2e = None if args.no_e2e else time_end_to_end(drv, spec, st0, args.steps, world, dist)

    rates = fp64_rates() if rank == 0 else None
    aw = algorithmic_work(spec, st0, OP_WEIGHTS) if rank == 0 else None
    roofline = roofline_of(kernel_ms, spec, args.precision, rates, aw)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, kind, threads, times = cpu_reference_sample(spec, 3)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"3 steps x 1 region of {spec.gall}x{spec.kall} cells (median), OpenMP"}

    mixed = args.precision == "mixed"
    line = {
        "metric": METRIC_MIXED if mixed else METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64", "data": "synthetic (seeded NICAM-like state)",
        "config": workload_config(spec, args.precision, world),
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
        "gpu_launches": 3 * args.steps,   # per step: nsw6_cell_kernel, nsw6_column_kernel, nsw6_satadj_kernel
    }

    if not args.no_extras and world == 1:
        # the other parts of the metric, each outside the headline's timed region
        other = "fp64" if mixed else "mixed"
        ms2, kernel_ms2, _ = device_run(other, False)
        sec = {"value": whole_job_rate(spec.cells, world, ms2 * 1e-3), "unit": UNIT, "ms_per_step": ms2,
               "mixed_speedup_over_fp64": (ms / ms2) if other == "mixed" else (ms2 / ms), "kernel_ms": kernel_ms2,
               "roofline": roofline_of(kernel_ms2, spec, other, rates, None)}
        if not args.no_e2e:
            drv.set_precision(other)
            sec["e2e"] = time_end_to_end(drv, spec, st0, args.steps, world)
        sec["error_vs_fp64"] = mixed_vs_fp64(drv, spec, st0)
        line["mixed" if other == "mixed" else "fp64"] = sec
        drv.set_precision(args.precision)
        line["adjoint"] = adjoint_ratio(args.seed, args.variant, args.steps, args.warmup)
        line["window"] = window_ratio(args.seed, args.variant)
    elif mixed:
        line["mixed_error_vs_fp64"] = mixed_vs_fp64(drv, spec, st0)
    if rank == 0:
        print(json.dumps(line), flush=True)
    drv.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

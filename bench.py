#!/usr/bin/env python
"""Benchmark of one NICAM NSW6 microphysics step on GB300.

Workload (N=1): gall = 16900 (130 x 130 points), kall = 42, lall = 10 regions
(7.1 M cells), dt = 60 s, FP64, seeded synthetic states (the NICAM snapshot the
reference ships without is replaced by nicam_kokkos_microphysics_gb300.state).
A step is one mp_driver call over all regions, in place, as the reference
harness loops over SET_iteration (src/main.cpp:261-319).  The working set
(about 3 GB) is far larger than the 129 MB L2, so no flush is needed between
steps.

Metric: cells per second per NSW6 step (gall * kall * lall / step time).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

For N > 1 (torchrun, one process per GPU) every rank steps its own lall
regions (weak scaling, no collective on the data path); rank 0 prints the
line with value = all cells / max step time over ranks.
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
                                                   make_state, region_view)

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
# DRAM bytes (read + write) per interior cell of the cell kernel and per cell of
# the column kernel, from ncu captures (--set full) of each kernel on one
# 16900 x 42 region; traffic grows in proportion to cells.
CELL_KERNEL_TRAFFIC_PER_CELL = {"fp64": 215.5, "mixed": 172.9}
COLUMN_KERNEL_TRAFFIC_PER_CELL = {"fp64": 375.1, "mixed": 383.3}
# FP64-pipe activity (fraction of active cycles) of each kernel in the same
# captures: the hardware-level utilisation of the bound the kernels sit on.
FP64_PIPE_ACTIVE = {"nsw6_cell_kernel": {"fp64": 0.842, "mixed": 0.747},
                    "nsw6_column_kernel": {"fp64": 0.708, "mixed": 0.679}}
# FP64 op weights in flop equivalents (an FMA counts 2): the cost of CUDA's FP64
# divide, sqrt, exp, log and pow relative to DFMA, measured once on a GB300 with
# the throughput probe (csrc/nsw6_probe.cu) and frozen here.
ADJOINT_LAUNCHES = 12   # kernels of one mp_driver_adjoint call (hand-written sweeps)
OP_WEIGHTS = {"add": 1.0, "mul": 1.0, "cmp": 1.0, "div": 15.0, "sqrt": 15.2, "exp": 30.0, "log": 58.4,
              "pow": 173.8}


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def rank_seed(seed: int, rank: int) -> int:
    """Each rank steps its own regions (weak scaling): a distinct state seed."""
    return seed + 7919 * rank


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
    from nicam_kokkos_microphysics_gb300 import _native
    if not _native.PROBE_LIB.exists():
        return None
    lib = ctypes.CDLL(str(_native.PROBE_LIB))
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
            "column_per_cell": work("column") / n_all,
            "counts_per_interior_cell": {k: (c["cell"][k] + c["zdis"][k]) / n_int for k in c["cell"]},
            "column_counts_per_cell": {k: c["column"][k] / n_all for k in c["column"]}}


# ----------------------------------------------------------------- CPU side
def cpu_reference_sample(spec: StateSpec, steps: int, use_port: bool = False):
    """Time the reference's CPU implementation on one region per step.

    Uses the reference's own sources built with the OpenMP Kokkos shim
    (oracle/_ref) when they are available, else the OpenMP build of the C
    restatement.  Returns (cells/s, kind, threads, seconds per step list)."""
    from oracle import build_ref, restatement
    one = StateSpec(gall=spec.gall, kall=spec.kall, lall=1, seed=spec.seed, variant=spec.variant, dt=spec.dt)
    st = make_state(one, out_fill=0.0)
    reg = region_view(st, 0)
    cells = one.gall * one.kall
    times = []
    if not use_port and build_ref.sources_available():
        from oracle import ref
        lib = ref.load(one.gall, one.kall, st["_gz"], st["_gzh"], variant="omp")
        kind = "reference"
        threads = os.cpu_count()
        run = lambda: ref.mp_driver(lib, reg, one.dt)  # noqa: E731
    else:
        kind = "port"
        lib = restatement.load("omp")
        threads = lib.nsw6o_max_threads()
        run = lambda: restatement.mp_driver(reg, st["_gz"], st["_gzh"], one.dt, variant="omp")  # noqa: E731
    run()  # warm-up
    for _ in range(steps):
        t0 = time.perf_counter()
        run()
        times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    return cells / med, kind, threads, times


def run_reference_arm(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    spec = StateSpec(gall=args.gall, kall=args.kall, lall=args.lall, seed=args.seed, variant=args.variant)
    total = max(args.warmup, 0)
    v, kind, threads, times = cpu_reference_sample(spec, max(args.steps, 1) + 0 * total)
    ms = statistics.median(times) * 1e3
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded NICAM-like state)",
        "impl": "reference",
        "config": {"workload": f"NSW6 step, gall={spec.gall} kall={spec.kall}, one region per step "
                               f"(sample of lall={spec.lall})", "variant": spec.variant},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"{args.steps} steps x 1 region of {spec.gall}x{spec.kall} cells, median"},
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
    import torch
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


def run_adjoint_bench(args) -> int:
    """Adjoint / forward time of one step (mp_driver_adjoint around the state,
    seeded with the loss sum (precip)^2 + column QC), or, with --window N, of
    the window gradient of the accumulated surface precipitation (forward in
    --precision, per-step checkpoints, FP64 adjoint)."""
    import torch
    from nicam_kokkos_microphysics_gb300 import mp_init
    from nicam_kokkos_microphysics_gb300.window import window_forward, window_gradient
    gall = args.gall if args.gall != 16900 or args.window else 4096
    lall = args.lall if args.window else 1
    spec = StateSpec(gall=gall, kall=args.kall, lall=lall, seed=args.seed, variant=args.variant)
    st = make_state(spec, out_fill=0.0)
    drv = mp_init("NSW6", spec.gall, spec.kall, st["_gz"], st["_gzh"], lall_max=spec.lall)
    x0 = {n: torch.from_numpy(st[n]).cuda() for n in ARG_NAMES}
    sampler = ClockSampler(0)
    line = {"n_gpus": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded NICAM-like state)", "unit": "ratio", "gpu_launches": None}
    if args.window:
        for _ in range(max(1, args.warmup // 3)):
            window_gradient(drv, spec.lall, x0, 2, spec.dt, precision=args.precision)
        torch.cuda.reset_peak_memory_stats()
        sampler.start()
        res = window_gradient(drv, spec.lall, x0, args.window, spec.dt, precision=args.precision)
        clocks = sampler.stop()
        # forward alone, without checkpoints, for the ratio
        xs = {n: t.clone() for n, t in x0.items()}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        window_forward(drv, spec.lall, xs, args.window, spec.dt, args.precision)
        torch.cuda.synchronize()
        t_plain = time.perf_counter() - t0
        line.update({
            "metric": "adjoint/forward time ratio, window gradient of accumulated surface precipitation",
            "value": res["t_adjoint"] / t_plain, "steps": args.window, "warmup": args.warmup,
            "ms_per_step": res["t_adjoint"] * 1e3 / args.window,
            "config": {"workload": f"{args.window}-step window, gall={spec.gall} kall={spec.kall} lall={spec.lall}, "
                                   f"dt={spec.dt}, forward {args.precision}, FP64 adjoint, per-step checkpoints",
                       "variant": spec.variant},
            "forward_ms": t_plain * 1e3, "forward_with_checkpoints_ms": res["t_forward"] * 1e3,
            "adjoint_ms": res["t_adjoint"] * 1e3, "peak_device_bytes": res["peak_bytes"],
            "J": res["J"], "dJ_dparams": res["dparams"].tolist(), "clocks": clocks,
            "gpu_launches": args.window * 2 + args.window * ADJOINT_LAUNCHES,
        })
    else:
        dev = {n: t.clone() for n, t in x0.items()}
        kinds = {n: k for n, k, _ in MP_DRIVER_ARGS}
        for _ in range(args.warmup):
            y = {n: t.clone() for n, t in x0.items()}
            drv.mp_driver_batched(spec.lall, *[y[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
        y = {n: t.clone() for n, t in x0.items()}
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            drv.mp_driver_batched(spec.lall, *[y[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
        e1.record()
        torch.cuda.synchronize()
        t_fwd = e0.elapsed_time(e1) / args.steps
        bar = {n: torch.zeros(batched_shape(kinds[n], spec.lall, spec.kall, spec.gall), dtype=torch.float64,
                              device="cuda") for n in ARG_NAMES}
        drv.adjoint(spec.lall, dev, {n: b.clone() for n, b in bar.items()}, dt=spec.dt)   # warm-up, tape sizing
        torch.cuda.reset_peak_memory_stats()
        # the output adjoints of every timed step, prepared beforehand (the
        # call overwrites them with the input adjoints)
        seeds = []
        for _ in range(args.steps):
            b = {n: t.clone() for n, t in bar.items()}
            b["precip"].fill_(1.0)
            b["rhogq"][:, 1] = 1.0
            seeds.append(b)
        sampler.start()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for b in seeds:
            drv.adjoint(spec.lall, dev, b, dt=spec.dt)
        torch.cuda.synchronize()
        t_adj = (time.perf_counter() - t0) / args.steps * 1e3
        clocks = sampler.stop()
        line.update({
            "metric": "adjoint/forward time ratio of one NSW6 step", "value": t_adj / t_fwd, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_adj,
            "config": {"workload": f"adjoint of one FP64 step, gall={spec.gall} kall={spec.kall} lall={spec.lall}, "
                                   f"dt={spec.dt}", "variant": spec.variant},
            "forward_ms": t_fwd, "adjoint_ms": t_adj, "clocks": clocks,
            # per call: the cell phase's forward, 3 forward stages, the flux
            # bounds, 2 seed kernels, 4 adjoint stages and the cell adjoint
            "gpu_launches": ADJOINT_LAUNCHES * args.steps,
        })
    print(json.dumps(line), flush=True)
    drv.close()
    return 0


# ----------------------------------------------------------------- GPU side
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
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="plain FP64 step, or FP32 process rates with FP64 budgets, flux sums and Newton")
    ap.add_argument("--adjoint", action="store_true",
                    help="time the adjoint step against the forward step (default workload 4096 x 42, one region)")
    ap.add_argument("--window", type=int, default=0,
                    help="with --adjoint: gradient over a window of this many steps with per-step checkpoints")
    args = ap.parse_args(argv)
    if args.adjoint:
        return run_adjoint_bench(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)

    import torch
    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from nicam_kokkos_microphysics_gb300 import mp_init

    spec = StateSpec(gall=args.gall, kall=args.kall, lall=args.lall, seed=rank_seed(args.seed, rank),
                     variant=args.variant)
    st = make_state(spec, out_fill=0.0)
    st0 = {k: v.copy() for k, v in st.items()}
    drv = mp_init("NSW6", spec.gall, spec.kall, st["_gz"], st["_gzh"], lall_max=spec.lall)
    drv.set_precision(args.precision)
    dev = {n: torch.from_numpy(st[n]).cuda() for n in ARG_NAMES}
    args_dev = [dev[n] for n in ARG_NAMES]
    drv.set_sync_check(False)

    def step():
        drv.mp_driver_batched(spec.lall, *args_dev, dt=spec.dt, ct=0.0)

    for _ in range(args.warmup):
        step()
    rc, cell = drv.last_error()
    if rc != 0:
        raise RuntimeError(f"warm-up step failed with status {rc} at {cell}")

    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    drv.set_timing(True)
    drv.read_timing()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    t_cell, t_col, nsteps = drv.read_timing()
    drv.set_timing(False)
    rc, cell = drv.last_error()
    if rc != 0:
        raise RuntimeError(f"timed steps failed with status {rc} at {cell}")
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dist)
    cells_rank = spec.cells
    value = whole_job_rate(cells_rank, world, ms * 1e-3)

    # ---- end to end through the public API with host (pinned) buffers
    e2e = None
    if not args.no_e2e:
        host = {}
        for n in ARG_NAMES:
            t = torch.empty(st[n].shape, dtype=torch.float64, pin_memory=True)
            t.numpy()[...] = st[n]
            host[n] = t.numpy()
        from nicam_kokkos_microphysics_gb300._native import load as _load  # noqa: F401
        import ctypes
        kinds = {n: k for n, k, _ in MP_DRIVER_ARGS}
        read_args = ["rhog", "rhogvx", "rhogvy", "rhogvz", "rhogw", "rhoge", "rhogq", "vx", "vy", "vz", "tem", "q",
                     "gsgam2", "gsgam2h", "gam2", "gam2h", "ix", "iy", "iz", "jx", "jy", "jz", "z"]
        write_args = ["rhog", "rhogvx", "rhogvy", "rhogvz", "rhogw", "rhoge", "rhogq", "rho", "tem", "pre", "q", "qd",
                      "precip", "ISO1_precip", "ISO2_precip", "precip_rhoe", "precip_lh_heat", "precip_rhophi",
                      "precip_rhokin", "re_liquid", "re_solid", "re_cld", "rctop", "rwtop", "tctop", "GDCLW",
                      "GDCFRC", "GPREC"]
        nbytes = lambda n: int(np.prod(batched_shape(kinds[n], spec.lall, spec.kall, spec.gall))) * 8  # noqa: E731
        h2d = sum(nbytes(n) for n in read_args)
        d2h = sum(nbytes(n) for n in write_args)
        drv.run(host, dt=spec.dt)  # warm-up (allocates the staging buffers)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            drv.run(host, dt=spec.dt)
        dt_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps, dist)
        e2e = {"value": whole_job_rate(cells_rank, world, dt_e2e), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": dt_e2e * 1e3}

    # ---- mixed precision: error of one step against the FP64 path on the same state
    mixed_error = None
    if args.precision == "mixed":
        mixed_error = mixed_vs_fp64(drv, spec, st0)

    # ---- roofline of the dominant kernel
    peaks, src = measured_peaks()
    n_int = spec.gall * (spec.kall - 2) * spec.lall
    cell_ms = t_cell / max(nsteps, 1)
    col_ms = t_col / max(nsteps, 1)
    rates = fp64_rates()
    hbm_cell = CELL_KERNEL_BYTES_PER_CELL * n_int / (cell_ms * 1e-3) / 1e9
    hbm = {"cell_kernel_gbs": hbm_cell, "cell_kernel_frac": hbm_cell / peaks["hbm_gbs"], "peak": peaks["hbm_gbs"],
           "unit": "GB/s", "peak_source": f"{src} copy bandwidth"}
    roofline = {"cell_kernel_ms": cell_ms, "column_kernel_ms": col_ms, "hbm": hbm}
    if rates:
        aw = algorithmic_work(spec, st0, OP_WEIGHTS)
        cell_flops = aw["cell_per_interior_cell"] * n_int
        col_flops = aw["column_per_cell"] * spec.cells
        cell = {"achieved": cell_flops / (cell_ms * 1e-3) / 1e12, "work_per_interior_cell": aw["cell_per_interior_cell"],
                "traffic": CELL_KERNEL_TRAFFIC_PER_CELL[args.precision] * n_int}
        col = {"achieved": col_flops / (col_ms * 1e-3) / 1e12, "work_per_cell": aw["column_per_cell"],
               "traffic": COLUMN_KERNEL_TRAFFIC_PER_CELL[args.precision] * spec.cells}
        for d in (cell, col):
            d["frac"] = d["achieved"] / rates["peak_tflops"]
        top, other, names = (cell, col, ("nsw6_cell_kernel", "nsw6_column_kernel")) if cell_ms >= col_ms else \
            (col, cell, ("nsw6_column_kernel", "nsw6_cell_kernel"))
        roofline.update({
            "kernel": names[0], "bound": "fp64", "achieved": top["achieved"], "peak": rates["peak_tflops"],
            "unit": "TFLOP/s", "frac": top["frac"], "traffic": top["traffic"],
            "peak_source": "measured in this run: FP64 FMA throughput probe (MEASURED_PEAKS.json has no FP64 peak)",
            "work_definition": "FP64 operations of the reference algorithm counted on this state (integer powers "
                               "as products), weighted add/mul/cmp 1, FMA 2, div/sqrt/exp/log/pow by their frozen "
                               "measured cost",
            "op_weights": OP_WEIGHTS,
            "op_weights_this_run": rates["weights"],
            "fp64_pipe_active_ncu": FP64_PIPE_ACTIVE[names[0]][args.precision],
            "frac_note": "achieved counts the reference algorithm's FP64 work, so frac > 1 means the kernel does "
                         "that work in less time than the FP64 pipe needs for it as written; the hardware "
                         "utilisation is fp64_pipe_active_ncu",
            names[1]: other,
        })
        roofline.update({"work_per_unit": top.get("work_per_interior_cell", top.get("work_per_cell"))})
    else:
        roofline.update({"kernel": "nsw6_cell_kernel", "bound": "hbm", "achieved": hbm_cell,
                         "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": hbm_cell / peaks["hbm_gbs"],
                         "traffic": None})

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
        "config": {"workload": f"NSW6 {'mixed-precision' if mixed else 'FP64'} step, gall={spec.gall} "
                               f"kall={spec.kall} lall={spec.lall} per GPU ({spec.cells} cells), dt={spec.dt}",
                   "variant": spec.variant, "precision": args.precision,
                   "l2": "working set >> L2 (no flush needed)", "parallelism": f"regions x{world}"},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
        "gpu_launches": 2 * args.steps,
    }
    if mixed_error is not None:
        line["mixed_error_vs_fp64"] = mixed_error
    if rank == 0:
        print(json.dumps(line), flush=True)
    drv.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Adjoint of a multi-step window of NSW6 steps with per-step checkpoints.

The forward pass runs ``nsteps`` steps (FP64 or the mixed-precision step) and
keeps, before every step, a copy of the fields the step changes (the
checkpoint); the fields it only reads are shared by all steps.  The backward
pass walks the window in reverse: for step n it recomputes the step from its
checkpoint inside ``mp_driver_adjoint`` and sweeps it back, so device memory
holds nsteps checkpoints and one step's work arrays, not nsteps tapes.  With
the mixed-precision forward the backward linearises the same step: its cell
physics with FP32 rates and FP32 rate adjoints, FP64 budgets, column stages
and accumulation of the state and parameter adjoints (``adjoint="fp64"``
linearises the FP64 step around the mixed trajectory's states instead).

The adjoint convention of mp_driver_adjoint makes the chaining direct: on
return the adjoint arrays of the fields a step both reads and writes hold the
adjoint of the previous step's outputs, the adjoints of read-only fields
accumulate over the window, and the write-only outputs are zero, ready for the
next seed.

The objective is the window-accumulated surface precipitation
J = sum_n sum_{l,g} (precip_rain + precip_solid)_n * dt.
"""
from __future__ import annotations

import time

import numpy as np

from .state import ARG_NAMES, MP_DRIVER_ARGS, batched_shape

# Fields a step changes and the next step reads (checkpointed); precip and the
# other write-only diagnostics are regenerated by every step.
EVOLVING = ["rhog", "rhogvx", "rhogvy", "rhogvz", "rhogw", "rhoge", "rhogq", "rho", "tem", "pre", "q"]


def window_forward(drv, lall: int, state: dict, nsteps: int, dt: float, precision: str = "fp64",
                   checkpoints: list | None = None) -> float:
    """Runs the window in place on ``state`` (CUDA tensors keyed by ARG_NAMES);
    appends the checkpoint of each step to ``checkpoints``; returns J."""
    import torch
    drv.set_precision(precision)
    J = torch.zeros((), dtype=torch.float64, device="cuda")
    for _ in range(nsteps):
        if checkpoints is not None:
            checkpoints.append({n: state[n].clone() for n in EVOLVING})
        drv.mp_driver_batched(lall, *[state[n] for n in ARG_NAMES], dt=dt, ct=0.0)
        J += (state["precip"][0] + state["precip"][1]).sum() * dt
    drv.set_precision("fp64")
    return float(J)


def window_gradient(drv, lall: int, state0: dict, nsteps: int, dt: float, precision: str = "fp64",
                    adjoint: str | None = None, free0: int | None = None) -> dict:
    """Gradient of J over the window with respect to the initial state and the
    seven parameters; ``adjoint`` is the precision of the step the backward
    linearises (default: that of the forward).  Returns {"J", "grad"
    (adjoints keyed by ARG_NAMES), "dparams" (7), "t_forward", "t_adjoint",
    "peak_bytes" (the most device memory in use beyond ``free0``, the free
    device memory to measure from; default: that at the call)}."""
    import torch
    kinds = {n: k for n, k, _ in MP_DRIVER_ARGS}
    if free0 is None:
        free0 = torch.cuda.mem_get_info()[0]
    peak = 0

    def track():
        nonlocal peak
        peak = max(peak, free0 - torch.cuda.mem_get_info()[0])

    st = {n: state0[n].clone() for n in ARG_NAMES}
    ckpt: list = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J = window_forward(drv, lall, st, nsteps, dt, precision, ckpt)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    track()

    bar = {n: torch.zeros(batched_shape(kinds[n], lall, drv.kall, drv.gall), dtype=torch.float64, device="cuda")
           for n in ARG_NAMES}
    dparams = np.zeros(7)
    x = {n: state0[n].clone() for n in ARG_NAMES}
    drv.set_precision(adjoint or precision)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for n in reversed(range(nsteps)):
        for f in EVOLVING:
            x[f].copy_(ckpt[n][f])
        bar["precip"] += dt       # dJ / dprecip of step n
        dparams += drv.adjoint(lall, x, bar, dt=dt)
        track()
    torch.cuda.synchronize()
    t_adj = time.perf_counter() - t0
    drv.set_precision("fp64")
    track()
    return {"J": J, "grad": bar, "dparams": dparams, "t_forward": t_fwd, "t_adjoint": t_adj, "peak_bytes": peak}

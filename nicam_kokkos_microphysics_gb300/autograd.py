"""torch.autograd wrapper of one NSW6 step, for checking the hand-built
derivative kernels with PyTorch's tooling (not a compute path: forward and
backward both call the C ABI of include/nsw6.h).

``NSW6Step.apply(drv, lall, dt, params, *inputs)`` takes the step's read
arguments (READ_NAMES, float64 CUDA tensors in the all-regions layout) and a
tensor of the 7 parameters, and returns the step's written arguments
(WRITE_NAMES).  The backward runs mp_driver_adjoint.  The parameter values
must equal the driver's (``drv.set_params``); only their gradient flows.
"""
from __future__ import annotations

import torch

from .state import ARG_NAMES, MP_DRIVER_ARGS, batched_shape

READ_NAMES = ["rhog", "rhogvx", "rhogvy", "rhogvz", "rhogw", "rhoge", "rhogq", "vx", "vy", "vz", "tem", "q",
              "gsgam2", "gsgam2h", "gam2", "gam2h", "ix", "iy", "iz", "jx", "jy", "jz", "z"]
WRITE_NAMES = ["rhog", "rhogvx", "rhogvy", "rhogvz", "rhogw", "rhoge", "rhogq", "rho", "tem", "pre", "q", "qd",
               "precip", "ISO1_precip", "ISO2_precip", "precip_rhoe", "precip_lh_heat", "precip_rhophi",
               "precip_rhokin", "re_liquid", "re_solid", "re_cld", "rctop", "rwtop", "tctop", "GDCLW", "GDCFRC",
               "GPREC"]


def _full_state(drv, lall, given: dict) -> dict:
    kinds = {n: k for n, k, _ in MP_DRIVER_ARGS}
    out = {}
    for n in ARG_NAMES:
        if n in given:
            out[n] = given[n].detach().clone().contiguous()
        else:
            out[n] = torch.zeros(batched_shape(kinds[n], lall, drv.kall, drv.gall), dtype=torch.float64, device="cuda")
    return out


class NSW6Step(torch.autograd.Function):
    @staticmethod
    def forward(ctx, drv, lall, dt, params, *inputs):
        x = dict(zip(READ_NAMES, inputs))
        ctx.drv, ctx.lall, ctx.dt = drv, lall, dt
        ctx.save_for_backward(*inputs)
        st = _full_state(drv, lall, x)
        drv.mp_driver_batched(lall, *[st[n] for n in ARG_NAMES], dt=dt, ct=0.0)
        return tuple(st[n] for n in WRITE_NAMES)

    @staticmethod
    def backward(ctx, *grads):
        drv, lall, dt = ctx.drv, ctx.lall, ctx.dt
        x = _full_state(drv, lall, dict(zip(READ_NAMES, ctx.saved_tensors)))
        bar = _full_state(drv, lall, {})
        for n, g in zip(WRITE_NAMES, grads):
            if g is not None:
                bar[n].copy_(g)
        pbar = drv.adjoint(lall, x, bar, dt=dt)
        gin = tuple(bar[n] for n in READ_NAMES)
        return (None, None, None, torch.as_tensor(pbar, dtype=torch.float64, device="cuda"), *gin)

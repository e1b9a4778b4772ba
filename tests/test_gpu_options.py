"""GPU parity of the scheme switches against the reference built with them.

Each fixture (tests/golden/options_*.npz, made by tests/golden/make_golden.py
with the "opt" build of the reference, oracle/build_ref.py) holds the inputs
and outputs of the reference's mp_driver with one or more of the NSW6
switches flipped from the reference configuration: the classic snow moments
with the Bergeron process and the mixed-phase saturation adjustment
(Roh_flag = false), Berry autoconversion, QI sedimentation ("4WATER"),
KIN2KIN and the aerosol indirect effect.  Pass criterion as in
test_gpu_parity (tests/_parity.py).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import options_files
from nicam_kokkos_microphysics_gb300.state import ARG_NAMES, MP_DRIVER_ARGS, OUTPUT_NAMES, batched_shape, region_shape
from _parity import compare, passes, summary

pytestmark = pytest.mark.gpu

OPTION_NAMES = ["roh2014", "explicit_icegen", "kk2000", "qi_sediment", "kin2kin", "aerosol_indirect"]


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def load_fixture(path):
    z = np.load(path)
    kall, gall = z["in_rhog"].shape
    reg = {}
    for name, kind, _ in MP_DRIVER_ARGS:
        key = f"in_{name}"
        reg[name] = z[key].copy() if key in z else np.full(region_shape(kind, kall, gall), np.nan)
    out = {n: z[f"out_{n}"] for n in OUTPUT_NAMES}
    opts = {n: int(v) for n, v in zip(OPTION_NAMES, z["options"])}
    return reg, out, z["gz"], z["gzh"], float(z["dt"]), opts


def run_gpu(reg, gz, gzh, dt, options):
    torch = _torch()
    from nicam_kokkos_microphysics_gb300 import mp_init
    kall, gall = reg["rhog"].shape
    drv = mp_init("NSW6", gall, kall, gz, gzh, options=options)
    assert drv.get_options() == {**options, "explicit_icegen": int(options["roh2014"] or options["explicit_icegen"])}
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in reg.items()}
    drv.mp_driver(0, *[t[n] for n in ARG_NAMES], dt=dt, ct=0.0)
    torch.cuda.synchronize()
    out = {k: v.cpu().numpy() for k, v in t.items()}
    drv.close()
    return out


@pytest.mark.parametrize("path", options_files(), ids=lambda p: p.stem)
def test_gpu_options_match_reference(path):
    reg, want, gz, gzh, dt, opts = load_fixture(path)
    got = run_gpu(reg, gz, gzh, dt, opts)
    stats = compare(got, want, OUTPUT_NAMES)
    print(f"\n[{path.stem}] {opts}\n" + summary(stats))
    bad = sorted(n for n, s in stats.items() if s["n_bad"])
    assert passes(stats), f"{path.stem}: fields outside tolerance: {bad}\n" + summary(stats)


def test_gpu_options_change_the_result():
    """The switched kernels are the ones that ran: every fixture's output
    differs from the reference configuration's on the same input somewhere."""
    torch = _torch()
    for path in options_files():
        reg, want, gz, gzh, dt, opts = load_fixture(path)
        got = run_gpu(reg, gz, gzh, dt, dict(zip(OPTION_NAMES, [1, 1, 1, 0, 0, 0])))
        assert any(not np.array_equal(got[n], want[n], equal_nan=True) for n in OUTPUT_NAMES), path.stem
    del torch


def test_gpu_options_reject_unsupported_paths():
    torch = _torch()
    from nicam_kokkos_microphysics_gb300 import NSW6Error, mp_init
    path = options_files()[0]
    reg, want, gz, gzh, dt, opts = load_fixture(path)
    kall, gall = reg["rhog"].shape
    drv = mp_init("NSW6", gall, kall, gz, gzh, options=opts)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in reg.items()}
    # the CUDA-libm kernels and the serial (derivative-path) step take no switches
    drv.set_math(1)
    with pytest.raises(NSW6Error) as e:
        drv.mp_driver(0, *[t[n] for n in ARG_NAMES], dt=dt, ct=0.0)
    assert e.value.code == 5
    drv.set_math(0)
    drv.set_precision("serial")
    with pytest.raises(NSW6Error) as e:
        drv.mp_driver(0, *[t[n] for n in ARG_NAMES], dt=dt, ct=0.0)
    assert e.value.code == 5
    drv.set_precision("fp64")
    # the serial tangent-linear step (adjoint mode "tape": one column per
    # thread) takes no switch; the staged derivative steps take them all
    kinds = {n: k for n, k, _ in MP_DRIVER_ARGS}
    tb = {n: v.reshape(batched_shape(kinds[n], 1, kall, gall)) for n, v in t.items()}   # one region
    bar = {n: torch.zeros_like(v) for n, v in tb.items()}
    drv.set_options(qi_sediment=1)
    drv.set_adjoint_mode("tape")
    with pytest.raises(NSW6Error) as e:
        drv.tlm(1, tb, bar, dt=dt)
    assert e.value.code == 5
    drv.set_adjoint_mode("hand")
    with pytest.raises(KeyError):
        drv.set_options(no_such_switch=1)
    with pytest.raises(NSW6Error):
        drv.set_options(kin2kin=2)
    drv.close()

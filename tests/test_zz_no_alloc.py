"""mp_driver_noalloc: the entry point that allocates nothing (fixed scratch
inside the library) against the handle-based mp_driver, on two steps in a
row of one full 130 x 130 region.  Collected last on purpose: it must also
pass after every other test has used the library in the same process."""
from __future__ import annotations

import numpy as np
import pytest

from nicam_kokkos_microphysics_gb300.state import ARG_NAMES, OUTPUT_NAMES, StateSpec, make_state, region_view
from _parity import compare, passes, summary

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_noalloc_matches_mp_driver_two_steps():
    torch = _torch()
    from nicam_kokkos_microphysics_gb300 import mp_driver_noalloc, mp_init
    spec = StateSpec(gall=16900, kall=42, lall=1, seed=1002, variant="convective")
    st = make_state(spec, out_fill=0.0)
    reg = region_view(st, 0)
    a = {n: torch.from_numpy(np.ascontiguousarray(reg[n])).cuda() for n in ARG_NAMES}
    b = {n: t.clone() for n, t in a.items()}
    drv = mp_init("NSW6", spec.gall, spec.kall, st["_gz"], st["_gzh"])
    try:
        for step in range(2):
            drv.mp_driver(0, *[a[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
            mp_driver_noalloc(spec.gall, spec.kall, st["_gz"], st["_gzh"], *[b[n] for n in ARG_NAMES],
                              dt=spec.dt, ct=0.0)
            torch.cuda.synchronize()
            want = {n: a[n].cpu().numpy() for n in OUTPUT_NAMES}
            got = {n: b[n].cpu().numpy() for n in OUTPUT_NAMES}
            stats = compare(got, want, OUTPUT_NAMES)
            print(f"\n[noalloc step {step}]\n" + summary(stats))
            assert passes(stats), f"step {step}\n" + summary(stats)
    finally:
        drv.close()


def test_noalloc_rejects_oversized_region():
    torch = _torch()
    from nicam_kokkos_microphysics_gb300 import NSW6Error, mp_driver_noalloc
    from nicam_kokkos_microphysics_gb300.state import vertical_grid
    gz, gzh = vertical_grid(42)
    gall = 2097152 // 42 + 1     # one column more than the scratch holds
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    from nicam_kokkos_microphysics_gb300 import _native
    import ctypes
    lib = _native.load()
    ptrs = (ctypes.c_void_p * len(ARG_NAMES))(*([dummy.data_ptr()] * len(ARG_NAMES)))
    rc = lib.mp_driver_noalloc(gall, 42, np.ascontiguousarray(gz).ctypes.data, np.ascontiguousarray(gzh).ctypes.data,
                               None, ptrs, 60.0, 0.0, None)
    assert rc == 6, rc
    assert b"too large" in lib.nsw6_strerror(rc)
    rc = lib.mp_driver_noalloc(16, 161, np.zeros(161).ctypes.data, np.zeros(161).ctypes.data, None, ptrs, 60.0, 0.0,
                               None)
    assert rc == 6, rc

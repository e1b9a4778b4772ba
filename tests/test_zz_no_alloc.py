"""mp_driver_noalloc: the entry point that allocates nothing (fixed scratch
inside the library) against the handle-based mp_driver.  Both run the same
kernels on the same inputs, so their outputs must be equal bit for bit: on
two steps in a row of one full 130 x 130 region, and on the largest region
the scratch takes.  Collected last on purpose: it must also pass after every
other test has used the library in the same process."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from nicam_kokkos_microphysics_gb300.state import ARG_NAMES, OUTPUT_NAMES, StateSpec, make_state, region_view
from _parity import compare, passes, summary

pytestmark = pytest.mark.gpu

MAX_CELLS = 2097152   # NSW6_NOALLOC_MAX_CELLS of include/nsw6.h


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _run_both(torch, spec, steps, check_oracle=False):
    """`steps` steps of mp_driver (handle) and of mp_driver_noalloc from the
    same state; asserts bitwise equality after every step."""
    from nicam_kokkos_microphysics_gb300 import mp_driver_noalloc, mp_init
    st = make_state(spec, out_fill=0.0)
    reg = region_view(st, 0)
    a = {n: torch.from_numpy(np.ascontiguousarray(reg[n])).cuda() for n in ARG_NAMES}
    b = {n: t.clone() for n, t in a.items()}
    drv = mp_init("NSW6", spec.gall, spec.kall, st["_gz"], st["_gzh"])
    free = []
    try:
        for step in range(steps):
            drv.mp_driver(0, *[a[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
            torch.cuda.synchronize()
            free.append(torch.cuda.mem_get_info()[0])
            mp_driver_noalloc(spec.gall, spec.kall, st["_gz"], st["_gzh"], *[b[n] for n in ARG_NAMES],
                              dt=spec.dt, ct=0.0)
            torch.cuda.synchronize()
            free.append(torch.cuda.mem_get_info()[0])
            for n in OUTPUT_NAMES:
                assert torch.equal(a[n], b[n]), (step, n)
            if check_oracle and step == 0:
                from oracle import restatement
                want = {k: v.copy() for k, v in reg.items()}
                rc, status = restatement.mp_driver(want, st["_gz"], st["_gzh"], spec.dt)
                assert rc == 0, status
                got = {n: b[n].cpu().numpy() for n in OUTPUT_NAMES}
                stats = compare(got, want, OUTPUT_NAMES)
                print(f"\n[noalloc against the oracle, {spec.gall}x{spec.kall}]\n" + summary(stats))
                assert passes(stats), summary(stats)
    finally:
        drv.close()
    return free


def test_noalloc_matches_mp_driver_two_steps():
    torch = _torch()
    spec = StateSpec(gall=16900, kall=42, lall=1, seed=1002, variant="convective")
    free = _run_both(torch, spec, 2, check_oracle=True)
    # the second call, the library's code long loaded, allocates no device memory
    assert free[3] == free[2], free


def test_noalloc_largest_region_matches_mp_driver():
    """gall x kall at the scratch's limit (49932 x 42 = 2,097,144 cells)."""
    torch = _torch()
    gall = MAX_CELLS // 42
    assert gall * 42 <= MAX_CELLS < (gall + 1) * 42
    _run_both(torch, StateSpec(gall=gall, kall=42, lall=1, seed=77, variant="standard"), 1)


def test_noalloc_rejects_oversized_region_and_capture():
    torch = _torch()
    from nicam_kokkos_microphysics_gb300 import _native
    from nicam_kokkos_microphysics_gb300.state import vertical_grid
    gz, gzh = vertical_grid(42)
    gall = MAX_CELLS // 42 + 1     # one column more than the scratch holds
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    lib = _native.load()
    ptrs = (ctypes.c_void_p * len(ARG_NAMES))(*([dummy.data_ptr()] * len(ARG_NAMES)))
    rc = lib.mp_driver_noalloc(gall, 42, np.ascontiguousarray(gz).ctypes.data, np.ascontiguousarray(gzh).ctypes.data,
                               None, ptrs, 60.0, 0.0, None)
    assert rc == 6, rc
    assert b"too large" in lib.nsw6_strerror(rc)
    rc = lib.mp_driver_noalloc(16, 161, np.zeros(161).ctypes.data, np.zeros(161).ctypes.data, None, ptrs, 60.0, 0.0,
                               None)
    assert rc == 6, rc
    # on a stream being captured: refused before anything is issued (the
    # capture stays valid and is ended normally)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        g.capture_begin()
        rc = lib.mp_driver_noalloc(16, 42, np.ascontiguousarray(gz).ctypes.data,
                                   np.ascontiguousarray(gzh).ctypes.data, None, ptrs, 60.0, 0.0,
                                   ctypes.c_void_p(s.cuda_stream))
        dummy.add_(1.0)
        g.capture_end()
    assert rc == 5, rc

"""The per-region drop-in called from C++ as the reference harness calls it:
tests/native/mp_driver_region.cpp, built with g++ against include/nsw6.h and
the library, steps region l = 1 of three in place on the all-regions device
arrays, passing each argument as the data pointer of its region subview and
the precipitation arrays as the strided subviews (ALL, l, 0, ALL) of
[2][lall][1][gall] arrays (src/main.cpp:37, 220-222).  Region 1 must equal
mp_driver_batched over all three regions bit for bit and match the oracle;
the other regions must be left untouched."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from nicam_kokkos_microphysics_gb300.state import (ARG_NAMES, MP_DRIVER_ARGS, OUTPUT_NAMES, StateSpec, make_state,
                                                   region_view)
from _parity import compare, passes, summary

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _build(tmp: Path) -> Path:
    from nicam_kokkos_microphysics_gb300 import _native
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent
    libdir = _native.LIB.parent
    exe = tmp / "mp_driver_region"
    subprocess.run([cxx, "-O2", "-std=c++17", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}",
                    str(ROOT / "tests" / "native" / "mp_driver_region.cpp"), "-o", str(exe),
                    f"-L{libdir}", "-lnsw6_gb300", f"-Wl,-rpath,{libdir}", f"-L{cuda / 'lib64'}", "-lcudart",
                    f"-Wl,-rpath,{cuda / 'lib64'}"], check=True)
    return exe


def test_per_region_call_from_cpp_with_strided_precip(tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nicam_kokkos_microphysics_gb300 import mp_init
    exe = _build(tmp_path)
    spec = StateSpec(gall=300, kall=42, lall=3, seed=321, variant="convective")
    l = 1
    st = make_state(spec, out_fill=-7.0)   # outputs of untouched regions keep this value
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([spec.gall, spec.kall, spec.lall, l], dtype=np.int32).tofile(f)
        np.array([spec.dt]).tofile(f)
        st["_gz"].astype(np.float64).tofile(f)
        st["_gzh"].astype(np.float64).tofile(f)
        for n in ARG_NAMES:
            np.ascontiguousarray(st[n], dtype=np.float64).tofile(f)
    run = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True,
                         text=True)
    assert run.returncode == 0, run.stdout + run.stderr
    raw = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
    got, pos = {}, 0
    for n in ARG_NAMES:
        got[n] = raw[pos:pos + st[n].size].reshape(st[n].shape)
        pos += st[n].size
    assert pos == raw.size

    # all regions in one batched call
    drv = mp_init("NSW6", spec.gall, spec.kall, st["_gz"], st["_gzh"], lall_max=spec.lall)
    t = {n: torch.from_numpy(st[n].copy()).cuda() for n in ARG_NAMES}
    drv.mp_driver_batched(spec.lall, *[t[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    torch.cuda.synchronize()
    drv.close()
    kinds = {n: k for n, k, _ in MP_DRIVER_ARGS}
    for n in OUTPUT_NAMES:
        b = t[n].cpu().numpy()
        for r in range(spec.lall):
            sel = (slice(None), r) if kinds[n] == "2g" else (r,)
            if r == l:
                assert np.array_equal(got[n][sel].view(np.int64), b[sel].view(np.int64)), n
            else:
                assert np.array_equal(got[n][sel].view(np.int64), st[n][sel].view(np.int64)), (n, r)
    # region 1 against the oracle
    from oracle import restatement
    want = region_view(st, l)
    rc, status = restatement.mp_driver(want, st["_gz"], st["_gzh"], spec.dt)
    assert rc == 0, status
    mine = region_view(got, l)
    stats = compare({n: mine[n] for n in OUTPUT_NAMES}, want, OUTPUT_NAMES)
    print("\n[C++ caller, region 1 of 3, strided precip]\n" + summary(stats))
    assert passes(stats), summary(stats)

"""Build recipe of the FP64 throughput probe that bench.py runs beside the
benchmark (probe/nsw6_probe.cu -> probe/_build/libnsw6_probe.so).

The probe measures the FP64 FMA rate of the GPU it runs on (the FP64 pipe's
peak, the denominator of the benchmark's FP64 roofline) and the rates of
CUDA's FP64 divide, sqrt, exp, log and pow (the op weights of the reference
algorithm's operation count).  It is measurement tooling, not part of the
library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libnsw6_probe.so"
sys.path.insert(0, str(HERE.parent))


def build(force: bool = False) -> Path:
    from nicam_kokkos_microphysics_gb300._native import ARCH, nvcc
    src = HERE / "nsw6_probe.cu"
    if not force and LIB.exists() and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", str(src), "-o", str(tmp)],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))

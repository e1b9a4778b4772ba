"""Generate the golden NSW6 fixtures from the reference code itself.

Runs the reference's own mp_driver (src/mod_mp_driver.cpp:335-613), compiled
from its unmodified sources against the host Kokkos shim by
``oracle/build_ref.py`` (strict serial build), on seeded synthetic states and
stores inputs and outputs as compressed npz files next to this script:

    golden_<variant>_g<gall>_k<kall>_s<seed>.npz
        in_<name>   every mp_driver argument the step reads, before the call
        out_<name>  every argument the step writes, after the call
        gz, gzh, dt, seed

The reference sources are needed to run this script; the fixtures it writes
are what the tests use wherever the reference tree is not available.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from nicam_kokkos_microphysics_gb300.state import MP_DRIVER_ARGS, StateSpec, make_state, region_view  # noqa: E402
from oracle import ref  # noqa: E402

CASES = [
    # (variant, gall, kall, seed)
    ("standard", 48, 42, 11),
    ("convective", 48, 42, 12),
    ("cold", 48, 42, 13),
    ("convective", 40, 12, 14),
]


def fixture_path(variant: str, gall: int, kall: int, seed: int) -> Path:
    return HERE / f"golden_{variant}_g{gall}_k{kall}_s{seed}.npz"


def make(variant: str, gall: int, kall: int, seed: int, dt: float = 60.0) -> Path:
    spec = StateSpec(gall=gall, kall=kall, lall=1, seed=seed, variant=variant, dt=dt)
    st = make_state(spec, out_fill=0.0)
    lib = ref.load(gall, kall, st["_gz"], st["_gzh"])
    reg = region_view(st, 0)
    inputs = {f"in_{n}": reg[n].copy() for n, _, it in MP_DRIVER_ARGS if it in ("in", "inout")}
    rc = ref.mp_driver(lib, reg, dt)
    if rc != 0:
        raise RuntimeError(f"reference mp_driver returned {rc}")
    outputs = {f"out_{n}": reg[n] for n, _, it in MP_DRIVER_ARGS if it in ("out", "inout")}
    path = fixture_path(variant, gall, kall, seed)
    np.savez_compressed(path, gz=st["_gz"], gzh=st["_gzh"], dt=np.float64(dt), seed=np.int64(seed),
                        **inputs, **outputs)
    return path


def main() -> int:
    for case in CASES:
        print(make(*case))
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Generate the golden NSW6 fixtures from the reference code itself.

Runs the reference's own mp_driver (src/mod_mp_driver.cpp:335-613), compiled
from its unmodified sources against the host Kokkos shim by
``oracle/build_ref.py`` (strict serial build), on seeded synthetic states and
stores inputs and outputs as compressed npz files next to this script:

    golden_<variant>_g<gall>_k<kall>_s<seed>.npz
        in_<name>   every mp_driver argument the step reads, before the call
        out_<name>  every argument the step writes, after the call
        gz, gzh, dt, seed

    options_<name>_g<gall>_k<kall>_s<seed>.npz
        the same for the scheme switches that the reference's defaults leave
        off (non-Roh snow, Berry warm rain, 4WATER ice sedimentation, KIN2KIN,
        the aerosol indirect effect, the mixed-phase saturation adjustment),
        made with the "opt" build of the reference (oracle/build_ref.py) and
        holding the switch values in ``options`` (nsw6_options order)

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
    ("convective", 8, 160, 15),   # the deepest column the build takes (MAX_KALL)
]


# (name, state variant, seed, switches that differ from the reference defaults[, gall, kall])
OPTION_CASES = [
    ("noroh", "standard", 11, dict(roh2014=0, explicit_icegen=0)),
    ("noroh", "cold", 13, dict(roh2014=0, explicit_icegen=0)),
    ("noroh_expice", "cold", 13, dict(roh2014=0, explicit_icegen=1)),
    ("berry", "standard", 11, dict(kk2000=0)),
    ("qi_sediment", "cold", 13, dict(qi_sediment=1)),
    ("qi_sediment", "standard", 11, dict(qi_sediment=1)),
    ("kin2kin", "convective", 12, dict(kin2kin=1)),
    ("indir", "standard", 11, dict(aerosol_indirect=1)),
    ("all", "convective", 12, dict(roh2014=0, explicit_icegen=0, kk2000=0, qi_sediment=1, kin2kin=1,
                                   aerosol_indirect=1)),
    ("all", "convective", 15, dict(roh2014=0, explicit_icegen=0, kk2000=0, qi_sediment=1, kin2kin=1,
                                   aerosol_indirect=1), 8, 160),
]


def unccn_field(shape, seed: int) -> np.ndarray:
    """Cloud condensation nuclei [1/m3] for the aerosol case: 1e7 to 2e9, so
    that max(unccn * 1e-6, Nc_def) takes both branches."""
    return np.random.default_rng(1000 + seed).uniform(1.0e7, 2.0e9, shape)


def options_path(name: str, variant: str, gall: int, kall: int, seed: int) -> Path:
    return HERE / f"options_{name}_{variant}_g{gall}_k{kall}_s{seed}.npz"


def make_options(name: str, variant: str, seed: int, opts: dict, gall: int = 48, kall: int = 42,
                 dt: float = 60.0) -> Path:
    spec = StateSpec(gall=gall, kall=kall, lall=1, seed=seed, variant=variant, dt=dt)
    st = make_state(spec, out_fill=0.0)
    reg = region_view(st, 0)
    if opts.get("aerosol_indirect"):
        reg["unccn"][...] = unccn_field(reg["unccn"].shape, seed)
    lib = ref.load(gall, kall, st["_gz"], st["_gzh"], variant="opt", options=opts)
    inputs = {f"in_{n}": reg[n].copy() for n, _, it in MP_DRIVER_ARGS if it in ("in", "inout")}
    rc = ref.mp_driver(lib, reg, dt)
    if rc != 0:
        raise RuntimeError(f"reference mp_driver returned {rc}")
    outputs = {f"out_{n}": reg[n] for n, _, it in MP_DRIVER_ARGS if it in ("out", "inout")}
    o = dict(ref.DEFAULT_OPTIONS, **opts)
    path = options_path(name, variant, gall, kall, seed)
    np.savez_compressed(path, gz=st["_gz"], gzh=st["_gzh"], dt=np.float64(dt), seed=np.int64(seed),
                        options=np.array([o[n] for n in ref.OPTION_NAMES], dtype=np.int32), **inputs, **outputs)
    return path


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
    for case in OPTION_CASES:
        print(make_options(*case))
    return 0


if __name__ == "__main__":
    sys.exit(main())

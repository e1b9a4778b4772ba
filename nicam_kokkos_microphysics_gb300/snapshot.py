"""Snapshot files of the reference harness: read, write and check.

The reference's driver program reads its input state from raw FP64 files
(src/main.cpp:128-174, src/data_io.cpp), its vertical grid from
data/vgrid/GRD_gz.dat and GRD_gzh.dat (src/mod_debug.cpp:189-195), and
compares its result with ref_verify/calculated_*_DP.dat through
PROF_val_check (src/mod_debug.cpp:23-79, main.cpp:322-351).  Every file is
one C-order array with no header, in the in-memory layout of the harness,
which is the all-regions layout of this package:

    3-D fields       [lall][kall][gall]
    tracers          [lall][6][kall][gall]           (*_Lswp files)
    precipitation    [2][lall][1][gall]              (precip*_mp files)
    column fields    [lall][1][gall]                 (rhoein_precip_mp ...)
    unit vectors     [lall][gall]                    (ix ... jz)
    grid heights     [kall]

so a real NICAM snapshot with its ref_verify pair can be run and checked
with this package unchanged.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .state import MP_DRIVER_ARGS, batched_shape

# mp_driver argument -> file of the harness (src/main.cpp:128-174).  The
# harness has no file for the diagnostics it zeroes (qd, re_*, rctop, rwtop,
# tctop, GDCLW, GDCFRC), and passes q_Lswp / rhogq_Lswp as the tracers.
FILES = {
    "rhog": "rhog.dat", "rhogvx": "rhogvx.dat", "rhogvy": "rhogvy.dat", "rhogvz": "rhogvz.dat",
    "rhogw": "rhogw.dat", "rhoge": "rhoge.dat", "vx": "vx.dat", "vy": "vy.dat", "vz": "vz.dat", "w": "w.dat",
    "unccn": "unccn.dat", "rho": "rho.dat", "pre": "pre.dat", "tem": "tem.dat",
    "rhogq": "rhogq_Lswp.dat", "q": "q_Lswp.dat",
    "precip": "precip_mp.dat", "ISO1_precip": "precip1_mp.dat", "ISO2_precip": "precip2_mp.dat",
    "precip_rhoe": "rhoein_precip_mp.dat", "precip_lh_heat": "lh_precip_mp.dat",
    "precip_rhophi": "rhophi_precip_mp.dat", "precip_rhokin": "rhokin_precip_mp.dat",
    "frhoge_af": "frhoge_af.dat", "frhogqv_af": "frhogqv_af.dat", "frhoge_rad": "frhoge_rad.dat",
    "rhogqke": "qke.dat", "gsgam2": "gsgam2.dat", "gsgam2h": "gsgam2h.dat", "gam2": "gam2.dat",
    "gam2h": "gam2h.dat", "ix": "ix.dat", "iy": "iy.dat", "iz": "iz.dat", "jx": "jx.dat", "jy": "jy.dat",
    "jz": "jz.dat", "z": "z.dat", "zh": "zh.dat", "GPREC": "GPREC.dat", "CBMFX": "CBMFX.dat",
}

# ref_verify files and the fields PROF_val_check compares (main.cpp:326-351).
CHECKS = [("rhog", "rhog", None), ("rhogvx", "rhogvx", None), ("rhogvy", "rhogvy", None),
          ("rhogvz", "rhogvz", None), ("rhogw", "rhogw", None), ("rhoge", "rhoge", None),
          ("QV", "rhogq", 0), ("QC", "rhogq", 1), ("QR", "rhogq", 2), ("QI", "rhogq", 3), ("QS", "rhogq", 4),
          ("QG", "rhogq", 5)]
CHECK_FILES = {"rhog": "calculated_rhog_DP.dat", "rhogvx": "calculated_rhogvx_DP.dat",
               "rhogvy": "calculated_rhogvy_DP.dat", "rhogvz": "calculated_rhogvz_DP.dat",
               "rhoge": "calculated_rhoge_DP.dat", "rhogw": "calculated_rhogw_DP.dat",
               "QV": "calculated_QV1_DP.dat", "QC": "calculated_QC2_DP.dat", "QR": "calculated_QR3_DP.dat",
               "QI": "calculated_QI4_DP.dat", "QS": "calculated_QS5_DP.dat", "QG": "calculated_QG6_DP.dat"}

_KINDS = {n: k for n, k, _ in MP_DRIVER_ARGS}


def _read(path: Path, shape) -> np.ndarray:
    a = np.fromfile(path, dtype="<f8")
    n = int(np.prod(shape))
    if a.size < n:
        raise ValueError(f"{path}: {a.size} values, {n} expected for shape {tuple(shape)}")
    return a[:n].reshape(shape).copy()


def read_vgrid(root: str | Path, kall: int) -> tuple[np.ndarray, np.ndarray]:
    """Heights of the vertical grid: data/vgrid/GRD_gz.dat and GRD_gzh.dat."""
    root = Path(root)
    return _read(root / "data" / "vgrid" / "GRD_gz.dat", (kall,)), _read(root / "data" / "vgrid" / "GRD_gzh.dat",
                                                                        (kall,))


def write_vgrid(root: str | Path, gz: np.ndarray, gzh: np.ndarray) -> None:
    d = Path(root) / "data" / "vgrid"
    d.mkdir(parents=True, exist_ok=True)
    np.ascontiguousarray(gz, dtype="<f8").tofile(d / "GRD_gz.dat")
    np.ascontiguousarray(gzh, dtype="<f8").tofile(d / "GRD_gzh.dat")


def read_snapshot(root: str | Path, gall: int, kall: int, lall: int) -> dict[str, np.ndarray]:
    """The harness's input state, keyed by mp_driver argument name (all-regions
    layout); arguments without a file are zero-filled, as the harness
    allocates them."""
    root = Path(root) / "data"
    out = {}
    for name, kind, _ in MP_DRIVER_ARGS:
        shape = batched_shape(kind, lall, kall, gall)
        f = FILES.get(name)
        out[name] = _read(root / f, shape) if f and (root / f).exists() else np.zeros(shape)
    return out


def write_snapshot(root: str | Path, state: dict[str, np.ndarray]) -> None:
    """Writes the fields of ``state`` that the harness reads, in its files."""
    d = Path(root) / "data"
    d.mkdir(parents=True, exist_ok=True)
    for name, f in FILES.items():
        if name in state:
            np.ascontiguousarray(state[name], dtype="<f8").tofile(d / f)


def write_check_files(root: str | Path, state: dict[str, np.ndarray]) -> None:
    """Writes ref_verify/calculated_*_DP.dat from a result state."""
    d = Path(root) / "ref_verify"
    d.mkdir(parents=True, exist_ok=True)
    for label, field, nq in CHECKS:
        a = state[field] if nq is None else state[field][:, nq]
        np.ascontiguousarray(a, dtype="<f8").tofile(d / CHECK_FILES[label])


def val_check(a: np.ndarray, b: np.ndarray) -> tuple[float, float, float]:
    """PROF_val_check (mod_debug.cpp:48-79): max, min and sum of |a - b|, with
    the maximum starting from DBL_MIN and the minimum from DBL_MAX, summed in
    the order of the loops (l, k, g)."""
    err = np.abs(np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)).reshape(-1)
    emax = max(float(err.max()) if err.size else 0.0, np.finfo(np.float64).tiny)
    emin = min(float(err.min()) if err.size else np.inf, np.finfo(np.float64).max)
    s = float(np.cumsum(err)[-1]) if err.size else 0.0   # sequential, as the loop adds
    return emax, emin, s


def check_results(root: str | Path, state: dict[str, np.ndarray]) -> list[tuple[str, float, float, float]]:
    """Compares a result state with ref_verify/calculated_*_DP.dat as the
    harness does; returns (name, max, min, sum) per checked field."""
    d = Path(root) / "ref_verify"
    lall, kall, gall = np.asarray(state["rhog"]).shape
    rows = []
    for label, field, nq in CHECKS:
        a = state[field] if nq is None else state[field][:, nq]
        ref = _read(d / CHECK_FILES[label], (lall, kall, gall))
        rows.append((label, *val_check(a, ref)))
    return rows


def format_check(rows) -> str:
    """The harness's printout (main.cpp:339-350)."""
    return "\n".join(f"Checking [{n}] Max = {mx:.16e}; Min = {mn:.16e}; Sum = {s:.16e}; " for n, mx, mn, s in rows)

"""Build recipe and ctypes wrapper for the C restatement oracle (TEST INFRASTRUCTURE ONLY).

``oracle/nsw6_oracle.c`` restates the reference's NSW6 step on the CPU; it is
compiled here into ``oracle/_build/libnsw6_oracle[_omp].so``:

  strict  -O2 -ffp-contract=off, serial: the checker used by the tests.
  omp     -O3 -fopenmp: the multi-threaded CPU baseline ("port") of bench.py.

Only tests, the golden-fixture script, ``__graft_entry__.smoke`` and the
CPU-baseline leg of bench.py use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
if str(HERE.parent) not in sys.path:
    sys.path.insert(0, str(HERE.parent))

from nicam_kokkos_microphysics_gb300.state import MP_DRIVER_ARGS, region_shape  # noqa: E402

VARIANTS = {
    "strict": ["-O2", "-ffp-contract=off"],
    "omp": ["-O3", "-ffp-contract=off", "-fopenmp"],
}

PARAM_NAMES = ["beta_saut", "qicrt_saut", "Cr", "Cs", "Cg", "ice_nuc", "kk_aut"]
OP_NAMES = ["add", "mul", "div", "sqrt", "exp", "log", "pow", "cmp"]
PHASES = ["setup", "cell", "column", "zdis"]


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in PARAM_NAMES]


def lib_path(variant: str = "strict") -> Path:
    return BUILD / ("libnsw6_oracle.so" if variant == "strict" else f"libnsw6_oracle_{variant}.so")


def build(variant: str = "strict", force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    so = lib_path(variant)
    src = [HERE / "nsw6_oracle.c", HERE / "nsw6_oracle.h", Path(__file__)]
    if so.exists() and not force and all(so.stat().st_mtime >= s.stat().st_mtime for s in src):
        return so
    cmd = ["gcc", "-std=c11", "-fPIC", "-shared", "-Wall", "-Wno-unused-variable",
           *VARIANTS[variant], str(HERE / "nsw6_oracle.c"), "-o", str(so), "-lm"]
    subprocess.run(cmd, check=True)
    return so


def build_opcount(force: bool = False) -> Path:
    """Operation-counting build (oracle/opcount.cpp)."""
    BUILD.mkdir(parents=True, exist_ok=True)
    so = BUILD / "libnsw6_opcount.so"
    src = [HERE / "opcount.cpp", HERE / "nsw6_oracle.c", HERE / "nsw6_oracle.h"]
    if so.exists() and not force and all(so.stat().st_mtime >= s.stat().st_mtime for s in src):
        return so
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-w", f"-I{HERE}", str(HERE / "opcount.cpp"),
                    "-o", str(so)], check=True)
    return so


def count_ops(reg: dict[str, np.ndarray], gz: np.ndarray, gzh: np.ndarray, dt: float) -> dict:
    """Per-phase counts of the reference algorithm's FP64 operations for one
    step on one region (the arrays are updated in place)."""
    lib = ctypes.CDLL(str(build_opcount()), mode=os.RTLD_LOCAL)
    dp = ctypes.POINTER(ctypes.c_double)
    lib.nsw6o_count_ops.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, ctypes.POINTER(ctypes.c_void_p),
                                    ctypes.c_double, ctypes.POINTER(ctypes.c_longlong)]
    kall, gall = reg["rhog"].shape
    p = np.array([default_params()[n] for n in PARAM_NAMES])
    ptrs = (ctypes.c_void_p * len(MP_DRIVER_ARGS))()
    for i, (name, _, _) in enumerate(MP_DRIVER_ARGS):
        ptrs[i] = reg[name].ctypes.data
    out = (ctypes.c_longlong * (4 * 8))()
    gz = np.ascontiguousarray(gz, dtype=np.float64)
    gzh = np.ascontiguousarray(gzh, dtype=np.float64)
    rc = lib.nsw6o_count_ops(gall, kall, gz.ctypes.data_as(dp), gzh.ctypes.data_as(dp), p.ctypes.data_as(dp), ptrs,
                             float(dt), out)
    res = {ph: {op: int(out[i * 8 + j]) for j, op in enumerate(OP_NAMES)} for i, ph in enumerate(PHASES)}
    res["rc"] = rc
    return res


def build_branchsig(force: bool = False) -> Path:
    """Decision-recording build (oracle/branchsig.cpp)."""
    BUILD.mkdir(parents=True, exist_ok=True)
    so = BUILD / "libnsw6_branchsig.so"
    src = [HERE / "branchsig.cpp", HERE / "nsw6_oracle.c", HERE / "nsw6_oracle.h"]
    if so.exists() and not force and all(so.stat().st_mtime >= s.stat().st_mtime for s in src):
        return so
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fPIC", "-shared", "-w", f"-I{HERE}",
                    str(HERE / "branchsig.cpp"), "-o", str(so)], check=True)
    return so


# Sites of the decision record (the enum in nsw6_oracle.c).
SITES = ["other", "rates", "limiter", "negfilter", "departure", "fluxsum", "epsfilter", "newton", "diag"]


def branch_record(reg: dict[str, np.ndarray], gz: np.ndarray, gzh: np.ndarray, dt: float,
                  params: dict[str, float] | None = None, inplace: bool = False) -> dict[str, np.ndarray]:
    """The discrete decisions of one step of the reference algorithm on one
    region, in program order (the region's arrays are stepped in place with
    ``inplace``, else left unchanged):

      code  uint8   site << 2 | kind << 1 | outcome (kind 1: an integer conversion)
      val   float64 the compared difference a - b, the sign argument, or the integer
      mag   float64 the larger magnitude of the compared operands

    Two steps whose records have equal codes (and equal integers) take the
    same branch everywhere."""
    lib = _LIBS.get("branchsig")
    if lib is None:
        lib = ctypes.CDLL(str(build_branchsig()), mode=os.RTLD_LOCAL)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.nsw6o_branch_record.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, ctypes.POINTER(ctypes.c_void_p),
                                            ctypes.c_double, ctypes.POINTER(ctypes.c_longlong)]
        lib.nsw6o_branch_copy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]
        _LIBS["branchsig"] = lib
    dp = ctypes.POINTER(ctypes.c_double)
    if inplace:
        work = reg
        for n, _, _ in MP_DRIVER_ARGS:
            if work[n].dtype != np.float64 or not work[n].flags.c_contiguous:
                raise ValueError(f"argument {n}: must be contiguous float64 to be stepped in place")
    else:
        work = {n: np.array(reg[n], dtype=np.float64, order="C", copy=True) for n, _, _ in MP_DRIVER_ARGS}
    kall, gall = work["rhog"].shape
    par = default_params()
    par.update(params or {})
    p = np.array([par[n] for n in PARAM_NAMES])
    ptrs = (ctypes.c_void_p * len(MP_DRIVER_ARGS))()
    for i, (name, _, _) in enumerate(MP_DRIVER_ARGS):
        ptrs[i] = work[name].ctypes.data
    gz = np.ascontiguousarray(gz, dtype=np.float64)
    gzh = np.ascontiguousarray(gzh, dtype=np.float64)
    n = ctypes.c_longlong(0)
    rc = lib.nsw6o_branch_record(gall, kall, gz.ctypes.data_as(dp), gzh.ctypes.data_as(dp), p.ctypes.data_as(dp),
                                 ptrs, float(dt), ctypes.byref(n))
    if rc != 0:
        raise RuntimeError(f"decision-recording step failed with status {rc}")
    out = {"code": np.empty(n.value, dtype=np.uint8), "val": np.empty(n.value), "mag": np.empty(n.value)}
    lib.nsw6o_branch_copy(out["code"].ctypes.data, out["val"].ctypes.data, out["mag"].ctypes.data, n.value)
    return out


def decision_changes(r0: dict[str, np.ndarray], r1: dict[str, np.ndarray], tie_rel: float = 0.0,
                     tie_abs: float = 0.0) -> dict | None:
    """Compares two decision records of the same region.  None when the
    control flow differs (a different number of decisions: a Newton iteration
    or a search loop ran a different number of times); else, per site, the
    number of decisions taken differently, the largest |val| and |val| / mag
    of those decisions in the first record (how far from its switch each one
    was), how many of them were not ties there (|val| > tie_abs and
    |val| > tie_rel * mag), and how many sat exactly on their switch there
    (val == 0: a kink at the point itself)."""
    if len(r0["code"]) != len(r1["code"]):
        return None
    c0, c1 = r0["code"], r1["code"]
    integer = (c0 & 2) != 0
    changed = (c0 != c1) | (integer & (r0["val"] != r1["val"]))
    site = c0 >> 2
    res = {}
    for s, name in enumerate(SITES):
        m = changed & (site == s)
        v = np.abs(r0["val"][m])
        mag = r0["mag"][m]
        rel = v / np.maximum(mag, 1e-300)
        res[name] = {"changed": int(m.sum()), "max_abs": float(v.max()) if v.size else 0.0,
                     "max_rel": float(rel.max()) if rel.size else 0.0,
                     "untied": int(((v > tie_abs) & (v > tie_rel * mag)).sum()),
                     "exact": int((v == 0.0).sum())}
    return res


_LIBS: dict[str, ctypes.CDLL] = {}


def load(variant: str = "strict", build_if_missing: bool = True) -> ctypes.CDLL:
    lib = _LIBS.get(variant)
    if lib is not None:
        return lib
    path = build(variant) if build_if_missing else lib_path(variant)
    lib = ctypes.CDLL(str(path), mode=os.RTLD_LOCAL)
    dp = ctypes.POINTER(ctypes.c_double)
    lib.nsw6o_default_params.argtypes = [ctypes.POINTER(Params)]
    lib.nsw6o_mp_driver.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, ctypes.POINTER(Params),
                                    ctypes.POINTER(ctypes.c_void_p), ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.nsw6o_mp_driver.restype = ctypes.c_int
    lib.nsw6o_max_threads.restype = ctypes.c_int
    _LIBS[variant] = lib
    return lib


def default_params() -> dict[str, float]:
    p = Params()
    load().nsw6o_default_params(ctypes.byref(p))
    return {n: getattr(p, n) for n in PARAM_NAMES}


def mp_driver(reg: dict[str, np.ndarray], gz: np.ndarray, gzh: np.ndarray, dt: float, ct: float = 0.0,
              params: dict[str, float] | None = None, variant: str = "strict", itelim: int = 100):
    """Run the restated mp_driver in place on one region (per-region layout).

    Returns (rc, status[4]) with rc 0 on success and 2 when the saturation
    Newton iteration did not converge within ``itelim`` iterations.
    """
    lib = load(variant)
    kall, gall = reg["rhog"].shape
    p = Params()
    lib.nsw6o_default_params(ctypes.byref(p))
    for k, v in (params or {}).items():
        setattr(p, k, float(v))
    ptrs = (ctypes.c_void_p * len(MP_DRIVER_ARGS))()
    for i, (name, kind, _) in enumerate(MP_DRIVER_ARGS):
        a = reg[name]
        if a.shape != region_shape(kind, kall, gall) or a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError(f"argument {name}: bad shape/dtype {a.shape} {a.dtype}")
        ptrs[i] = a.ctypes.data
    gz = np.ascontiguousarray(gz, dtype=np.float64)
    gzh = np.ascontiguousarray(gzh, dtype=np.float64)
    st = (ctypes.c_int * 4)()
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lib.nsw6o_mp_driver(gall, kall, gz.ctypes.data_as(dp), gzh.ctypes.data_as(dp), ctypes.byref(p), ptrs,
                             float(dt), float(ct), int(itelim), st)
    return rc, list(st)

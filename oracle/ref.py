"""ctypes wrapper around the reference NSW6 build (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/_ref/<variant>_g<gall>_k<kall>/libnsw6ref.so`` produced by
``oracle/build_ref.py`` and runs the reference's own ``mp_driver``
(src/mod_mp_driver.cpp:335-613) on numpy arrays.  Only tests, the golden
fixture generator and the CPU-baseline leg of bench.py use this module.
"""
from __future__ import annotations

import ctypes
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
if str(HERE.parent) not in sys.path:
    sys.path.insert(0, str(HERE.parent))

from nicam_kokkos_microphysics_gb300.state import MP_DRIVER_ARGS, region_shape  # noqa: E402

from oracle import build_ref  # noqa: E402

_LIBS: dict[tuple[int, int, str], ctypes.CDLL] = {}


def available() -> bool:
    return build_ref.sources_available()


# Scheme switches in the order of nsw6ref_set_options (oracle/ref_driver.cpp)
# and of nsw6_options (include/nsw6.h), with the reference's defaults.
OPTION_NAMES = ["roh2014", "explicit_icegen", "kk2000", "qi_sediment", "kin2kin", "aerosol_indirect"]
DEFAULT_OPTIONS = {"roh2014": 1, "explicit_icegen": 1, "kk2000": 1, "qi_sediment": 0, "kin2kin": 0,
                   "aerosol_indirect": 0}


def load(gall: int, kall: int, gz: np.ndarray, gzh: np.ndarray, variant: str = "strict",
         build: bool = True, options: dict | None = None) -> ctypes.CDLL:
    """Load (building if needed) the reference compiled for (gall, kall) and run its set-up.

    The reference keeps its grid and parameters in process globals, so one
    library instance serves one (gall, kall) grid; loading twice with a
    different grid re-runs the set-up.  ``options`` (the "opt" variant only)
    sets the scheme switches before the set-up; missing keys take the
    reference's defaults.
    """
    if options is not None and variant != "opt":
        raise ValueError("scheme options need the 'opt' build of the reference")
    key = (gall, kall, variant)
    lib = _LIBS.get(key)
    if lib is None:
        path = build_ref.build(gall, kall, variant) if build else build_ref.lib_path(gall, kall, variant)
        lib = ctypes.CDLL(str(path), mode=os.RTLD_LOCAL)
        lib.nsw6ref_setup.argtypes = [ctypes.POINTER(ctypes.c_double)] * 2
        lib.nsw6ref_mp_driver.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.c_double, ctypes.c_double]
        lib.nsw6ref_set_params.argtypes = [ctypes.POINTER(ctypes.c_double)]
        lib.nsw6ref_get_params.argtypes = [ctypes.POINTER(ctypes.c_double)]
        lib.nsw6ref_set_options.argtypes = [ctypes.POINTER(ctypes.c_int)]
        _LIBS[key] = lib
    if variant == "opt":
        o = dict(DEFAULT_OPTIONS, **(options or {}))
        arr = (ctypes.c_int * len(OPTION_NAMES))(*[int(o[n]) for n in OPTION_NAMES])
        if lib.nsw6ref_set_options(arr) != 0:
            raise RuntimeError("reference build without scheme switches")
    gz = np.ascontiguousarray(gz, dtype=np.float64)
    gzh = np.ascontiguousarray(gzh, dtype=np.float64)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lib.nsw6ref_setup(gz.ctypes.data_as(dp), gzh.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"reference set-up failed ({rc})")
    return lib


def get_params(lib) -> np.ndarray:
    p = np.zeros(5)
    lib.nsw6ref_get_params(p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return p


def set_params(lib, p) -> None:
    p = np.ascontiguousarray(p, dtype=np.float64)
    lib.nsw6ref_set_params(p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))


def mp_driver(lib, reg: dict[str, np.ndarray], dt: float, ct: float = 0.0, l_region: int = 0) -> int:
    """Run the reference mp_driver in place on one region's arrays (per-region layout)."""
    gall, kall = lib.nsw6ref_gall(), lib.nsw6ref_kall()
    ptrs = (ctypes.c_void_p * len(MP_DRIVER_ARGS))()
    for i, (name, kind, _) in enumerate(MP_DRIVER_ARGS):
        a = reg[name]
        if a.shape != region_shape(kind, kall, gall) or a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError(f"argument {name}: bad shape/dtype {a.shape} {a.dtype}")
        ptrs[i] = a.ctypes.data
    return lib.nsw6ref_mp_driver(l_region, ptrs, float(dt), float(ct))

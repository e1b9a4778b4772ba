"""Build and load the in-tree CUDA library ``libnsw6_gb300.so`` (sm_103a).

The library is compiled with nvcc directly (no CMake, no torch extension
machinery) so that the same recipe works on every host that has the CUDA 13
toolkit.  ``load()`` raises if the library is missing: there is no CPU or
PyTorch fallback for the NSW6 step.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libnsw6_gb300.so"

SOURCES = ["nsw6_kernels.cu", "nsw6_deriv.cu", "nsw6_adjoint.cu", "nsw6_driver.cu"]
HEADERS = ["nsw6_common.cuh", "nsw6_cell.cuh", "nsw6_fastmath.cuh", "nsw6_ad.cuh", "nsw6_column_step.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false keeps every product and sum separately rounded, as the
# reference's arithmetic is written; fused operations are spelled out
# explicitly where they are wanted.
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-shared"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise FileNotFoundError("nvcc not found: the CUDA 13 toolkit is required to build the NSW6 library")
    return cand


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / s for s in SOURCES + HEADERS] + [INCLUDE / "nsw6.h", Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the translation units in parallel, then link the library."""
    if not force and not _stale():
        return LIB
    import concurrent.futures as cf
    LIBDIR.mkdir(parents=True, exist_ok=True)
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)
    compile_flags = [f for f in NVCC_FLAGS if f != "-shared"]

    def compile_one(src: str) -> Path:
        obj = objdir / (Path(src).stem + ".o")
        cmd = [nvcc(), *ARCH, *compile_flags, "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        subprocess.run(cmd, check=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([nvcc(), *ARCH, "-shared", *[str(o) for o in objs], "-o", str(tmp)], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib: ctypes.CDLL | None = None


def load() -> ctypes.CDLL:
    """Load the CUDA library (built by ``build()``); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        raise RuntimeError(
            f"{LIB} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(str(LIB), mode=os.RTLD_GLOBAL)
    c_int, c_double, vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    lib.nsw6_create.argtypes = [ctypes.POINTER(vp), c_int, c_int, c_int, vp, vp]
    lib.nsw6_destroy.argtypes = [vp]
    lib.nsw6_set_params.argtypes = [vp, vp]
    lib.nsw6_get_params.argtypes = [vp, vp]
    lib.nsw6_default_params.argtypes = [vp]
    lib.nsw6_default_params.restype = None
    lib.nsw6_set_stream.argtypes = [vp, vp]
    lib.nsw6_set_sync_check.argtypes = [vp, c_int]
    lib.nsw6_set_itelim.argtypes = [vp, c_int]
    lib.nsw6_set_precip_stride.argtypes = [vp, ctypes.c_longlong]
    lib.nsw6_last_error.argtypes = [vp] + [ctypes.POINTER(c_int)] * 4
    lib.nsw6_set_timing.argtypes = [vp, c_int]
    lib.nsw6_set_math.argtypes = [vp, c_int]
    lib.nsw6_eval_math.argtypes = [vp, c_int, vp, vp, vp, c_int]
    lib.nsw6_read_timing.argtypes = [vp, ctypes.POINTER(c_double), c_int, ctypes.POINTER(c_int)]
    lib.nsw6_strerror.argtypes = [c_int]
    lib.nsw6_strerror.restype = ctypes.c_char_p
    lib.mp_driver_argv.argtypes = [vp, c_int, ctypes.POINTER(vp), c_double, c_double, c_int]
    lib.nsw6_host_copy_bytes.argtypes = [vp, c_int, ctypes.POINTER(ctypes.c_ulonglong),
                                         ctypes.POINTER(ctypes.c_ulonglong)]
    lib.mp_driver.argtypes = [vp, c_int] + [vp] * 46 + [c_double, c_double] + [vp] * 4
    lib.mp_driver_batched.argtypes = [vp, c_int] + [vp] * 46 + [c_double, c_double] + [vp] * 4
    lib.mp_driver_mixed.argtypes = [vp, c_int] + [vp] * 46 + [c_double, c_double] + [vp] * 4
    lib.nsw6_set_precision.argtypes = [vp, c_int]
    lib.nsw6_set_adjoint_mode.argtypes = [vp, c_int]
    lib.nsw6_default_options.argtypes = [vp]
    lib.nsw6_default_options.restype = None
    lib.nsw6_set_options.argtypes = [vp, vp]
    lib.nsw6_get_options.argtypes = [vp, vp]
    lib.mp_driver_steps.argtypes = [vp, c_int, ctypes.POINTER(vp), c_double, c_double, c_int]
    lib.mp_driver_tlm.argtypes = [vp, c_int, ctypes.POINTER(vp), ctypes.POINTER(vp), vp, c_double, c_double]
    lib.mp_driver_adjoint.argtypes = [vp, c_int, ctypes.POINTER(vp), ctypes.POINTER(vp), vp, c_double, c_double]
    lib.mp_driver_noalloc.argtypes = [c_int, c_int, vp, vp, vp, ctypes.POINTER(vp), c_double, c_double, vp]
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    """Function names declared in include/nsw6.h."""
    import re
    text = (INCLUDE / "nsw6.h").read_text()
    return sorted(set(re.findall(r"^(?:int|void|const char\*)\s+(\w+)\(", text, flags=re.M)))

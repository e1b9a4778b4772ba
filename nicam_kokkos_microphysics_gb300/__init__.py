"""GB300-native NICAM NSW6 microphysics step.

Python mirror of the reference's driver interface (src/mod_mp_driver.h):

* ``mp_init(MP_TYPE, gall, kall, gz, gzh, lall_max=1)`` replaces the set-up
  sequence GRD_Setup / CVW_CPW_Setup / SATURATION_Setup / mp_init of the
  reference harness (src/main.cpp:177-189) and returns an :class:`MPDriver`.
  Like the reference (mod_mp_driver.cpp:11-24) it accepts only "NSW6".
* ``MPDriver.mp_driver(l_region, rhog, ..., dt, ct, GDCLW, GDCFRC, GPREC,
  CBMFX)`` takes the reference's 50 array arguments in the reference's order
  (float64 CUDA tensors, updated in place) and runs one NSW6 step on one
  region through the C ABI of ``include/nsw6.h``.
* ``MPDriver.mp_driver_batched(lall, ...)`` does the same for ``lall``
  regions stored in the all-regions layout of the reference harness.
* ``MPDriver.run(state, dt)`` takes a dict keyed by the reference argument
  names; numpy (host) arrays go through the host-memory entry point.

All compute runs in the CUDA library built from ``csrc/``; when it is missing
the import of this API fails with an explicit error.
"""
from __future__ import annotations

import ctypes
from typing import Any

import numpy as np

from . import _native
from .state import ARG_NAMES, MP_DRIVER_ARGS, batched_shape, region_shape

__all__ = ["MPDriver", "mp_init", "mp_driver_noalloc", "NSW6Error", "PARAM_NAMES", "OPTION_NAMES", "default_params",
           "default_options"]

PARAM_NAMES = ["beta_saut", "qicrt_saut", "Cr", "Cs", "Cg", "ice_nuc", "kk_aut"]
# Scheme switches of nsw6_options (include/nsw6.h), in its order.
OPTION_NAMES = ["roh2014", "explicit_icegen", "kk2000", "qi_sediment", "kin2kin", "aerosol_indirect"]

NSW6_OK, NSW6_ERR_BAD_ARG, NSW6_ERR_CUDA, NSW6_ERR_NOCONV, NSW6_ERR_NAN = 0, 1, 2, 3, 4


class _Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in PARAM_NAMES]


class _Options(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in OPTION_NAMES]


class NSW6Error(RuntimeError):
    def __init__(self, code: int, msg: str, cell: tuple[int, int, int, int] | None = None):
        super().__init__(f"nsw6 error {code}: {msg}" + (f" (k={cell[0]} g={cell[1]} l={cell[2]} iters={cell[3]})"
                                                        if cell else ""))
        self.code = code
        self.cell = cell


def default_params() -> dict[str, float]:
    lib = _native.load()
    p = _Params()
    lib.nsw6_default_params(ctypes.byref(p))
    return {n: getattr(p, n) for n in PARAM_NAMES}


def default_options() -> dict[str, int]:
    """The reference's scheme configuration (nsw6_default_options)."""
    lib = _native.load()
    o = _Options()
    lib.nsw6_default_options(ctypes.byref(o))
    return {n: getattr(o, n) for n in OPTION_NAMES}


def _check(rc: int, lib, handle=None) -> None:
    if rc == NSW6_OK:
        return
    cell = None
    msg = lib.nsw6_strerror(rc).decode()
    raise NSW6Error(rc, msg, cell)


class MPDriver:
    """One NSW6 configuration on one grid: owns the device workspace."""

    def __init__(self, gall: int, kall: int, gz, gzh, lall_max: int = 1, params: dict | None = None,
                 options: dict | None = None):
        self._lib = _native.load()
        self.gall, self.kall, self.lall_max = int(gall), int(kall), int(lall_max)
        gz = np.ascontiguousarray(gz, dtype=np.float64)
        gzh = np.ascontiguousarray(gzh, dtype=np.float64)
        if gz.shape != (self.kall,) or gzh.shape != (self.kall,):
            raise ValueError("gz and gzh must have kall elements")
        h = ctypes.c_void_p()
        rc = self._lib.nsw6_create(ctypes.byref(h), self.gall, self.kall, self.lall_max,
                                   gz.ctypes.data, gzh.ctypes.data)
        _check(rc, self._lib)
        self._h = h
        if params:
            self.set_params(**params)
        if options:
            self.set_options(**options)

    # ------------------------------------------------------------ lifetime
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.nsw6_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ settings
    def get_params(self) -> dict[str, float]:
        p = _Params()
        _check(self._lib.nsw6_get_params(self._h, ctypes.byref(p)), self._lib)
        return {n: getattr(p, n) for n in PARAM_NAMES}

    def set_params(self, **kw: float) -> None:
        cur = self.get_params()
        for k, v in kw.items():
            if k not in cur:
                raise KeyError(f"unknown NSW6 parameter {k!r}")
            cur[k] = float(v)
        p = _Params(**cur)
        _check(self._lib.nsw6_set_params(self._h, ctypes.byref(p)), self._lib)

    def get_options(self) -> dict[str, int]:
        o = _Options()
        _check(self._lib.nsw6_get_options(self._h, ctypes.byref(o)), self._lib)
        return {n: getattr(o, n) for n in OPTION_NAMES}

    def set_options(self, **kw: int) -> None:
        """Scheme switches (nsw6_options): roh2014, explicit_icegen, kk2000,
        qi_sediment, kin2kin, aerosol_indirect; unnamed ones keep their value."""
        cur = self.get_options()
        for k, v in kw.items():
            if k not in cur:
                raise KeyError(f"unknown NSW6 option {k!r}")
            cur[k] = int(v)
        o = _Options(**cur)
        _check(self._lib.nsw6_set_options(self._h, ctypes.byref(o)), self._lib)

    def set_precip_stride(self, ld: int) -> None:
        """Row stride of precip / ISO1_precip / ISO2_precip in ``mp_driver``
        (per-region) calls: ``lall * gall`` takes the reference harness's
        subview of its [2][lall][1][gall] array; 0 restores [2][gall]."""
        _check(self._lib.nsw6_set_precip_stride(self._h, ctypes.c_longlong(int(ld))), self._lib)

    def set_itelim(self, itelim: int) -> None:
        _check(self._lib.nsw6_set_itelim(self._h, int(itelim)), self._lib)

    def set_sync_check(self, on: bool) -> None:
        _check(self._lib.nsw6_set_sync_check(self._h, int(bool(on))), self._lib)

    def set_stream(self, stream: Any) -> None:
        """cudaStream_t as int, or a torch.cuda.Stream."""
        ptr = getattr(stream, "cuda_stream", stream)
        _check(self._lib.nsw6_set_stream(self._h, ctypes.c_void_p(int(ptr or 0))), self._lib)

    def set_precision(self, mode: int | str) -> None:
        """0 / "fp64": the plain FP64 step (default); 1 / "mixed": FP32 process
        rates with FP64 budgets, flux sums and saturation adjustment; 2 /
        "serial": the FP64 step one column per thread, by the code of the
        derivative kernels (for checking them)."""
        m = {"fp64": 0, "mixed": 1, "serial": 2}.get(mode, mode) if isinstance(mode, str) else int(mode)
        _check(self._lib.nsw6_set_precision(self._h, int(m)), self._lib)

    def set_adjoint_mode(self, mode: int | str) -> None:
        """Implementation of ``adjoint``: 0 / "hand" the hand-written reverse
        sweeps (default), 1 / "tape" the recorded operations, 2 / "check" as
        "hand" with its forward checked bitwise against the step's cell
        physics on every cell (a difference raises NSW6_ERR_CHECK)."""
        m = {"hand": 0, "tape": 1, "check": 2}.get(mode, mode) if isinstance(mode, str) else int(mode)
        _check(self._lib.nsw6_set_adjoint_mode(self._h, int(m)), self._lib)

    def set_math(self, mode: int) -> None:
        """0: table-driven exp/log/pow (default), 1: CUDA math library."""
        _check(self._lib.nsw6_set_math(self._h, int(mode)), self._lib)

    def eval_math(self, fn: int, x, y=None):
        """Evaluate the table-driven exp (0), log (1) or pow (2) on CUDA tensors."""
        import torch
        out = torch.empty_like(x)
        yp = y.data_ptr() if y is not None else None
        _check(self._lib.nsw6_eval_math(self._h, int(fn), x.data_ptr(), yp, out.data_ptr(), x.numel()), self._lib)
        return out

    def set_timing(self, on: bool) -> None:
        _check(self._lib.nsw6_set_timing(self._h, int(bool(on))), self._lib)

    def read_timing(self) -> tuple[float, float, int]:
        """(cell kernel ms, column kernel ms, steps) accumulated since the last read."""
        t = (ctypes.c_double * 2)()
        n = ctypes.c_int()
        _check(self._lib.nsw6_read_timing(self._h, t, 2, ctypes.byref(n)), self._lib)
        return t[0], t[1], n.value

    def host_copy_bytes(self, lall: int | None = None) -> tuple[int, int]:
        """(bytes in, bytes out) that one host-memory call on lall (default lall_max) regions copies."""
        h2d, d2h = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        n = self.lall_max if lall is None else lall
        _check(self._lib.nsw6_host_copy_bytes(self._h, n, ctypes.byref(h2d), ctypes.byref(d2h)), self._lib)
        return h2d.value, d2h.value

    def last_error(self) -> tuple[int, tuple[int, int, int, int]]:
        k, g, l, it = (ctypes.c_int() for _ in range(4))
        rc = self._lib.nsw6_last_error(self._h, ctypes.byref(k), ctypes.byref(g), ctypes.byref(l), ctypes.byref(it))
        return rc, (k.value, g.value, l.value, it.value)

    def _raise_status(self, rc: int) -> None:
        if rc == NSW6_OK:
            return
        raise NSW6Error(rc, self._lib.nsw6_strerror(rc).decode())

    # ------------------------------------------------------------ calls
    def _device_ptrs(self, args, shapes) -> list[int]:
        import torch
        ptrs = []
        for (name, _, _), a, shp in zip(MP_DRIVER_ARGS, args, shapes):
            if not isinstance(a, torch.Tensor):
                raise TypeError(f"{name}: expected a CUDA tensor, got {type(a).__name__}")
            if a.device.type != "cuda" or a.dtype != torch.float64 or not a.is_contiguous():
                raise ValueError(f"{name}: expected a contiguous float64 CUDA tensor")
            if tuple(a.shape) != tuple(shp):
                raise ValueError(f"{name}: expected shape {tuple(shp)}, got {tuple(a.shape)}")
            ptrs.append(a.data_ptr())
        return ptrs

    def _use_torch_stream(self) -> None:
        import torch
        self.set_stream(torch.cuda.current_stream().cuda_stream)

    def mp_driver(self, l_region: int, *args, dt: float | None = None, ct: float = 0.0):
        """Reference argument order: 46 arrays, dt, ct, 4 arrays (mod_mp_driver.h:71-124)."""
        arrays, dt, ct = _split_args(args, dt, ct)
        shapes = [region_shape(kind, self.kall, self.gall) for _, kind, _ in MP_DRIVER_ARGS]
        ptrs = self._device_ptrs(arrays, shapes)
        self._use_torch_stream()
        rc = self._lib.mp_driver(self._h, int(l_region), *ptrs[:46], float(dt), float(ct), *ptrs[46:])
        self._raise_status(rc)

    def mp_driver_mixed(self, l_region: int, *args, dt: float | None = None, ct: float = 0.0):
        """mp_driver in mixed precision for this call (C ABI mp_driver_mixed)."""
        arrays, dt, ct = _split_args(args, dt, ct)
        shapes = [region_shape(kind, self.kall, self.gall) for _, kind, _ in MP_DRIVER_ARGS]
        ptrs = self._device_ptrs(arrays, shapes)
        self._use_torch_stream()
        rc = self._lib.mp_driver_mixed(self._h, int(l_region), *ptrs[:46], float(dt), float(ct), *ptrs[46:])
        self._raise_status(rc)

    def mp_driver_batched(self, lall: int, *args, dt: float | None = None, ct: float = 0.0):
        arrays, dt, ct = _split_args(args, dt, ct)
        shapes = [batched_shape(kind, lall, self.kall, self.gall) for _, kind, _ in MP_DRIVER_ARGS]
        ptrs = self._device_ptrs(arrays, shapes)
        self._use_torch_stream()
        rc = self._lib.mp_driver_batched(self._h, int(lall), *ptrs[:46], float(dt), float(ct), *ptrs[46:])
        self._raise_status(rc)

    def run(self, state: dict, dt: float, ct: float = 0.0, lall: int | None = None) -> None:
        """Run one step in place on a dict keyed by the reference argument names.

        Arrays are in the all-regions layout (see ``state.batched_shape``).
        CUDA tensors run on the device; numpy arrays go through the host entry
        point, which copies inputs in and outputs back inside the call.
        """
        first = state[ARG_NAMES[0]]
        if lall is None:
            lall = first.shape[0]
        if isinstance(first, np.ndarray):
            ptrs = (ctypes.c_void_p * len(ARG_NAMES))()
            for i, (name, kind, _) in enumerate(MP_DRIVER_ARGS):
                a = state[name]
                if a.shape != batched_shape(kind, lall, self.kall, self.gall) or a.dtype != np.float64 \
                        or not a.flags.c_contiguous:
                    raise ValueError(f"{name}: expected contiguous float64 array of shape "
                                     f"{batched_shape(kind, lall, self.kall, self.gall)}")
                ptrs[i] = a.ctypes.data
            rc = self._lib.mp_driver_argv(self._h, int(lall), ptrs, float(dt), float(ct), 1)
            self._raise_status(rc)
            return
        self.mp_driver_batched(lall, *[state[n] for n in ARG_NAMES], dt=dt, ct=ct)

    def mp_driver_steps(self, lall: int, state: dict, nsteps: int, dt: float, ct: float = 0.0) -> None:
        """nsteps steps in place on ``state`` (CUDA tensors keyed by the
        argument names, all-regions layout) from one captured CUDA graph."""
        self._use_torch_stream()
        rc = self._lib.mp_driver_steps(self._h, int(lall), self._ptr_array(state, lall), float(dt), float(ct),
                                       int(nsteps))
        self._raise_status(rc)

    # ------------------------------------------------------- derivatives
    def _ptr_array(self, state: dict, lall: int):
        import torch
        arr = (ctypes.c_void_p * len(ARG_NAMES))()
        for i, (name, kind, _) in enumerate(MP_DRIVER_ARGS):
            t = state[name]
            shp = batched_shape(kind, lall, self.kall, self.gall)
            if not isinstance(t, torch.Tensor) or t.device.type != "cuda" or t.dtype != torch.float64 \
                    or not t.is_contiguous() or tuple(t.shape) != tuple(shp):
                raise ValueError(f"{name}: expected a contiguous float64 CUDA tensor of shape {tuple(shp)}")
            arr[i] = t.data_ptr()
        return arr

    def tlm(self, lall: int, state: dict, tangent: dict, dparams=None, dt: float = 60.0, ct: float = 0.0) -> None:
        """Tangent-linear step (C ABI mp_driver_tlm): advances ``state`` by one
        FP64 step and maps ``tangent`` (same keys and shapes) in place; dparams:
        7 parameter tangents or None."""
        self._use_torch_stream()
        dp = None
        if dparams is not None:
            dp = (ctypes.c_double * 7)(*[float(v) for v in dparams])
        rc = self._lib.mp_driver_tlm(self._h, int(lall), self._ptr_array(state, lall), self._ptr_array(tangent, lall),
                                     dp, float(dt), float(ct))
        self._raise_status(rc)

    def adjoint(self, lall: int, state: dict, adjoint: dict, dt: float = 60.0, ct: float = 0.0) -> np.ndarray:
        """Adjoint step (C ABI mp_driver_adjoint) around ``state`` (unchanged):
        ``adjoint`` holds the output adjoints on entry and the input adjoints on
        exit; returns the adjoint of the 7 parameters."""
        self._use_torch_stream()
        dp = (ctypes.c_double * 7)()
        rc = self._lib.mp_driver_adjoint(self._h, int(lall), self._ptr_array(state, lall),
                                         self._ptr_array(adjoint, lall), dp, float(dt), float(ct))
        self._raise_status(rc)
        return np.array(dp[:], dtype=np.float64)

    def run_argv(self, lall: int, ptrs: list[int], dt: float, ct: float = 0.0, host: bool = False) -> int:
        """Raw entry point: 50 pointers in reference order; returns the status code."""
        arr = (ctypes.c_void_p * len(ARG_NAMES))(*ptrs)
        return self._lib.mp_driver_argv(self._h, int(lall), arr, float(dt), float(ct), int(host))


def _split_args(args, dt, ct):
    """Accept either (46 arrays, dt, ct, 4 arrays) or 50 arrays with dt/ct keywords."""
    if len(args) == 52:
        return list(args[:46]) + list(args[48:]), float(args[46]), float(args[47])
    if len(args) == 50 and dt is not None:
        return list(args), float(dt), float(ct)
    raise TypeError("expected the 50 mp_driver arrays with dt and ct in the reference order")


def mp_init(MP_TYPE: str, gall: int, kall: int, gz, gzh, lall_max: int = 1, params: dict | None = None,
            options: dict | None = None) -> MPDriver:
    """Set up the microphysics driver (mod_mp_driver.cpp:11-24): only "NSW6" exists."""
    if MP_TYPE != "NSW6":
        raise ValueError(f"mp_init: NOT appropriate type. Type: {MP_TYPE}")
    return MPDriver(gall, kall, gz, gzh, lall_max=lall_max, params=params, options=options)


def mp_driver_noalloc(gall: int, kall: int, gz, gzh, *args, dt: float | None = None, ct: float = 0.0,
                      params: dict | None = None) -> None:
    """One NSW6 step on one region through ``mp_driver_noalloc`` of the C ABI,
    which allocates no device memory (its workspace is a fixed array inside the
    library; regions up to 2,097,152 cells and kall <= 160).  Arguments as
    ``MPDriver.mp_driver`` without the region index; runs on torch's current
    stream and returns after the step has finished."""
    import torch
    lib = _native.load()
    arrays, dt, ct = _split_args(args, dt, ct)
    shapes = [region_shape(kind, kall, gall) for _, kind, _ in MP_DRIVER_ARGS]
    ptrs = (ctypes.c_void_p * len(ARG_NAMES))()
    for i, ((name, _, _), a, shp) in enumerate(zip(MP_DRIVER_ARGS, arrays, shapes)):
        if not isinstance(a, torch.Tensor) or a.device.type != "cuda" or a.dtype != torch.float64 \
                or not a.is_contiguous() or tuple(a.shape) != tuple(shp):
            raise ValueError(f"{name}: expected a contiguous float64 CUDA tensor of shape {tuple(shp)}")
        ptrs[i] = a.data_ptr()
    gz = np.ascontiguousarray(gz, dtype=np.float64)
    gzh = np.ascontiguousarray(gzh, dtype=np.float64)
    if gz.shape != (kall,) or gzh.shape != (kall,):
        raise ValueError("gz and gzh must hold kall heights")
    p = None
    if params is not None:
        p = _Params()
        lib.nsw6_default_params(ctypes.byref(p))
        for k, v in params.items():
            setattr(p, k, float(v))
    rc = lib.mp_driver_noalloc(int(gall), int(kall), gz.ctypes.data, gzh.ctypes.data,
                               ctypes.addressof(p) if p is not None else None, ptrs, float(dt), float(ct),
                               torch.cuda.current_stream().cuda_stream)
    _check(rc, lib)

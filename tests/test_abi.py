"""CPU tests of the C ABI library: it builds, loads and exports every symbol
declared in include/nsw6.h (no compute call: there is no GPU here)."""
from __future__ import annotations

import ctypes
import subprocess

import pytest

from nicam_kokkos_microphysics_gb300 import _native


@pytest.fixture(scope="module")
def lib():
    _native.build()
    return ctypes.CDLL(str(_native.LIB))


def test_every_declared_symbol_exported(lib):
    names = _native.exported_symbols()
    assert "mp_driver" in names and "mp_driver_batched" in names and "nsw6_create" in names
    for n in names:
        assert hasattr(lib, n), n


def test_symbols_are_c_linkage():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_native.LIB)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for n in _native.exported_symbols():
        assert n in exported, n


def test_strerror_and_defaults(lib):
    lib.nsw6_strerror.restype = ctypes.c_char_p
    assert lib.nsw6_strerror(3) == b"saturation adjustment did not converge"
    p = (ctypes.c_double * 7)()
    lib.nsw6_default_params(p)
    assert p[0] == 5.0e-3 and p[2] == 130.0 and abs(p[4] - 82.48585739) < 1e-6 and p[6] == 1350.0


def test_bad_arguments_rejected(lib):
    h = ctypes.c_void_p()
    gz = (ctypes.c_double * 42)()
    # invalid sizes are rejected before any CUDA call
    assert lib.nsw6_create(ctypes.byref(h), 0, 42, 1, gz, gz) == 1
    assert lib.nsw6_create(ctypes.byref(h), 10, 3, 1, gz, gz) == 1
    assert lib.mp_driver_argv(None, 1, None, ctypes.c_double(60.0), ctypes.c_double(0.0), 0) == 1


def test_eps_bit_pattern_matches_eps():
    """The integer-pipe |f| >= EPS test of the column kernel uses EPS's bit pattern."""
    import re
    import struct
    from nicam_kokkos_microphysics_gb300 import _native
    text = (_native.CSRC / "nsw6_common.cuh").read_text()
    eps = float(re.search(r"constexpr double EPS = ([0-9.Ee+-]+);", text).group(1))
    bits = int(re.search(r"constexpr long long EPS_BITS = (0x[0-9a-fA-F]+)LL;", text).group(1), 16)
    assert struct.unpack("<q", struct.pack("<d", eps))[0] == bits

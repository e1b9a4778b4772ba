"""The integer-pipe double comparisons the kernels use (csrc/nsw6_fpcmp.cuh)
return what the IEEE comparisons return for every pair tried: the special
values pairwise (zeros, subnormals, infinities, NaNs of both signs) and four
million random and nearby pairs (tests/native/fpcmp_check.cpp, built with the
host compiler).  That covers the general comparisons, the cell physics'
comparisons with constants and the min / max selects they make (the same
double bit for bit, or both NaN), the limiters' forms for a bound that is not
negative, and the addition of +0."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_integer_comparisons_match_ieee(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "fpcmp_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "nicam_kokkos_microphysics_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "fpcmp_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout

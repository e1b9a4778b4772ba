"""The column kernel's saturation test, decided in FP32 outside a margin.

nsw6_column_kernel first decides qsum - qsat(T) > EPS in FP32: T, rho and
qsum are converted, the exponent is LovR (Tf - T00f) / (Tf T00f) (|x| <= 80),
and a cell is saturated when qsum_f > 1.0001 qsat_f, unsaturated when
qsum_f < 0.9999 qsat_f (qsat_f in [1e-11, 1e30]); the FP64 test decides the
rest.  This replays that rule with numpy's IEEE float32 arithmetic (round to
nearest, no contraction, as the kernel is built) and checks on states spread
over the temperatures, densities and distances from saturation the step meets,
most of them close to the threshold, that no decided cell takes the other
branch than the FP64 test, and that the FP32 qsat stays inside the error bound
the margin rests on: 4.2e-7 |x| + LovR 2^-24 (1/T00 + 1/T) for the exponent
(seven roundings, the conversions of T and T00) and 7.2e-7 for expf's 2 ulp
and the eight roundings after it.  numpy's float32 exp stands in for CUDA's
expf; both are within 2 ulp.
"""
from __future__ import annotations

import numpy as np

from nicam_kokkos_microphysics_gb300.state import LHV, PSAT0, RVAP, TEM00

EPS = 2.220446e-16
TEM_MIN = 10.0


def fp64_test(qsum, tem, rho):
    rtem = 1.0 / np.maximum(tem, TEM_MIN)
    qsat = PSAT0 * np.exp(LHV / RVAP * (1.0 / TEM00 - rtem)) / (rho * RVAP * tem)
    return qsum - qsat > EPS, qsat


def fp32_screen(qsum, tem, rho):
    """1 saturated, 0 not, -1 deferred to the FP64 test; and the FP32 qsat."""
    f = np.float32
    with np.errstate(over="ignore", under="ignore", invalid="ignore", divide="ignore"):
        tf = tem.astype(f)
        tcf = np.where(tf < f(TEM_MIN), f(TEM_MIN), tf)
        xf = f(LHV / RVAP) * ((tcf - f(TEM00)) / (tcf * f(TEM00)))
        qsf = (f(PSAT0) * np.exp(xf)) / (rho.astype(f) * f(RVAP) * tf)
        qq = qsum.astype(f)
        ok = (np.abs(xf) <= f(80.0)) & (qsf >= f(1.0e-11)) & (qsf <= f(1.0e30))
        sat = np.full(qsum.shape, -1)
        sat[ok & (qq > qsf * f(1.0001))] = 1
        sat[ok & (sat < 0) & (qq < qsf * f(0.9999))] = 0
    return sat, qsf.astype(np.float64), xf


def test_fp32_screen_takes_the_fp64_branch():
    rng = np.random.default_rng(7)
    n = 2_000_000
    tem = rng.uniform(150.0, 340.0, n)
    rho = 10.0 ** rng.uniform(-3.5, 0.3, n)
    _, qsat = fp64_test(np.zeros(n), tem, rho)
    # distances from saturation from 1e-12 to 1 (relative), both signs, and
    # some cells exactly at saturation
    off = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-12.0, 0.0, n)
    off[: n // 50] = 0.0
    qsum = qsat * (1.0 + off)
    ref, qsat64 = fp64_test(qsum, tem, rho)
    sat, qs, xf = fp32_screen(qsum, tem, rho)
    decided = sat >= 0
    assert not np.any(sat[decided] != ref[decided].astype(int))
    # the bound the 1e-4 margin rests on
    rel = np.abs(qs / qsat64 - 1.0)
    tc = np.maximum(tem, TEM_MIN)
    bound = 4.2e-7 * np.abs(xf.astype(np.float64)) + LHV / RVAP * 2.0**-24 * (1.0 / TEM00 + 1.0 / tc) + 7.2e-7
    assert bound[decided].max() < 4.3e-5
    assert np.all(rel[decided] <= bound[decided])
    # the margin defers only cells near the threshold
    assert decided[np.abs(off) > 1.5e-4].all()
    assert not decided[np.abs(off) < 5.7e-5].any()


def test_fp32_screen_defers_out_of_range_and_invalid():
    # below TEM_MIN the exponent leaves the range; NaN and negative temperatures
    # and zero density defer to the FP64 test
    tem = np.array([5.0, 9.0, np.nan, -20.0, 250.0])
    rho = np.array([1.0, 1.0, 1.0, 1.0, 0.0])
    qsum = np.array([1e-3, 1e-3, 1e-3, 1e-3, 1e-3])
    sat, _, _ = fp32_screen(qsum, tem, rho)
    assert (sat == -1).all()

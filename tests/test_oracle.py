"""CPU tests of the oracle: the C restatement against the reference's own results.

* golden fixtures (made by tests/golden/make_golden.py from the reference's
  unmodified sources) are reproduced by the restatement;
* where the reference tree is present, the restatement equals the reference
  build bit for bit on fresh seeded states of several shapes and variants.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from conftest import golden_files
from nicam_kokkos_microphysics_gb300.state import (MP_DRIVER_ARGS, OUTPUT_NAMES, StateSpec, make_state,
                                                   region_shape, region_view)
from oracle import ref, restatement
from _parity import compare, passes, summary


def load_golden(path):
    z = np.load(path)
    gz, gzh = z["gz"], z["gzh"]
    kall, gall = z["in_rhog"].shape
    reg = {}
    for name, kind, intent in MP_DRIVER_ARGS:
        if f"in_{name}" in z:
            reg[name] = z[f"in_{name}"].copy()
        else:
            reg[name] = np.full(region_shape(kind, kall, gall), np.nan)
    out = {n: z[f"out_{n}"] for n in OUTPUT_NAMES}
    return reg, out, gz, gzh, float(z["dt"])


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.stem)
def test_restatement_reproduces_golden(path):
    reg, out, gz, gzh, dt = load_golden(path)
    rc, st = restatement.mp_driver(reg, gz, gzh, dt)
    assert rc == 0, st
    # the golden outputs come from the reference built on x86-64; another
    # host's libm may differ in the last place, hence the tight tolerance and
    # the threshold-cell allowance instead of bit equality
    stats = compare(reg, out, OUTPUT_NAMES, rtol=1e-13, atol=1e-300)
    assert passes(stats), summary(stats)


def test_outputs_fully_written():
    """Every output element is written (outputs start as NaN)."""
    path = golden_files()[0]
    reg, out, gz, gzh, dt = load_golden(path)
    rc, _ = restatement.mp_driver(reg, gz, gzh, dt)
    assert rc == 0
    for n in OUTPUT_NAMES:
        assert np.isfinite(reg[n]).all(), n


needs_ref = pytest.mark.skipif(not ref.available(), reason="reference sources not present")


@needs_ref
@pytest.mark.parametrize("variant,gall,kall,seed", [
    ("standard", 64, 42, 101), ("convective", 64, 42, 102), ("cold", 64, 42, 103),
    ("convective", 96, 12, 104), ("standard", 33, 7, 105),
])
def test_restatement_bitwise_equals_reference(variant, gall, kall, seed):
    spec = StateSpec(gall=gall, kall=kall, lall=1, seed=seed, variant=variant)
    st = make_state(spec, out_fill=np.nan)
    lib = ref.load(gall, kall, st["_gz"], st["_gzh"])
    r1 = region_view(st, 0)
    r2 = {k: v.copy() for k, v in r1.items()}
    assert ref.mp_driver(lib, r1, spec.dt) == 0
    rc, s = restatement.mp_driver(r2, st["_gz"], st["_gzh"], spec.dt)
    assert rc == 0, s
    for n in OUTPUT_NAMES:
        assert np.array_equal(r1[n].view(np.int64), r2[n].view(np.int64)), n


@needs_ref
def test_restatement_bitwise_with_changed_parameters():
    """The five tunables the reference exposes through GlobalParams."""
    spec = StateSpec(gall=48, kall=42, lall=1, seed=7, variant="convective")
    st = make_state(spec, out_fill=np.nan)
    lib = ref.load(spec.gall, spec.kall, st["_gz"], st["_gzh"])
    p = {"beta_saut": 7.5e-3, "qicrt_saut": 1.0e-6, "Cr": 120.0, "Cs": 5.1, "Cg": 70.0}
    default = ref.get_params(lib)
    try:
        ref.set_params(lib, [p["beta_saut"], p["qicrt_saut"], p["Cr"], p["Cs"], p["Cg"]])
        r1 = region_view(st, 0)
        r2 = {k: v.copy() for k, v in r1.items()}
        assert ref.mp_driver(lib, r1, spec.dt) == 0
    finally:
        ref.set_params(lib, default)
    rc, _ = restatement.mp_driver(r2, st["_gz"], st["_gzh"], spec.dt, params=p)
    assert rc == 0
    for n in OUTPUT_NAMES:
        assert np.array_equal(r1[n].view(np.int64), r2[n].view(np.int64)), n


def test_restatement_reports_nonconvergence():
    """An iteration limit of 1 makes saturated cells fail; the oracle reports it."""
    reg, out, gz, gzh, dt = load_golden(golden_files()[0])
    rc, st = restatement.mp_driver(reg, gz, gzh, dt, itelim=1)
    assert rc == 2
    assert st[0] == 2 and 1 <= st[1] <= reg["rhog"].shape[0] - 2


@needs_ref
@pytest.mark.parametrize("variant,seed", [("convective", 1002), ("cold", 1003)])
def test_reference_own_build_spread(variant, seed):
    """The reference compiled with fused multiply-add contraction (as its nvcc
    and -Ofast builds are) against its strict build, on one full 130 x 130
    region: every cell is inside the scale-aware tolerance of tests/_parity.py,
    yet a few hundred near-zero mixing ratios (cancellation residues of fully
    consumed species, cloud water from qsum - qsat) miss the bare 1e-11
    relative / 1e-20 absolute bound.  This is the spread the GPU parity tests'
    threshold-cell budget is calibrated against."""
    spec = StateSpec(gall=16900, kall=42, lall=1, seed=seed, variant=variant)
    st = make_state(spec, out_fill=np.nan)
    a = region_view(st, 0)
    b = {k: v.copy() for k, v in a.items()}
    assert ref.mp_driver(ref.load(spec.gall, spec.kall, st["_gz"], st["_gzh"], variant="strict"), a, spec.dt) == 0
    assert ref.mp_driver(ref.load(spec.gall, spec.kall, st["_gz"], st["_gzh"], variant="fma"), b, spec.dt) == 0
    stats = compare(b, a, OUTPUT_NAMES)
    thr = sum(s["n_threshold"] for s in stats.values())
    print(f"\nreference fma vs strict, {variant}: {thr} threshold cells\n" + summary(stats))
    assert all(s["n_bad"] == 0 for s in stats.values())
    assert passes(stats)


@needs_ref
@pytest.mark.parametrize("variant,seed", [("standard", 201), ("cold", 202)])
def test_reference_switch_build_equals_strict_at_defaults(variant, seed):
    """The "opt" build (switch assignments of mp_nsw6_init turned into
    variables) computes exactly what the unmodified build computes when the
    switches hold the reference's values."""
    spec = StateSpec(gall=40, kall=42, lall=1, seed=seed, variant=variant)
    st = make_state(spec, out_fill=np.nan)
    r1 = region_view(st, 0)
    r2 = {k: v.copy() for k, v in r1.items()}
    assert ref.mp_driver(ref.load(40, 42, st["_gz"], st["_gzh"]), r1, spec.dt) == 0
    assert ref.mp_driver(ref.load(40, 42, st["_gz"], st["_gzh"], variant="opt", options={}), r2, spec.dt) == 0
    for n in OUTPUT_NAMES:
        assert np.array_equal(r1[n].view(np.int64), r2[n].view(np.int64)), n


@needs_ref
@pytest.mark.parametrize("path", sorted((Path(__file__).parent / "golden").glob("options_*.npz")),
                         ids=lambda p: p.stem)
def test_reference_reproduces_options_fixture(path):
    """Each switch fixture is what the reference's "opt" build gives for its
    switches, bit for bit."""
    z = np.load(path)
    reg, out, gz, gzh, dt = load_golden(path)
    kall, gall = reg["rhog"].shape
    opts = {n: int(v) for n, v in zip(ref.OPTION_NAMES, z["options"])}
    lib = ref.load(gall, kall, gz, gzh, variant="opt", options=opts)
    assert ref.mp_driver(lib, reg, dt) == 0
    for n in OUTPUT_NAMES:
        assert np.array_equal(np.asarray(reg[n]).view(np.int64), np.asarray(out[n]).view(np.int64)), n

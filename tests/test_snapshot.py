"""Snapshot files of the reference harness (nicam_kokkos_microphysics_gb300.snapshot):
round trip, agreement with the reference's own readers (src/data_io.cpp) and
its result check PROF_val_check (src/mod_debug.cpp:48-79)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from nicam_kokkos_microphysics_gb300 import snapshot
from nicam_kokkos_microphysics_gb300.state import ARG_NAMES, StateSpec, make_state
from oracle import ref

needs_ref = pytest.mark.skipif(not ref.available(), reason="reference sources not present")


def test_round_trip(tmp_path):
    spec = StateSpec(gall=130, kall=12, lall=2, seed=9, variant="convective")
    st = make_state(spec, out_fill=0.0)
    snapshot.write_snapshot(tmp_path, st)
    snapshot.write_vgrid(tmp_path, st["_gz"], st["_gzh"])
    back = snapshot.read_snapshot(tmp_path, spec.gall, spec.kall, spec.lall)
    for n in ARG_NAMES:
        if n in snapshot.FILES:
            assert np.array_equal(back[n], st[n]), n
    gz, gzh = snapshot.read_vgrid(tmp_path, spec.kall)
    assert np.array_equal(gz, st["_gz"]) and np.array_equal(gzh, st["_gzh"])


def test_val_check_matches_the_reference_definition(tmp_path):
    spec = StateSpec(gall=64, kall=12, lall=1, seed=4, variant="standard")
    st = make_state(spec, out_fill=0.0)
    snapshot.write_check_files(tmp_path, st)
    rows = snapshot.check_results(tmp_path, st)
    assert [r[0] for r in rows] == ["rhog", "rhogvx", "rhogvy", "rhogvz", "rhogw", "rhoge", "QV", "QC", "QR", "QI",
                                    "QS", "QG"]
    for _, mx, mn, s in rows:   # identical fields: max stays at DBL_MIN, min and sum are 0
        assert mx == np.finfo(np.float64).tiny and mn == 0.0 and s == 0.0
    other = {k: v.copy() for k, v in st.items()}
    other["rhog"][0, 3, 5] += 1e-3
    other["rhog"][0, 4, 6] -= 2e-3
    r = snapshot.check_results(tmp_path, other)[0]
    assert r[1] == pytest.approx(2e-3) and r[2] == 0.0 and r[3] == pytest.approx(3e-3)
    assert "Checking [rhog] Max = " in snapshot.format_check([r])


@needs_ref
def test_reference_readers_read_the_written_files(tmp_path):
    spec = StateSpec(gall=40, kall=12, lall=1, seed=21, variant="convective")
    st = make_state(spec, out_fill=0.0)
    lib = ref.load(spec.gall, spec.kall, st["_gz"], st["_gzh"])
    snapshot.write_snapshot(tmp_path, st)
    snapshot.write_vgrid(tmp_path, st["_gz"], st["_gzh"])
    d = tmp_path / "data"
    cases = [("rhog", "3d"), ("tem", "3d"), ("rhogq", "4d"), ("q", "4d"), ("ix", "2d"), ("precip", "precip")]
    for name, kind in cases:
        out = np.zeros_like(st[name])
        fn = getattr(lib, f"nsw6ref_read_{kind}")
        fn.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
        fn.restype = None
        fn(str(d / snapshot.FILES[name]).encode(), out.ctypes.data)
        assert np.array_equal(out, st[name]), name
    out = np.zeros(spec.kall)
    lib.nsw6ref_read_1d.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    lib.nsw6ref_read_1d(str(d / "vgrid" / "GRD_gzh.dat").encode(), out.ctypes.data)
    assert np.array_equal(out, st["_gzh"])

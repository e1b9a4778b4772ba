"""CPU tests of the synthetic state generator and the grid convention."""
from __future__ import annotations

import numpy as np

from nicam_kokkos_microphysics_gb300.state import (I_QV, MP_DRIVER_ARGS, StateSpec, batched_shape, grid_factors,
                                                   make_state, vertical_grid)


def test_grid_halo_convention():
    gz, gzh = vertical_grid(42)
    assert gzh[1] == 0.0 and abs(gzh[41] - 40000.0) < 1e-9
    assert gzh[0] == -gzh[2] and gz[0] == -gz[1]
    assert gz[41] == 2 * gzh[41] - gz[40]
    assert np.all(np.diff(gzh) > 0) and np.all(np.diff(gz) > 0)
    f = grid_factors(gz, gzh)
    assert np.allclose(f["afact"] + f["bfact"], 1.0)


def test_state_deterministic_and_shapes():
    spec = StateSpec(gall=37, kall=12, lall=2, seed=5, variant="convective")
    a, b = make_state(spec), make_state(spec)
    for name, kind, intent in MP_DRIVER_ARGS:
        assert a[name].shape == batched_shape(kind, 2, 12, 37)
        if intent != "out":
            assert np.array_equal(a[name], b[name]), name


def test_state_physical_ranges():
    spec = StateSpec(gall=200, kall=42, lall=1, seed=3)
    st = make_state(spec)
    tem = st["tem"][0, 1:41]
    assert 200 < tem.min() and tem.max() < 310
    assert (st["rhog"] > 0).all()
    q = st["q"][0]
    assert (q >= 0).all() and q[I_QV].max() < 0.05
    assert np.array_equal(q, st["rhogq"][0] / st["rhog"][0][None])

"""Accuracy of the table-driven FP64 exp / log / pow used by the step, on the
GPU, against correctly rounded values (tests/golden/fastmath_cr.npz) and next
to CUDA's own functions."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "fastmath_cr.npz"


def ulp_err(got, want):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    sp = np.spacing(np.abs(want))
    sp = np.where(sp == 0, np.finfo(np.float64).tiny, sp)
    return np.abs(got - want) / sp


@pytest.fixture(scope="module")
def drv():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nicam_kokkos_microphysics_gb300 import mp_init
    from nicam_kokkos_microphysics_gb300.state import vertical_grid
    gz, gzh = vertical_grid(12)
    d = mp_init("NSW6", 8, 12, gz, gzh)
    yield d
    d.close()


@pytest.mark.parametrize("fn,name,bound", [(0, "exp", 1.0), (1, "log", 1.0), (2, "pow", 2.0)])
def test_fast_transcendental_accuracy(drv, fn, name, bound):
    import torch
    z = np.load(GOLD)
    x = torch.from_numpy(z[f"{name}_x"]).cuda()
    if fn == 2:
        y = torch.from_numpy(z["pow_y"]).cuda()
        want = z["pow_r"]
        lib = torch.pow(x, y).cpu().numpy()
        got = drv.eval_math(2, x, y).cpu().numpy()
    else:
        want = z[f"{name}_y"]
        lib = (torch.exp(x) if fn == 0 else torch.log(x)).cpu().numpy()
        got = drv.eval_math(fn, x).cpu().numpy()
    e = ulp_err(got, want)
    el = ulp_err(lib, want)
    print(f"\n{name}: fast max {e.max():.3f} ulp, mean {e.mean():.3f}, correctly rounded {np.mean(e <= 0.5):.4f}; "
          f"CUDA max {el.max():.3f} ulp, correctly rounded {np.mean(el <= 0.5):.4f}")
    assert e.max() <= bound, f"{name}: max error {e.max()} ulp"

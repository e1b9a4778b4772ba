"""Parity statistics between a candidate result and the oracle.

`field_stats` reports, per output field, the reference's own check statistic
(signed max / min / sum of candidate - oracle, as PROF_val_check prints it,
src/mod_debug.cpp:363-410) and the per-cell agreement used as the pass
criterion:

    |a - b| <= ATOL + RTOL * |b| + FLOOR * scale

with RTOL = 1e-11 and ATOL = 1e-20.  `scale` is the field's dynamic range
(max |b| over the region) and, for the tracer fields q and rhogq, the cell's
total water (sum over the six species); FLOOR = 1e-14.

The floor exists because the reference computes some values by cancellation
of much larger numbers: the cloud water of the saturation adjustment is
qsum - qsat (mod_satadjust.cpp:859-860) with qsum ~ 1e-2 and the result as
small as 1e-7, so one unit in the last place of qsat (~2e-18) is a relative
error of 1e-11 in qc; and the absolute flux filter |F| < EPS
(mod_vadv1d.cpp:446-449) switches tiny fluxes on or off.  Cells that pass only
thanks to the floor are counted as threshold cells (`n_threshold`); the tests
bound their number by the count of the reference's own fma build against its
strict build on the same state (`reference_spread`), and check the
reference's statistic against the same per-cell bound (`statistic_ok`).
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-11
ATOL = 1e-20
FLOOR = 1e-14
TRACER_FIELDS = ("q", "rhogq")
MAX_THRESHOLD_FRACTION = 1e-4


def field_stats(a: np.ndarray, b: np.ndarray, rtol: float = RTOL, atol: float = ATOL,
                scale: np.ndarray | float | None = None, floor: float = FLOOR) -> dict:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.where(both_nan, 0.0, a - b)
    strict = np.abs(d) <= atol + rtol * np.abs(b)
    if scale is None:
        scale = float(np.nanmax(np.abs(b))) if b.size else 0.0
    ok = np.abs(d) <= atol + rtol * np.abs(b) + floor * scale
    ok |= both_nan
    strict |= both_nan
    rel = np.abs(d) / np.maximum(np.abs(b), 1e-300)
    rel = np.where(np.abs(d) <= atol, 0.0, rel)
    bound = atol + rtol * np.abs(np.where(np.isnan(b), 0.0, b)) + floor * np.broadcast_to(scale, b.shape)
    return {
        "max": float(d.max()) if d.size else 0.0,
        "min": float(d.min()) if d.size else 0.0,
        "sum": float(d.sum()) if d.size else 0.0,
        "max_rel": float(rel.max()) if rel.size else 0.0,
        "max_abs": float(np.abs(d).max()) if d.size else 0.0,
        "n_bad": int((~ok).sum()),
        "n_threshold": int((ok & ~strict).sum()),
        "n": int(d.size),
        "bitwise_equal": int((a.view(np.int64) == b.view(np.int64)).sum()) if a.size else 0,
        # the reference's statistic (signed max, min and sum of the
        # difference) is within the per-cell bound's largest value and sum
        "statistic_ok": bool(max(abs(float(d.max())), abs(float(d.min()))) <= float(bound.max())
                             and abs(float(d.sum())) <= float(bound.sum())) if d.size else True,
    }


def compare(cand: dict, oracle: dict, names, rtol: float = RTOL, atol: float = ATOL, floor: float = FLOOR) -> dict:
    out = {}
    for n in names:
        b = np.asarray(oracle[n])
        scale = None
        if n in TRACER_FIELDS and b.ndim >= 3:
            # tracer axis is the one of length 6 right before [kall][gall]
            tot = np.abs(b).sum(axis=-3, keepdims=True)
            scale = np.broadcast_to(tot, b.shape)
        out[n] = field_stats(cand[n], b, rtol, atol, scale, floor)
    return out


def passes(stats: dict, max_fraction: float = MAX_THRESHOLD_FRACTION) -> bool:
    n = sum(s["n"] for s in stats.values())
    thr = sum(s["n_threshold"] for s in stats.values())
    return (all(s["n_bad"] == 0 and s["statistic_ok"] for s in stats.values())
            and thr <= max(8, max_fraction * n))


def threshold_cells(stats: dict) -> int:
    """Values that miss the bare bound ATOL + RTOL |b| (admitted by the scale term)."""
    return int(sum(s["n_threshold"] for s in stats.values()))


def reference_spread() -> dict:
    """Threshold cells of the reference's own fma build against its strict
    build, per state of the GPU parity tests (tests/golden/make_spread.py)."""
    import json
    from pathlib import Path
    p = Path(__file__).resolve().parent / "golden" / "reference_spread.json"
    return json.loads(p.read_text())


def summary(stats: dict) -> str:
    lines = []
    for n, s in stats.items():
        lines.append(f"{n:15s} max={s['max']:+.3e} min={s['min']:+.3e} sum={s['sum']:+.3e} "
                     f"max_rel={s['max_rel']:.2e} bad={s['n_bad']} thr={s['n_threshold']}/{s['n']} "
                     f"bitwise={s['bitwise_equal']}")
    return "\n".join(lines)

"""Parity statistics between a candidate result and the oracle.

`field_stats` reports, per output field, the reference's own check statistic
(signed max / min / sum of candidate - oracle, as PROF_val_check prints it,
src/mod_debug.cpp:363-410) together with the per-cell agreement used as the
pass criterion: |a - b| <= atol + rtol * |b| with rtol = 1e-11 and
atol = 1e-20 (the absolute floor applies to near-zero mixing ratios).
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-11
ATOL = 1e-20


def field_stats(a: np.ndarray, b: np.ndarray, rtol: float = RTOL, atol: float = ATOL) -> dict:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = a - b
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.where(both_nan, 0.0, d)
    bad = ~(np.abs(d) <= atol + rtol * np.abs(b))
    bad &= ~both_nan
    rel = np.abs(d) / np.maximum(np.abs(b), 1e-300)
    rel = np.where(np.abs(d) <= atol, 0.0, rel)
    return {
        "max": float(d.max()) if d.size else 0.0,
        "min": float(d.min()) if d.size else 0.0,
        "sum": float(d.sum()) if d.size else 0.0,
        "max_rel": float(rel.max()) if rel.size else 0.0,
        "n_bad": int(bad.sum()),
        "n": int(d.size),
        "bitwise_equal": int((a.view(np.int64) == b.view(np.int64)).sum()) if a.size else 0,
    }


def compare(cand: dict, oracle: dict, names, rtol: float = RTOL, atol: float = ATOL) -> dict:
    return {n: field_stats(cand[n], oracle[n], rtol, atol) for n in names}


def summary(stats: dict) -> str:
    lines = []
    for n, s in stats.items():
        lines.append(f"{n:15s} max={s['max']:+.3e} min={s['min']:+.3e} sum={s['sum']:+.3e} "
                     f"max_rel={s['max_rel']:.2e} bad={s['n_bad']}/{s['n']} bitwise={s['bitwise_equal']}")
    return "\n".join(lines)

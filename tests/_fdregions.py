"""Regions and certified finite-difference points for the parameter-gradient
checks of the adjoint step (test infrastructure).

The loss of the derivative checks is L = sum_g (precip_rain + precip_solid)^2
+ sum_{g,k} rhogq[QC] dz.  A central difference of L with respect to one of
the seven NSW6 parameters, with the relative step 1e-6, resolves the
derivative to 1e-6 only where two conditions hold:

* the step's rounding noise in L is far below the change the step h makes.
  Wherever the saturation adjustment leaves cloud water, rhogq[QC] = rhog
  (qsum - qsat(T)) is a cancellation residue with a relative rounding noise
  of order 1e-14 qsat / qc, and the column-integrated cloud water dominates L
  by orders of magnitude (precip^2 is of order 1e-10).  A parameter that
  changes L by a relative 1e-5 (the fall speeds, autoconversion and ice
  autoconversion do, through the surface precipitation) then moves L by
  1e-11 of itself at h, which that noise swamps.  The *precipitating* region
  below is therefore assembled from columns that the step leaves without
  cloud water (every cell ends subsaturated, so rhogq[QC] is exactly zero)
  and whose surface precipitation is above the median of the precipitating
  columns: L is then the surface precipitation alone.  The autoconversion
  rate's share of the surface rain is small except in a few columns; it is
  checked on those (the *autoconversion* region).  The ice-nucleation
  coefficient acts on L through the cloud water only (nucleated ice takes
  vapour, the adjustment then leaves less cloud water); it is checked on a
  *cloudy* region, where its effect is large enough.
* no discrete decision of the step changes between p - h and p + h.  The
  decision-recording build of the reference algorithm
  (oracle/branchsig.cpp) lists every decision; `certify` accepts a finite-
  difference point when the control flow is the same, none of the decisions
  the adjoint holds fixed changes (departure cells, flux bounds, the flux
  integral's weights, the saturation test and the Newton iteration), and
  every other decision that changes was a tie at p: its two sides agreed to
  a few units in the last place, or it tested a rounding residue below
  1e-13 (the |flux| < EPS filter on a flux that is a cancellation residue,
  the negative filter on a residue around zero).
"""
from __future__ import annotations

import numpy as np

from nicam_kokkos_microphysics_gb300.state import MP_DRIVER_ARGS, StateSpec, make_state, region_view

# Sites whose decisions the tangent-linear and adjoint steps hold fixed: any
# change there disqualifies a finite-difference point.
FIXED_SITES = ("departure", "fluxsum", "newton")
# A changed decision elsewhere is a tie at p when its compared difference was
# within TIE_REL of the operands' magnitude, or below TIE_ABS in absolute value.
TIE_REL = 1e-15
TIE_ABS = 1e-13

# (variant, seed) of the three column pools of the precipitating region
POOLS = (("standard", 2024), ("cold", 2025), ("convective", 2026))


def _oracle():
    from oracle import restatement
    return restatement


def _step(reg, gz, gzh, dt=60.0, params=None):
    R = _oracle()
    y = {k: v.copy() for k, v in reg.items()}
    rc, status = R.mp_driver(y, gz, gzh, dt, params=params)
    if rc != 0:
        raise RuntimeError(f"oracle step failed: {status}")
    return y


def _columns(reg, cols):
    out = {}
    for name, kind, _ in MP_DRIVER_ARGS:
        out[name] = np.ascontiguousarray(reg[name][..., cols])
    return out


def _concat(parts):
    return {name: np.ascontiguousarray(np.concatenate([p[name] for p in parts], axis=-1))
            for name, _, _ in MP_DRIVER_ARGS}


def precipitating_region(per_pool: int = 32, kall: int = 42, pool_gall: int = 4096):
    """The first `per_pool` columns of each pool (standard, cold and
    convective generator states of `pool_gall` columns) that the reference
    step leaves without cloud water and whose surface precipitation is above
    the median of the pool's precipitating columns.  Returns (region arrays
    in the per-region layout, gz, gzh)."""
    parts = []
    for variant, seed in POOLS:
        st = make_state(StateSpec(gall=pool_gall, kall=kall, lall=1, seed=seed, variant=variant), out_fill=0.0)
        reg = region_view(st, 0)
        y = _step(reg, st["_gz"], st["_gzh"])
        pr = y["precip"][0] + y["precip"][1]
        cloud_free = (y["rhogq"][1] == 0.0).all(axis=0)
        above = pr > np.median(pr[pr > 0.0])
        cols = np.nonzero(cloud_free & above)[0][:per_pool]
        parts.append(_columns(reg, cols))
    return _concat(parts), st["_gz"], st["_gzh"]


def autoconversion_region(ncol: int = 8, kall: int = 42, pool_gall: int = 4096, seed: int = 2024):
    """The KK2000 autoconversion rate changes the surface precipitation by the
    rain it makes in the lowest layer, a small share of that layer's rain
    except where cloud water is plentiful and rain scarce.  The `ncol`
    columns of a standard generator state that the reference step leaves
    without cloud water, that precipitate, and whose lowest layer holds cloud
    water and rain with the largest qc^2.47 / qr (the autoconversion rate's
    share of the rain there)."""
    st = make_state(StateSpec(gall=pool_gall, kall=kall, lall=1, seed=seed, variant="standard"), out_fill=0.0)
    reg = region_view(st, 0)
    y = _step(reg, st["_gz"], st["_gzh"])
    pr = y["precip"][0] + y["precip"][1]
    cloud_free = (y["rhogq"][1] == 0.0).all(axis=0)
    qc, qr = reg["q"][1][1], reg["q"][2][1]
    share = np.where((qc > 0.0) & (qr > 0.0), qc ** 2.47 / np.where(qr > 0.0, qr, 1.0), 0.0)
    cand = np.nonzero(cloud_free & (pr > 0.0) & (share > 0.0))[0]
    cols = np.sort(cand[np.argsort(share[cand], kind="stable")[::-1][:ncol]])
    return _columns(reg, cols), st["_gz"], st["_gzh"]


def cloudy_region(ncol: int = 64, kall: int = 42, pool_gall: int = 4096, seed: int = 2024):
    """The first `ncol` columns of a standard generator state that the
    reference step leaves with cloud water below a cold layer (ice
    nucleation acts above, the adjustment below)."""
    st = make_state(StateSpec(gall=pool_gall, kall=kall, lall=1, seed=seed, variant="standard"), out_fill=0.0)
    reg = region_view(st, 0)
    y = _step(reg, st["_gz"], st["_gzh"])
    cloudy = (y["rhogq"][1] > 0.0).any(axis=0)
    cols = np.nonzero(cloudy)[0][:ncol]
    return _columns(reg, cols), st["_gz"], st["_gzh"]


def loss_weights(gzh: np.ndarray) -> np.ndarray:
    """dz of every interior level (0 at the two halo levels)."""
    kall = len(gzh)
    dgz = np.diff(gzh, append=gzh[-1] + (gzh[-1] - gzh[-2]))
    w = np.zeros(kall)
    w[1:kall - 1] = dgz[1:kall - 1]
    return w


def certify(reg, gz, gzh, name: str, p0: float, steps, dt: float = 60.0) -> dict:
    """Decision records of the reference step at p0 and at p0 + s for every s
    in `steps`; returns {"ok": bool, "per_step": [...]} where each entry gives
    per site the number of changed decisions and their largest margins."""
    R = _oracle()
    r0 = R.branch_record(reg, gz, gzh, dt, {name: p0})
    ok = True
    per_step = []
    for s in steps:
        ch = R.decision_changes(r0, R.branch_record(reg, gz, gzh, dt, {name: p0 + s}), TIE_REL, TIE_ABS)
        if ch is None:
            ok = False
            per_step.append({"step": s, "control_flow": "differs"})
            continue
        for site, c in ch.items():
            if not c["changed"]:
                continue
            if site in FIXED_SITES or c["untied"]:
                ok = False
        per_step.append({"step": s, **{k: v for k, v in ch.items() if v["changed"]}})
    return {"ok": ok, "per_step": per_step}


def certify_window(reg, gz, gzh, name: str, p0: float, steps, nsteps: int, dt: float = 60.0) -> dict:
    """`certify` over a window of `nsteps` steps: the decision records of every
    step along the trajectory from p0 and along each trajectory from p0 + s."""
    R = _oracle()
    base, r0 = {k: v.copy() for k, v in reg.items()}, []
    for _ in range(nsteps):
        r0.append(R.branch_record(base, gz, gzh, dt, {name: p0}, inplace=True))
    ok = True
    per_step = []
    for s in steps:
        x = {k: v.copy() for k, v in reg.items()}
        entry = {"step": s}
        for n in range(nsteps):
            ch = R.decision_changes(r0[n], R.branch_record(x, gz, gzh, dt, {name: p0 + s}, inplace=True),
                                    TIE_REL, TIE_ABS)
            if ch is None:
                ok = False
                entry[f"step{n}"] = "control flow differs"
                break
            for site, c in ch.items():
                if c["changed"] and (site in FIXED_SITES or c["untied"]):
                    ok = False
            entry[f"step{n}"] = {k: v for k, v in ch.items() if v["changed"]}
        per_step.append(entry)
    return {"ok": ok, "per_step": per_step}

"""Tangent-linear and adjoint steps (mp_driver_tlm / mp_driver_adjoint).

* their forward, the FP64 step evaluated one column per thread, equals the
  production kernels bit for bit;
* adjoint dot-product test: <ybar, TLM dx> = <ADJ ybar, dx> + <pbar, dp>;
* the gradient of the loss L = sum_g (precip_rain + precip_solid)^2 +
  sum_{g,k} rhogq[QC] dgz(k) (surface precipitation and column-integrated
  cloud water) with respect to state components and the seven NSW6 parameters
  against FP64 central finite differences of the production step (relative
  step 1e-6), at points away from the scheme's switches: a point is used when
  the differences with steps h and h/4 agree (no switch flips in between).
"""
from __future__ import annotations

import numpy as np
import pytest

from nicam_kokkos_microphysics_gb300.autograd import READ_NAMES, WRITE_NAMES
from nicam_kokkos_microphysics_gb300.state import ARG_NAMES, OUTPUT_NAMES, StateSpec, make_state, vertical_grid

pytestmark = pytest.mark.gpu
PARAMS = ["beta_saut", "qicrt_saut", "Cr", "Cs", "Cg", "ice_nuc", "kk_aut"]


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


# the scheme switches that act in the cell physics only (the derivative
# entry points take these): Berry warm rain, the aerosol effect, the classic
# snow moments with explicit ice generation
CELL_SWITCHES = dict(roh2014=0, explicit_icegen=1, kk2000=0, aerosol_indirect=1)
# and with the Bergeron process and the mixed-phase saturation adjustment
ICE_SWITCHES = dict(roh2014=0, explicit_icegen=0, kk2000=0, aerosol_indirect=1)
# the transport's kinetic-energy correction KIN2KIN in place of KIN2EIN
KIN2KIN = dict(kin2kin=1)
# cloud ice sediments as a fourth tracer ("4WATER")
QI_SEDIMENT = dict(qi_sediment=1)
# every switch off its default at once
ALL_SWITCHES = dict(roh2014=0, explicit_icegen=0, kk2000=0, qi_sediment=1, kin2kin=1, aerosol_indirect=1)


def _setup(gall=4096, kall=42, lall=1, seed=2024, variant="standard", options=None):
    torch = _torch()
    from nicam_kokkos_microphysics_gb300 import mp_init
    spec = StateSpec(gall=gall, kall=kall, lall=lall, seed=seed, variant=variant)
    st = make_state(spec, out_fill=0.0)
    if options and options.get("aerosol_indirect"):
        st["unccn"][...] = np.random.default_rng(seed).uniform(1.0e7, 2.0e9, st["unccn"].shape)
    drv = mp_init("NSW6", gall, kall, st["_gz"], st["_gzh"], lall_max=lall, options=options)
    x0 = {n: torch.from_numpy(st[n].copy()).cuda() for n in ARG_NAMES}
    return torch, drv, spec, st, x0


def _clone(d):
    return {k: v.clone() for k, v in d.items()}


@pytest.mark.parametrize("variant,gall,kall", [("standard", 500, 42), ("convective", 500, 42), ("cold", 300, 42),
                                               ("convective", 129, 12)])
def test_serial_forward_bitwise_equals_production(variant, gall, kall):
    torch, drv, spec, st, x0 = _setup(gall, kall, 2, 11, variant)
    a, b = _clone(x0), _clone(x0)
    drv.mp_driver_batched(spec.lall, *[a[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    drv.set_precision("serial")
    drv.mp_driver_batched(spec.lall, *[b[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    torch.cuda.synchronize()
    for n in OUTPUT_NAMES:
        assert torch.equal(a[n], b[n]), n
    drv.close()


@pytest.mark.parametrize("gall,kall,lall,options,variant", [
    (1024, 42, 1, None, "convective"), (192, 160, 2, None, "convective"),
    (1024, 42, 1, CELL_SWITCHES, "convective"), (1024, 42, 1, ICE_SWITCHES, "cold"),
    (1024, 42, 1, KIN2KIN, "convective"), (1024, 42, 2, QI_SEDIMENT, "cold"),
    (192, 160, 1, QI_SEDIMENT, "cold"), (1024, 42, 1, ALL_SWITCHES, "cold")],
    ids=["42", "160", "switches", "ice-switches", "kin2kin", "qi-sediment", "qi-sediment-160", "all-switches"])
def test_adjoint_dot_product(gall, kall, lall, options, variant):
    """<ybar, J dx> + 0 = <J^T ybar, dx> + <pbar, dp> between the staged
    tangent-linear and adjoint steps, also on the deepest columns (160 levels,
    beyond the serial column step's 48), with the cell-physics switches and
    with cloud ice sedimenting as a fourth tracer."""
    torch, drv, spec, st, x0 = _setup(gall, kall, lall, 77, variant, options)
    g = torch.Generator(device="cuda").manual_seed(5)
    dx = {n: torch.zeros_like(v) for n, v in x0.items()}
    for n in READ_NAMES:
        dx[n] = 1e-3 * x0[n].abs().mean() * torch.randn(x0[n].shape, generator=g, device="cuda", dtype=torch.float64)
    dp = np.array([1e-5, 1e-7, 1.0, 0.05, 0.5, 1e-13, 10.0])
    # output weights: every output, or with KIN2KIN the four momenta alone
    # (which it changes; the other outputs' terms would dominate the sums)
    ynames = ("rhogvx", "rhogvy", "rhogvz", "rhogw") if options is KIN2KIN else WRITE_NAMES
    ybar = {n: torch.zeros_like(v) for n, v in x0.items()}
    for n in ynames:
        ybar[n] = torch.randn(x0[n].shape, generator=g, device="cuda", dtype=torch.float64) / \
            (x0[n].abs().mean() + 1e-30)
    # TLM
    x, t = _clone(x0), _clone(dx)
    drv.tlm(spec.lall, x, t, dparams=dp, dt=spec.dt)
    lhs = sum(float((ybar[n] * t[n]).sum()) for n in ynames)
    # adjoint
    bar = _clone(ybar)
    pbar = drv.adjoint(spec.lall, _clone(x0), bar, dt=spec.dt)
    rhs = sum(float((bar[n] * dx[n]).sum()) for n in READ_NAMES) + float(np.dot(pbar, dp))
    print(f"\ndot-product test ({gall}x{kall}x{lall}): <ybar, J dx> = {lhs:.17e}, <J^T ybar, dx> = {rhs:.17e}, "
          f"rel diff {abs(lhs - rhs) / abs(lhs):.2e}")
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)
    # the TLM's forward is the FP64 step
    y = _clone(x0)
    drv.mp_driver_batched(spec.lall, *[y[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    for n in OUTPUT_NAMES:
        assert torch.equal(y[n], x[n]), n
    drv.close()


@pytest.mark.parametrize("variant,seed", [("standard", 51), ("convective", 52), ("cold", 53)])
def test_staged_tlm_equals_serial(variant, seed):
    """The tangent-linear step in stages (every cell in parallel) gives the
    serial column step's tangents (adjoint mode 1: one column per thread over
    Dual) to rounding, and the same output values bit for bit."""
    torch, drv, spec, st, x0 = _setup(1024, 42, 2, seed, variant)
    g = torch.Generator(device="cuda").manual_seed(seed)
    dx = {n: torch.zeros_like(v) for n, v in x0.items()}
    for n in READ_NAMES:
        dx[n] = 1e-3 * x0[n].abs().mean() * torch.randn(x0[n].shape, generator=g, device="cuda", dtype=torch.float64)
    dp = np.array([1e-5, 1e-7, 1.0, 0.05, 0.5, 1e-13, 10.0])
    xs, ts = _clone(x0), _clone(dx)
    drv.tlm(spec.lall, xs, ts, dparams=dp, dt=spec.dt)
    drv.set_adjoint_mode("tape")
    xr, tr = _clone(x0), _clone(dx)
    drv.tlm(spec.lall, xr, tr, dparams=dp, dt=spec.dt)
    worst = 0.0
    for n in OUTPUT_NAMES:
        assert torch.equal(xs[n], xr[n]), n
    for n in WRITE_NAMES:
        scale = float(tr[n].abs().max())
        err = float((ts[n] - tr[n]).abs().max()) / scale if scale > 0 else float(ts[n].abs().max())
        worst = max(worst, err)
        assert err <= 1e-9, (n, err)
    print(f"\nstaged vs serial tangent-linear step ({variant}): worst field {worst:.2e}")
    drv.close()


@pytest.mark.parametrize("variant,seed", [("standard", 41), ("convective", 42), ("cold", 43)])
def test_adjoint_forward_checkpoint_bitwise(variant, seed):
    """The hand-written forward the cell adjoint's checkpoint comes from gives
    the step's cell-physics outputs bit for bit on every cell (adjoint mode
    "check" compares them in the kernel and fails the call otherwise), and the
    checked adjoint equals the plain one up to the order of its atomic sums
    (some input adjoints are sums that cancel, so the bound is relative to
    the field's largest entry)."""
    torch, drv, spec, st, x0 = _setup(1024, 42, 2, seed, variant)
    g = torch.Generator(device="cuda").manual_seed(seed)
    ybar = {n: torch.zeros_like(v) for n, v in x0.items()}
    for n in WRITE_NAMES:
        ybar[n] = torch.randn(x0[n].shape, generator=g, device="cuda", dtype=torch.float64)
    drv.set_adjoint_mode("check")
    b2 = _clone(ybar)
    p2 = drv.adjoint(spec.lall, _clone(x0), b2, dt=spec.dt)
    drv.set_adjoint_mode("hand")
    b0 = _clone(ybar)
    p0 = drv.adjoint(spec.lall, _clone(x0), b0, dt=spec.dt)
    for n in READ_NAMES:
        scale = float(b0[n].abs().max())
        if scale > 0.0:
            err = float((b2[n] - b0[n]).abs().max()) / scale
            assert err <= 1e-9, (n, err)
    assert np.allclose(p2, p0, rtol=1e-9, atol=0.0)
    drv.close()


@pytest.mark.parametrize("variant,seed,options", [("standard", 31, None), ("convective", 32, None), ("cold", 33, None),
                                                  ("cold", 34, QI_SEDIMENT)],
                         ids=["standard", "convective", "cold", "qi-sediment"])
def test_hand_written_adjoint_equals_recorded(variant, seed, options):
    """The hand-written adjoints of the cell physics and of the column
    phase's stages give the input and parameter adjoints of the
    operation-recording ones (their atomic sums make the last bits
    order-dependent); with QI sedimenting, those of the transport's four
    tracers."""
    torch, drv, spec, st, x0 = _setup(1024, 42, 1, seed, variant, options)
    g = torch.Generator(device="cuda").manual_seed(seed)
    ybar = {n: torch.zeros_like(v) for n, v in x0.items()}
    for n in WRITE_NAMES:
        ybar[n] = torch.randn(x0[n].shape, generator=g, device="cuda", dtype=torch.float64) / \
            (x0[n].abs().mean() + 1e-30)
    drv.set_adjoint_mode("tape")
    b1 = _clone(ybar)
    p1 = drv.adjoint(spec.lall, _clone(x0), b1, dt=spec.dt)
    drv.set_adjoint_mode("hand")
    b0 = _clone(ybar)
    p0 = drv.adjoint(spec.lall, _clone(x0), b0, dt=spec.dt)
    worst = 0.0
    for n in READ_NAMES:
        scale = float(b1[n].abs().max())
        if scale == 0.0:
            assert float(b0[n].abs().max()) == 0.0, n
            continue
        err = float((b0[n] - b1[n]).abs().max()) / scale
        worst = max(worst, err)
        assert err <= 1e-9, (n, err)
    perr = np.abs(p0 - p1) / np.maximum(np.abs(p1), 1e-300)
    print(f"\nhand-written vs recorded adjoint ({variant}): worst field {worst:.2e}, parameters {perr.max():.2e}")
    assert np.all(perr <= 1e-9), (p0, p1)
    drv.close()


@pytest.mark.parametrize("variant,seed", [("standard", 61), ("convective", 62), ("cold", 63)])
def test_mixed_adjoint_against_fp64_adjoint(variant, seed):
    """With the mixed-precision step selected, the adjoint's cell phase
    linearises that step's cell physics (FP32 rates and rate adjoints, FP64
    budgets; the column stages are FP64 in both): its forward reproduces the
    mixed-precision cell kernel bit for bit on every cell (adjoint mode
    "check"), and its input and parameter adjoints agree with those of the
    FP64 adjoint to the FP32 rounding of the rates.  Output seeds are random,
    scaled by each output's mean.  The adjoints with respect to tracer
    contents that are zero are compared apart: there a flux bound of the
    transport, set by the region's extreme departure distance and so by the
    last bits of a fall speed, decides whether an empty layer's (zero) source
    enters a flux integral, which changes that entry's adjoint and nothing
    else."""
    torch, drv, spec, st, x0 = _setup(4096, 42, 1, seed, variant)
    y0 = _clone(x0)
    drv.mp_driver_batched(spec.lall, *[y0[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
    g = torch.Generator(device="cuda").manual_seed(seed)
    ybar = {n: torch.zeros_like(v) for n, v in x0.items()}
    for n in WRITE_NAMES:
        scale = float(y0[n].abs().mean())
        if scale > 0.0:
            ybar[n] = torch.randn(x0[n].shape, generator=g, device="cuda", dtype=torch.float64) / scale
    b64 = _clone(ybar)
    p64 = drv.adjoint(spec.lall, _clone(x0), b64, dt=spec.dt)
    drv.set_precision("mixed")
    drv.set_adjoint_mode("check")
    b32 = _clone(ybar)
    p32 = drv.adjoint(spec.lall, _clone(x0), b32, dt=spec.dt)
    drv.set_adjoint_mode("hand")
    drv.set_precision("fp64")

    def rel(a, b):
        ref = float(torch.linalg.vector_norm(b))
        return float(torch.linalg.vector_norm(a - b)) / ref if ref > 0 else 0.0

    present = x0["rhogq"] > 0.0
    errs = {n: rel(b32[n], b64[n]) for n in READ_NAMES if n != "rhogq"}
    errs["rhogq (present)"] = rel(b32["rhogq"][present], b64["rhogq"][present])
    empty = rel(b32["rhogq"][~present], b64["rhogq"][~present])
    perr = np.abs(p32 - p64) / np.maximum(np.abs(p64), 1e-300)
    print(f"\nmixed vs FP64 adjoint ({variant}), relative 2-norm: "
          + ", ".join(f"{n} {e:.1e}" for n, e in errs.items())
          + f"; rhogq (empty) {empty:.1e}; parameters " + ", ".join(f"{v:.1e}" for v in perr))
    assert max(errs.values()) <= 1e-4, errs
    # a parameter's adjoint is a sum over every cell with terms of both
    # signs, so the FP32 rounding of the rates shows more in it
    assert np.all(perr <= 1e-3), perr
    drv.close()


def _loss_terms(torch, spec):
    gz, gzh = vertical_grid(spec.kall)
    dgz = torch.tensor(np.diff(gzh, append=gzh[-1] + (gzh[-1] - gzh[-2])), dtype=torch.float64, device="cuda")
    w = torch.zeros(spec.kall, dtype=torch.float64, device="cuda")
    w[1:spec.kall - 1] = dgz[1:spec.kall - 1]
    return w


def _loss(torch, y, w):
    p = y["precip"][0] + y["precip"][1]
    return float((p * p).sum() + (y["rhogq"][:, 1] * w[None, :, None]).sum())


def _loss_diff(torch, yp, ym, w):
    """L(yp) - L(ym) summed term by term (no cancellation against the total)."""
    pp = yp["precip"][0] + yp["precip"][1]
    pm = ym["precip"][0] + ym["precip"][1]
    return float(((pp - pm) * (pp + pm)).sum() + ((yp["rhogq"][:, 1] - ym["rhogq"][:, 1]) * w[None, :, None]).sum())


@pytest.mark.parametrize("options,variant", [(None, "standard"), (CELL_SWITCHES, "standard"), (ICE_SWITCHES, "cold")],
                         ids=["reference", "switches", "ice-switches"])
def test_gradient_against_finite_differences(options, variant):
    """The adjoint gradient of L = sum (precip)^2 + sum rhogq[QC] dz against
    central differences of the forward step.  The saturation adjustment is
    differentiated implicitly at its converged temperature, while the forward
    returns the Newton's last iterate, whose sensitivity differs from the
    root's by the iteration's contraction factor to the power of its
    iterations; the reference's mixed-phase Newton uses a coarser slope than
    the liquid one, so that case is held to 1e-5 instead of 1e-6."""
    tol = 1e-5 if options is ICE_SWITCHES else 1e-6
    torch, drv, spec, st, x0 = _setup(4096, 42, 1, 2024, variant, options)
    if options:
        # the autoconversion threshold off its default 0, where every cell
        # without ice sits on the switch of max(beta (qi - qicrt), 0) and of
        # its limiter (derivatives are checked away from the scheme's
        # threshold switches; the switched cold state has many such cells)
        drv.set_params(qicrt_saut=2e-9)
    w = _loss_terms(torch, spec)

    def forward(x):
        y = _clone(x)
        drv.mp_driver_batched(spec.lall, *[y[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
        return y

    y0 = forward(x0)
    bar = {n: torch.zeros_like(v) for n, v in x0.items()}
    bar["precip"] = 2.0 * (y0["precip"][0] + y0["precip"][1]).unsqueeze(0).expand_as(y0["precip"]).contiguous()
    bar["rhogq"][:, 1] = w[None, :, None].expand(spec.lall, spec.kall, spec.gall)
    pbar = drv.adjoint(spec.lall, _clone(x0), bar, dt=spec.dt)

    def fd(setter, h):
        xp, xm = _clone(x0), _clone(x0)
        setter(xp, +h)
        setter(xm, -h)
        return _loss_diff(torch, forward(xp), forward(xm), w) / (2 * h)

    rng = np.random.default_rng(3)
    # columns with rain reaching the surface, where the loss is sensitive
    prc = (y0["precip"][0, 0] + y0["precip"][1, 0]).abs().cpu().numpy()
    cols = rng.choice(np.argsort(prc)[-400:], 16, replace=False)
    checked = skipped = unresolved = 0
    worst = 0.0
    fields = (("tem", lambda k, g: (0, k, g), None), ("q", lambda k, g: (0, 0, k, g), 0),
              ("rhogq", lambda k, g: (0, 2, k, g), 2), ("rhog", lambda k, g: (0, k, g), None))
    for g in cols:
        for name, idx, nq in fields:
            # the level where the loss is most sensitive to this field
            gcol = bar[name][0, :, g] if nq is None else bar[name][0, nq, :, g]
            k = int(gcol[1:spec.kall - 1].abs().argmax()) + 1
            ix = idx(k, int(g))
            x = float(x0[name][ix])
            h = 1e-6 * abs(x)
            adj = float(bar[name][ix])
            if h == 0.0:   # a zero value has no relative step
                unresolved += 1
                continue

            def setter(xx, d, name=name, ix=ix):
                xx[name][ix] += d

            # rounding noise of the difference of this column's loss terms
            pcol = float((y0["precip"][0, 0, g] + y0["precip"][1, 0, g]) ** 2)
            qcol = float((y0["rhogq"][0, 1, :, g].abs() * w).sum())
            noise = 4e-16 * (pcol + qcol) / h
            if abs(adj) < 1e4 * noise:   # a 1e-6 relative step cannot resolve this derivative
                unresolved += 1
                continue
            a1, a2 = fd(setter, h), fd(setter, h / 4)
            scale = max(abs(a1), abs(adj), 1e-300)
            if abs(a1 - a2) > 1e-6 * scale:   # a switch flips between the FD points
                skipped += 1
                continue
            checked += 1
            err = abs(adj - a1) / scale
            worst = max(worst, err)
            print(f"  d L / d {name}{ix}: adjoint {adj:+.10e}  FD {a1:+.10e}  rel {err:.1e}")
            assert err <= tol, (name, ix, adj, a1)
    # the seven parameters
    Ltot = float((y0["precip"][0] + y0["precip"][1]).pow(2).sum() + (y0["rhogq"][:, 1].abs() * w[None, :, None]).sum())
    base = drv.get_params()
    for i, pn in enumerate(PARAMS):
        p0 = base[pn]
        h = 1e-6 * abs(p0) if p0 != 0 else 1e-9   # the threshold at 0: an absolute step of 1e-9 kg/kg
        if options and pn == "qicrt_saut":
            h = 1e-9
        if abs(pbar[i]) < 1e4 * 4e-16 * Ltot / h:
            unresolved += 1
            continue

        def yp(v):
            drv.set_params(**{pn: v})
            out = forward(x0)
            drv.set_params(**{pn: p0})
            return out

        y_plus, y_minus = yp(p0 + h), yp(p0 - h)
        a1 = _loss_diff(torch, y_plus, y_minus, w) / (2 * h)
        a2 = _loss_diff(torch, yp(p0 + h / 4), yp(p0 - h / 4), w) / (h / 2)
        # a kink at p0 (a threshold parameter at a value some cells sit at,
        # qicrt_saut = 0 against cells without ice) shows as differing
        # one-sided differences
        right = _loss_diff(torch, y_plus, y0, w) / h
        left = _loss_diff(torch, y0, y_minus, w) / h
        scale = max(abs(a1), abs(pbar[i]), 1e-300)
        if abs(a1 - a2) > 1e-6 * scale or abs(right - left) > 1e-4 * scale:
            skipped += 1
            print(f"  d L / d {pn}: at a switch (one-sided {left:+.6e} / {right:+.6e}), not checked")
            continue
        checked += 1
        err = abs(pbar[i] - a1) / scale
        worst = max(worst, err)
        print(f"  d L / d {pn}: adjoint {pbar[i]:+.10e}  FD {a1:+.10e}  rel {err:.1e}")
        assert err <= tol, (pn, pbar[i], a1)
    print(f"\ngradient vs FD ({variant}, {options or 'reference'}): {checked} components checked, {skipped} "
          f"next to a switch, {unresolved} below the resolution of the step, worst rel err {worst:.2e}")
    assert checked >= 20
    drv.close()


def _region_fd_check(torch, reg, gz, gzh, names, dt=60.0):
    """Adjoint parameter gradients of L on one region against central
    differences of the production step (relative step 1e-6, and 1e-6 / 4 to
    show the difference resolves the derivative), and against central
    differences of the reference algorithm (the oracle) with the same step.
    Every finite-difference point is certified by the reference's decision
    record (no switch between p - h and p + h)."""
    import _fdregions as F
    from nicam_kokkos_microphysics_gb300 import mp_init
    from nicam_kokkos_microphysics_gb300.state import regions_to_batched
    kall, gall = reg["rhog"].shape
    drv = mp_init("NSW6", gall, kall, gz, gzh, lall_max=1)
    x0 = {n: torch.from_numpy(v).cuda() for n, v in regions_to_batched([reg]).items()}
    w = torch.from_numpy(F.loss_weights(gzh)).cuda()

    def forward():
        y = _clone(x0)
        drv.mp_driver_batched(1, *[y[n] for n in ARG_NAMES], dt=dt, ct=0.0)
        return y

    y0 = forward()
    bar = {n: torch.zeros_like(v) for n, v in x0.items()}
    bar["precip"] = 2.0 * (y0["precip"][0] + y0["precip"][1]).unsqueeze(0).expand_as(y0["precip"]).contiguous()
    bar["rhogq"][:, 1] = w[None, :, None].expand(1, kall, gall)
    pbar = drv.adjoint(1, _clone(x0), bar, dt=dt)
    wn = F.loss_weights(gzh)

    def oracle_diff(a, b):
        pa, pb = a["precip"][0] + a["precip"][1], b["precip"][0] + b["precip"][1]
        return float(((pa - pb) * (pa + pb)).sum() + ((a["rhogq"][1] - b["rhogq"][1]) * wn[:, None]).sum())

    base = drv.get_params()
    rows = []
    for pn in names:
        i = PARAMS.index(pn)
        p0 = base[pn]
        h = 1e-6 * abs(p0) if p0 != 0.0 else 1e-9   # the threshold at 0: an absolute 1e-9 kg/kg
        cert = F.certify(reg, gz, gzh, pn, p0, (h, -h, h / 4, -h / 4), dt)
        assert cert["ok"], (pn, cert["per_step"])

        def at(v, pn=pn, p0=p0):
            drv.set_params(**{pn: v})
            out = forward()
            drv.set_params(**{pn: p0})
            return out

        a1 = _loss_diff(torch, at(p0 + h), at(p0 - h), w) / (2 * h)
        a2 = _loss_diff(torch, at(p0 + h / 4), at(p0 - h / 4), w) / (h / 2)
        o1 = oracle_diff(F._step(reg, gz, gzh, dt, {pn: p0 + h}), F._step(reg, gz, gzh, dt, {pn: p0 - h})) / (2 * h)
        scale = max(abs(a1), abs(pbar[i]), 1e-300)
        err, err_ref, res = abs(pbar[i] - a1) / scale, abs(pbar[i] - o1) / scale, abs(a1 - a2) / scale
        changed = sum(v.get("changed", 0) for st in cert["per_step"] for k, v in st.items() if isinstance(v, dict))
        rows.append((pn, pbar[i], a1, o1, err, err_ref, res, changed))
        print(f"  d L / d {pn:10s}: adjoint {pbar[i]:+.10e}  FD {a1:+.10e}  FD(reference) {o1:+.10e}  "
              f"rel {err:.1e} / {err_ref:.1e}  (h vs h/4 {res:.1e}; {changed} tie decisions changed)")
        assert res <= 1e-7, (pn, a1, a2)
        assert err <= 1e-6, (pn, pbar[i], a1)
        assert err_ref <= 1e-6, (pn, pbar[i], o1)
    drv.close()
    return rows


def test_parameter_gradients_against_finite_differences():
    """All seven NSW6 parameters, with the reference configuration's scheme
    switches and parameter values: the adjoint gradient of L = sum (precip)^2
    + sum rhogq[QC] dz against central differences (relative step 1e-6, the
    threshold qicrt_saut = 0 with an absolute 1e-9) of the production step and
    of the reference algorithm.  Six parameters act on L through the surface
    precipitation and are checked on columns that the step leaves without
    cloud water (the autoconversion rate on the few whose surface rain it
    feeds most); the ice-nucleation coefficient acts through the cloud water
    and is checked on cloudy columns (where the cloud water's cancellation
    noise hides the others' smaller effects).  The
    finite-difference points are certified switch-free by the reference's
    decision record (tests/_fdregions.py)."""
    torch = _torch()
    import _fdregions as F
    reg, gz, gzh = F.precipitating_region()
    rows = _region_fd_check(torch, reg, gz, gzh, ["beta_saut", "qicrt_saut", "Cr", "Cs", "Cg"])
    reg, gz, gzh = F.autoconversion_region()
    rows += _region_fd_check(torch, reg, gz, gzh, ["kk_aut"])
    reg, gz, gzh = F.cloudy_region(ncol=1024)
    rows += _region_fd_check(torch, reg, gz, gzh, ["ice_nuc"])
    assert sorted(r[0] for r in rows) == sorted(PARAMS)
    print(f"\nparameter gradients vs FD: {len(rows)} of 7 checked, worst rel err "
          f"{max(r[4] for r in rows):.2e} (production step), {max(r[5] for r in rows):.2e} (reference)")


def test_kin2kin_gradient_against_finite_differences():
    """With KIN2KIN the final momenta are the transported ones rescaled to
    carry the transported kinetic energy.  The adjoint gradient of a random
    weighted sum of the four momentum outputs against central differences of
    the forward step, in columns with falling rain, for the momenta, the
    density and the rain water, and for the fall-speed parameters."""
    torch, drv, spec, st, x0 = _setup(1024, 42, 1, 2024, "convective", KIN2KIN)
    gen = torch.Generator(device="cuda").manual_seed(9)
    mom = ("rhogvx", "rhogvy", "rhogvz", "rhogw")
    wts = {n: torch.randn(x0[n].shape, generator=gen, device="cuda", dtype=torch.float64) for n in mom}

    def forward(x):
        y = _clone(x)
        drv.mp_driver_batched(spec.lall, *[y[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
        return y

    def ldiff(yp, ym):   # L(yp) - L(ym) term by term
        return float(sum((wts[n] * (yp[n] - ym[n])).sum() for n in mom))

    y0 = forward(x0)
    bar = {n: torch.zeros_like(v) for n, v in x0.items()}
    for n in mom:
        bar[n] = wts[n].clone()
    pbar = drv.adjoint(spec.lall, _clone(x0), bar, dt=spec.dt)
    prc = (y0["precip"][0, 0] + y0["precip"][1, 0]).abs().cpu().numpy()
    cols = np.random.default_rng(4).choice(np.argsort(prc)[-200:], 12, replace=False)
    fields = (("rhogvx", lambda k, g: (0, k, g), None), ("rhogw", lambda k, g: (0, k, g), None),
              ("rhog", lambda k, g: (0, k, g), None), ("rhogq", lambda k, g: (0, 2, k, g), 2))
    checked = skipped = 0
    worst = 0.0
    for g in cols:
        for name, idx, nq in fields:
            gcol = bar[name][0, :, g] if nq is None else bar[name][0, nq, :, g]
            k = int(gcol[1:spec.kall - 1].abs().argmax()) + 1
            ix = idx(k, int(g))
            x = float(x0[name][ix])
            adj = float(bar[name][ix])
            if x == 0.0 or adj == 0.0:
                continue
            h = 1e-6 * abs(x)

            def fd(hh, name=name, ix=ix):
                xp, xm = _clone(x0), _clone(x0)
                xp[name][ix] += hh
                xm[name][ix] -= hh
                return ldiff(forward(xp), forward(xm)) / (2 * hh)

            a1, a2 = fd(h), fd(h / 4)
            scale = max(abs(a1), abs(adj), 1e-300)
            if abs(a1 - a2) > 1e-6 * scale:   # a switch flips between the FD points
                skipped += 1
                continue
            checked += 1
            err = abs(adj - a1) / scale
            worst = max(worst, err)
            print(f"  d L / d {name}{ix}: adjoint {adj:+.10e}  FD {a1:+.10e}  rel {err:.1e}")
            assert err <= 1e-6, (name, ix, adj, a1)
    base = drv.get_params()
    for pn in ("Cr", "Cs", "Cg"):
        i = PARAMS.index(pn)
        p0 = base[pn]
        h = 1e-6 * abs(p0)

        def yp(v, pn=pn, p0=p0):
            drv.set_params(**{pn: v})
            out = forward(x0)
            drv.set_params(**{pn: p0})
            return out

        a1 = ldiff(yp(p0 + h), yp(p0 - h)) / (2 * h)
        a2 = ldiff(yp(p0 + h / 4), yp(p0 - h / 4)) / (h / 2)
        scale = max(abs(a1), abs(pbar[i]), 1e-300)
        if abs(a1 - a2) > 1e-6 * scale:
            skipped += 1
            continue
        checked += 1
        err = abs(pbar[i] - a1) / scale
        worst = max(worst, err)
        print(f"  d L / d {pn}: adjoint {pbar[i]:+.10e}  FD {a1:+.10e}  rel {err:.1e}")
        assert err <= 1e-6, (pn, pbar[i], a1)
    print(f"\nKIN2KIN gradient vs FD: {checked} components checked, {skipped} next to a switch, "
          f"worst rel err {worst:.2e}")
    assert checked >= 20
    drv.close()


def _fd_ladder(fd, x):
    """Central differences fd(h) at h = 1e-3 .. 1e-6 of |x|: the value at the
    smaller step of the two neighbouring steps that agree best, and their
    relative disagreement."""
    vals = [fd(r * x) for r in (1e-3, 1e-4, 1e-5, 1e-6)]
    gaps = [abs(vals[i] - vals[i + 1]) / max(abs(vals[i + 1]), 1e-300) for i in range(3)]
    i = int(np.argmin(gaps))
    return vals[i + 1], gaps[i]


def test_qi_sediment_gradient_against_finite_differences():
    """With cloud ice sedimenting ("4WATER", mod_mp_nsw6.cpp:596-599) the
    transport carries QI as a fourth tracer with the fall speed
    Vti = -3.29 (rho qi)^0.16 (mod_mp_nsw6.cpp:1073-1075), and its surface
    flux joins the solid precipitation.  The adjoint gradient of a random
    weighted sum of the cloud-ice output and of the solid surface
    precipitation against central differences of the forward step, in the
    columns with the most ice, for the ice and snow contents, the temperature
    and the density."""
    torch, drv, spec, st, x0 = _setup(1024, 42, 1, 2024, "cold", QI_SEDIMENT)
    gen = torch.Generator(device="cuda").manual_seed(12)
    wq = torch.randn(x0["rhogq"][:, 3].shape, generator=gen, device="cuda", dtype=torch.float64)
    wp = torch.randn(x0["precip"][1].shape, generator=gen, device="cuda", dtype=torch.float64)
    # the two terms of comparable size
    sq = float(x0["rhogq"][:, 3].abs().mean())

    def forward(x):
        y = _clone(x)
        drv.mp_driver_batched(spec.lall, *[y[n] for n in ARG_NAMES], dt=spec.dt, ct=0.0)
        return y

    y0 = forward(x0)
    sp = sq / max(float(y0["precip"][1].abs().mean()), 1e-300)

    def ldiff(yp, ym):   # L(yp) - L(ym) term by term
        return float((wq * (yp["rhogq"][:, 3] - ym["rhogq"][:, 3])).sum() +
                     sp * (wp * (yp["precip"][1] - ym["precip"][1])).sum())

    bar = {n: torch.zeros_like(v) for n, v in x0.items()}
    bar["rhogq"][:, 3] = wq
    bar["precip"][1] = sp * wp
    drv.adjoint(spec.lall, _clone(x0), bar, dt=spec.dt)
    ice = x0["rhogq"][0, 3].sum(dim=0).cpu().numpy()
    cols = np.random.default_rng(6).choice(np.argsort(ice)[-200:], 12, replace=False)
    fields = (("rhogq", lambda k, g: (0, 3, k, g), 3), ("rhogq", lambda k, g: (0, 4, k, g), 4),
              ("tem", lambda k, g: (0, k, g), None), ("rhog", lambda k, g: (0, k, g), None))
    checked = skipped = 0
    worst = 0.0
    for g in cols:
        for name, idx, nq in fields:
            gcol = bar[name][0, :, g] if nq is None else bar[name][0, nq, :, g]
            k = int(gcol[1:spec.kall - 1].abs().argmax()) + 1
            ix = idx(k, int(g))
            x = float(x0[name][ix])
            adj = float(bar[name][ix])
            if x == 0.0 or adj == 0.0:
                continue

            def fd(hh, name=name, ix=ix):
                xp, xm = _clone(x0), _clone(x0)
                xp[name][ix] += hh
                xm[name][ix] -= hh
                return ldiff(forward(xp), forward(xm)) / (2 * hh)

            # a ladder of steps (relative 1e-3 .. 1e-6): where the input is
            # weakly coupled to the loss, the small steps drown in the
            # rounding of the outputs, the large ones in the curvature; the
            # estimate is the pair of neighbouring steps that agree best
            a1, spread = _fd_ladder(fd, abs(x))
            scale = max(abs(a1), abs(adj), 1e-300)
            if spread > 1e-7:   # no two steps agree: a switch flips between the FD points
                skipped += 1
                continue
            checked += 1
            err = abs(adj - a1) / scale
            worst = max(worst, err)
            print(f"  d L / d {name}{ix}: adjoint {adj:+.10e}  FD {a1:+.10e}  rel {err:.1e}")
            assert err <= 1e-6, (name, ix, adj, a1)
    print(f"\nQI sedimentation gradient vs FD: {checked} components checked, {skipped} next to a switch, "
          f"worst rel err {worst:.2e}")
    assert checked >= 24
    drv.close()


def test_window_gradient_against_finite_differences():
    """Three-step window with per-step checkpoints (FP64 forward): the gradient
    of the accumulated surface precipitation J with respect to the initial
    temperature and vapour and to all seven parameters, against term-wise
    central differences of the FP64 window (relative step 1e-6; the threshold
    qicrt_saut = 0 with an absolute 1e-9), on the precipitating region of
    tests/_fdregions.py.  Every parameter point is certified switch-free over
    the whole window by the reference's decision records; the differences with
    h and h/4 agree to 5e-7 (three steps accumulate more rounding noise than
    one)."""
    torch = _torch()
    import _fdregions as F
    from nicam_kokkos_microphysics_gb300 import mp_init
    from nicam_kokkos_microphysics_gb300.state import regions_to_batched
    from nicam_kokkos_microphysics_gb300.window import window_gradient
    reg, gz, gzh = F.precipitating_region()
    kall, gall = reg["rhog"].shape
    dt, nsteps = 60.0, 3
    drv = mp_init("NSW6", gall, kall, gz, gzh, lall_max=1)
    x0 = {n: torch.from_numpy(v).cuda() for n, v in regions_to_batched([reg]).items()}
    res = window_gradient(drv, 1, x0, nsteps, dt, precision="fp64")
    bar, pbar = res["grad"], res["dparams"]

    def precip_series(x):
        y = _clone(x)
        out = []
        for _ in range(nsteps):
            drv.mp_driver_batched(1, *[y[n] for n in ARG_NAMES], dt=dt, ct=0.0)
            out.append((y["precip"][0] + y["precip"][1]).clone())
        return out

    def dJ(sp, sm):
        return float(sum((a - b).sum() for a, b in zip(sp, sm))) * dt

    y1 = _clone(x0)
    drv.mp_driver_batched(1, *[y1[n] for n in ARG_NAMES], dt=dt, ct=0.0)
    prc = (y1["precip"][0, 0] + y1["precip"][1, 0]).abs().cpu().numpy()
    rng = np.random.default_rng(8)
    checked = skipped = 0
    worst = 0.0
    for g in rng.choice(np.argsort(prc)[-48:], 8, replace=False):
        for name, nq in (("tem", None), ("q", 0)):
            gcol = bar[name][0, :, g] if nq is None else bar[name][0, nq, :, g]
            k = int(gcol[1:kall - 1].abs().argmax()) + 1   # the most sensitive level
            ix = (0, k, int(g)) if nq is None else (0, nq, k, int(g))
            h = 1e-6 * abs(float(x0[name][ix]))
            vals = []
            for hh in (h, h / 4):
                xp, xm = _clone(x0), _clone(x0)
                xp[name][ix] += hh
                xm[name][ix] -= hh
                vals.append(dJ(precip_series(xp), precip_series(xm)) / (2 * hh))
            adj = float(bar[name][ix])
            scale = max(abs(vals[0]), abs(adj), 1e-300)
            # a derivative 1e-10 below the field's largest is rounding noise
            # of the adjoint, not a sensitivity a 1e-6 step resolves
            if abs(vals[0] - vals[1]) > 1e-6 * scale or scale < 1e-10 * float(bar[name].abs().max()):
                skipped += 1
                continue
            checked += 1
            err = abs(adj - vals[0]) / scale
            worst = max(worst, err)
            print(f"  window dJ/d{name}{ix}: adjoint {adj:+.10e} FD {vals[0]:+.10e} rel {err:.1e}")
            assert err <= 1e-6, (name, ix, adj, vals[0])
    base = drv.get_params()
    for i, pn in enumerate(PARAMS):
        p0 = base[pn]
        h = 1e-6 * abs(p0) if p0 != 0.0 else 1e-9
        cert = F.certify_window(reg, gz, gzh, pn, p0, (h, -h, h / 4, -h / 4), nsteps, dt)
        assert cert["ok"], (pn, cert["per_step"])

        def series(v, pn=pn, p0=p0):
            drv.set_params(**{pn: v})
            out = precip_series(x0)
            drv.set_params(**{pn: p0})
            return out

        a1 = dJ(series(p0 + h), series(p0 - h)) / (2 * h)
        a2 = dJ(series(p0 + h / 4), series(p0 - h / 4)) / (h / 2)
        scale = max(abs(a1), abs(pbar[i]), 1e-300)
        err, resol = abs(pbar[i] - a1) / scale, abs(a1 - a2) / scale
        worst = max(worst, err)
        print(f"  window dJ/d{pn:10s}: adjoint {pbar[i]:+.10e} FD {a1:+.10e} rel {err:.1e} (h vs h/4 {resol:.1e})")
        assert resol <= 5e-7, (pn, a1, a2)
        assert err <= 1e-6, (pn, pbar[i], a1)
        checked += 1
    print(f"\nwindow gradient: {checked} checked (7 parameters), {skipped} state points skipped, "
          f"worst rel err {worst:.2e}; J = {res['J']:.6e}; forward {res['t_forward'] * 1e3:.1f} ms, "
          f"adjoint {res['t_adjoint'] * 1e3:.1f} ms")
    assert checked >= 6 + len(PARAMS)
    drv.close()


def test_window_gradient_mixed_forward_against_fp64_forward():
    """The configured 12-step window runs the mixed-precision forward with FP64
    adjoint accumulation.  Its gradient (the adjoint of the mixed step around
    the mixed forward's checkpoints: FP32 rate adjoints, FP64 budgets, column
    stages and accumulation), and the same window's with the FP64 adjoint
    around the same checkpoints, against the window with the FP64 forward,
    on a 16900-column region, reported per parameter and for the gradient
    fields of the initial temperature and vapour.  They are gradients of
    trajectories that part by the mixed step's errors (about 1e-6): where a
    cell of one trajectory sits on the other side of a limiter or threshold
    switch than in the other, its derivative differs outright, so the
    parameters that act through such switches (the ice autoconversion rate
    and threshold) differ by a few per cent, the others by 1e-6 to 1e-4, the
    fields by a few 1e-3 (relative L2)."""
    torch, drv, spec, st, x0 = _setup(16900, 42, 1, 1005, "standard")
    from nicam_kokkos_microphysics_gb300.window import window_gradient
    r64 = window_gradient(drv, 1, x0, 12, spec.dt, precision="fp64")
    for adjoint in ("mixed", "fp64"):
        rmx = window_gradient(drv, 1, x0, 12, spec.dt, precision="mixed", adjoint=adjoint)
        print(f"\n12-step window, {adjoint} adjoint: J fp64 {r64['J']:.10e} mixed {rmx['J']:.10e} "
              f"(rel {abs(rmx['J'] - r64['J']) / abs(r64['J']):.2e})")
        worst = {}
        for i, pn in enumerate(PARAMS):
            a, b = rmx["dparams"][i], r64["dparams"][i]
            rel = abs(a - b) / max(abs(b), 1e-300)
            worst[pn] = rel
            print(f"  dJ/d{pn:10s}: fp64 forward {b:+.10e}  mixed forward {a:+.10e}  rel {rel:.2e}")
        for name, sl in (("tem", (slice(None),)), ("q[QV]", (slice(None), 0))):
            f = "tem" if name == "tem" else "q"
            a, b = rmx["grad"][f][sl], r64["grad"][f][sl]
            l2 = float((a - b).norm() / b.norm())
            mx = float((a - b).abs().max() / b.abs().max())
            worst[name] = l2
            print(f"  dJ/d{name} field: relative L2 difference {l2:.2e}, field-normalised max {mx:.2e}")
        for pn in ("Cr", "Cs", "Cg", "ice_nuc", "kk_aut"):
            assert worst[pn] <= 1e-3, (adjoint, pn, worst[pn])
        for pn in ("beta_saut", "qicrt_saut"):
            assert worst[pn] <= 0.1, (adjoint, pn, worst[pn])
        assert worst["tem"] <= 1e-2 and worst["q[QV]"] <= 1e-2, (adjoint, worst)
    drv.close()

"""The finite-difference points of the parameter-gradient checks, certified on
the CPU with the reference algorithm (no GPU needed):

* the decision record (oracle/branchsig.cpp) is reproducible, and a parameter
  step that moves a departure cell shows as a change at a site the adjoint
  holds fixed;
* on the precipitating region (tests/_fdregions.py), for six parameters, the
  points p +- h and p +- h/4 (relative h = 1e-6) take the reference's
  decisions, and the central differences of the reference step with h and h/4
  agree to 1e-7: the difference resolves the derivative; the same holds for
  the autoconversion rate on the autoconversion region and for the
  ice-nucleation coefficient on the cloudy region;
* over a three-step window on the precipitating region, all seven.
"""
from __future__ import annotations

import numpy as np
import pytest

import _fdregions as F

PARAMS = ["beta_saut", "qicrt_saut", "Cr", "Cs", "Cg", "ice_nuc", "kk_aut"]


@pytest.fixture(scope="module")
def oracle():
    from oracle import restatement
    restatement.build_branchsig()
    return restatement


@pytest.fixture(scope="module")
def precipitating():
    return F.precipitating_region()


def _step_h(p0):
    return 1e-6 * abs(p0) if p0 != 0.0 else 1e-9


def _loss_diff(a, b, w):
    pa, pb = a["precip"][0] + a["precip"][1], b["precip"][0] + b["precip"][1]
    return float(((pa - pb) * (pa + pb)).sum() + ((a["rhogq"][1] - b["rhogq"][1]) * w[:, None]).sum())


def test_decision_record_is_reproducible_and_sees_departure_cells(oracle, precipitating):
    reg, gz, gzh = precipitating
    r0 = oracle.branch_record(reg, gz, gzh, 60.0)
    r1 = oracle.branch_record(reg, gz, gzh, 60.0)
    ch = oracle.decision_changes(r0, r1)
    assert ch is not None and all(c["changed"] == 0 for c in ch.values())
    assert np.array_equal(r0["val"], r1["val"])
    # rain falling twice as fast crosses level boundaries: the departure cells
    # (or the search over them) change
    cr = oracle.default_params()["Cr"]
    cert = F.certify(reg, gz, gzh, "Cr", cr, (cr,))
    assert not cert["ok"]


@pytest.mark.parametrize("name", ["beta_saut", "qicrt_saut", "Cr", "Cs", "Cg"])
def test_precipitating_region_points_are_switch_free(oracle, precipitating, name):
    reg, gz, gzh = precipitating
    p0 = oracle.default_params()[name]
    h = _step_h(p0)
    cert = F.certify(reg, gz, gzh, name, p0, (h, -h, h / 4, -h / 4))
    assert cert["ok"], cert["per_step"]
    w = F.loss_weights(gzh)
    f = lambda d: F._step(reg, gz, gzh, params={name: p0 + d})  # noqa: E731
    a1 = _loss_diff(f(h), f(-h), w) / (2 * h)
    a2 = _loss_diff(f(h / 4), f(-h / 4), w) / (h / 2)
    assert a1 != 0.0
    assert abs(a1 - a2) <= 1e-7 * abs(a1), (a1, a2)


@pytest.mark.parametrize("name", ["kk_aut", "ice_nuc"])
def test_autoconversion_and_cloudy_region_points_are_switch_free(oracle, name):
    reg, gz, gzh = F.autoconversion_region() if name == "kk_aut" else F.cloudy_region(ncol=1024)
    p0 = oracle.default_params()[name]
    h = _step_h(p0)
    cert = F.certify(reg, gz, gzh, name, p0, (h, -h, h / 4, -h / 4))
    assert cert["ok"], cert["per_step"]
    w = F.loss_weights(gzh)
    f = lambda d: F._step(reg, gz, gzh, params={name: p0 + d})  # noqa: E731
    a1 = _loss_diff(f(h), f(-h), w) / (2 * h)
    a2 = _loss_diff(f(h / 4), f(-h / 4), w) / (h / 2)
    assert a1 != 0.0
    assert abs(a1 - a2) <= 1e-7 * abs(a1), (a1, a2)


@pytest.mark.parametrize("name", PARAMS)
def test_window_points_are_switch_free(oracle, precipitating, name):
    reg, gz, gzh = precipitating
    p0 = oracle.default_params()[name]
    h = _step_h(p0)
    cert = F.certify_window(reg, gz, gzh, name, p0, (h, -h), 3)
    assert cert["ok"], cert["per_step"]

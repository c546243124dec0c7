"""Iteration checkpoints in the reference's format (SaveIterChpoint / LoadIterChpoint, src/iterative.c:165-278), oracle
side: the reference's own chp.0 files for all seven methods (tests/golden/chpoint, made by make_chpoint.py) against
the oracle's restatement. The oracle's state after the same iterations equals the reference's file field by field
(rounding only), and the oracle resumed from the reference's file continues with the reference's residual history
and cross sections."""
import json
import os

import numpy as np
import pytest

from conftest import ROOT
from helpers import oracle_for, oracle_solve, parse_chpoint, setup_for

GOLD = os.path.join(ROOT, "tests", "golden")
CHP = json.load(open(os.path.join(GOLD, "reference_chpoint.json")))
CASES = CHP["cases"]


def ref_file(method):
    return open(os.path.join(GOLD, "chpoint", method + ".chp"), "rb").read()


def setup():
    g = CHP["setup"]
    return setup_for(dict(grid=g["grid"], m=complex(*g["m"])))


def compare_state(got, want, method, tol):
    """header exact where it is an integer, the rest relative to tol; vectors by relative L2 norm"""
    hg, sg, vg = parse_chpoint(got, method)
    hw, sw, vw = parse_chpoint(want, method)
    assert len(got) == len(want)
    assert hg[:4] == hw[:4], (hg[:4], hw[:4])  # ind_m, nRows, niter, counter
    for a, b in zip(hg[4:], hw[4:]):  # inprodR, prev_err, resid_scale
        assert abs(a - b) <= tol * abs(b), (a, b)
    for a, b in zip(sg, sw):
        assert abs(a - b) <= tol * max(abs(b), 1e-300), (method, sg, sw)
    for k, (a, b) in enumerate(zip(vg, vw)):
        assert np.linalg.norm(a - b) <= tol * np.linalg.norm(b), (method, k)


def test_fixtures_are_the_reference_format():
    s = setup()
    for c in CASES:
        raw = ref_file(c["method"])
        assert len(raw) == c["chp_bytes"]
        head, sc, vec = parse_chpoint(raw, c["method"])
        assert head[1] == 3 * s.n == 3 * c["ndip"]
        assert head[2] == len(c["resid_before"]) == c["first_loaded"]   # niter = iterations done + 1
        assert abs(np.sqrt(head[6] * head[4]) / min(c["resid_before"]) - 1) < 1e-9  # |r| of the best iterate


@pytest.mark.parametrize("c", CASES, ids=[c["method"] for c in CASES])
def test_oracle_state_matches_reference_file(c):
    s = setup()
    o = oracle_for(s)
    nsave = len(c["resid_before"]) - 1
    r = oracle_solve(o, s, 0, method=c["method"], eps=CHP["eps"], maxiter=nsave, chp_save=True)
    np.testing.assert_allclose(r["resid"], c["resid_before"], rtol=1e-9)
    # measured: every field within 2e-12 of the reference's (FFT rounding), vectors swapped by niter parity where
    # the method swaps pointers (QMR_CS, CSYM)
    compare_state(r["chp"], ref_file(c["method"]), c["method"], 1e-10)
    o.close()


@pytest.mark.parametrize("c", CASES, ids=[c["method"] for c in CASES])
def test_oracle_resumes_reference_file(c):
    s = setup()
    o = oracle_for(s)
    r = oracle_solve(o, s, 0, method=c["method"], eps=CHP["eps"], chp_in=ref_file(c["method"]))
    want = np.array(c["resid_after"])
    assert r["niter"] == c["first_loaded"] - 1 + len(want)
    assert abs(r["resid"][0] / c["resid_before"][-1] - 1) < 1e-9   # prev_err restored
    np.testing.assert_allclose(r["resid"][1:], want, rtol=1e-9)
    for q in ("Cext", "Cabs"):
        assert abs(r[q] / c["cross"][q] - 1) < 6e-10, (q, r[q], c["cross"][q])
    o.close()


def test_oracle_rejects_other_method_and_size():
    s = setup()
    o = oracle_for(s)
    with pytest.raises(ValueError):
        oracle_solve(o, s, 0, method="bicgstab", chp_in=ref_file("qmr"))
    with pytest.raises(ValueError):
        oracle_solve(o, s, 0, method="qmr", chp_in=ref_file("qmr")[:-16])
    with pytest.raises(ValueError):
        oracle_solve(o, s, 0, method="qmr", chp_in=ref_file("qmr") + b"\0")
    o.close()

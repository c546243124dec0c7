"""Krylov breakdown as the reference detects it (QMR_CS |vT.v|/(v.v) < 1e-10, iterative.c:958-960; BiCG_CS
|rT.r|/(r.r) < 1e-10, :559-560; QMR_CS_2 |vT.v| < 1e-10, :1086-1089), made by the input, not by a fault: an incident
field E = (e, i e, 0) per dipole gives b = S.E with bT.b = 0 (the bilinear form of these complex-symmetric methods),
so the methods break down at their first step while the Hermitian norm |b| stays large. The GPU reports the
breakdown for that right-hand side, stops it, and keeps solving the other right-hand side of the same batch exactly
as it would alone; the oracle reports the same breakdown."""
import numpy as np
import pytest

from helpers import case, oracle_for, rel, setup_for

METHODS = ["qmr", "bicg", "qmr2"]


def isotropic_null_field(s):
    """E = (e, i e, 0) with e the x component of the Y-polarised plane wave's phase: bT.b = 0 for isotropic cc"""
    e = np.exp(1j * s.wavenum * s.gridspace * s.pos[:, 2].astype(float))
    E = np.zeros((s.n, 3), np.complex128)
    E[:, 0] = e
    E[:, 1] = 1j * e
    return E.reshape(-1)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("method", METHODS)
def test_breakdown_reported_and_isolated(method, prec):
    import adda_gb300 as A
    s = setup_for(case("mgn")["setup"])
    ctx = A.Context.from_setup(s, nrhs_max=2)
    bad = isotropic_null_field(s)
    both = ctx.solve(np.stack([bad, s.einc[1]]), method=method, prec=prec, eps=1e-8, init="zero")
    assert both["stats"][0]["status"] == "breakdown", both["stats"][0]
    assert both["stats"][1]["status"] == "ok", both["stats"][1]
    # the healthy RHS of the batch is unaffected: the same iterations and solution as the same RHS solved alone
    alone = ctx.solve(np.stack([s.einc[0], s.einc[1]]), method=method, prec=prec, eps=1e-8, init="zero")
    assert both["stats"][1]["niter"] == alone["stats"][1]["niter"]
    assert rel(both["x"][1], alone["x"][1]) < 1e-12
    assert np.all(np.isfinite(both["x"][1]))


@pytest.mark.parametrize("method", METHODS)
def test_oracle_reports_the_same_breakdown(method):
    from oracle import oracle as O
    s = setup_for(case("mgn")["setup"])
    o = oracle_for(s)
    o.set_cc(s.cc[0].reshape(1, 3))
    m = {"qmr": O.QMR_CS, "bicg": O.BICG_CS, "qmr2": O.QMR_CS_2}[method]
    r = o.solve(isotropic_null_field(s), method=m, eps=1e-8, init_field=O.IF_ZERO)
    assert r["status"] == 1 and r["niter"] == 0, (r["status"], r["niter"])
    # a method with Hermitian products (BiCGStab: r.r~*) does not break down on the same field and converges
    r2 = o.solve(isotropic_null_field(s), method=O.BICGSTAB, eps=1e-8, init_field=O.IF_ZERO)
    assert r2["status"] == 0 and r2["niter"] > 0
    o.close()

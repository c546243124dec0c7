"""Csca and the asymmetry vector (-Csca -asym): the scattered field on the alldir grid (ScanIntegrParms / CalcAlldir,
src/crosssec.c:233-307,991-1050) integrated by the two-level Romberg scheme (Romberg2D, src/Romberg.c:175-533;
ScaCross / AsymParm_x,y,z, crosssec.c:1116-1260). Checked against reference runs with the default grid, an adaptive
one (eps > 0) and a partial, non-periodic one: the oracle's integrals (CPU) to the printed digits, the library's
host Romberg against the oracle's on the same values, and the GPU's integrals (C ABI) against both."""
import numpy as np
import pytest

from helpers import golden, oracle_for, oracle_solve, setup_for, solver_opts

CASES = [c for c in golden()["cases"] if "alldir" in c["setup"]]
KINDS = {"default": ((0, 180, 2, 6, 0, False, False), (0, 360, 2, 5, 0, True, True)),
         "adapt": ((0, 180, 3, 7, 1e-3, False, False), (0, 360, 2, 5, 1e-4, True, True)),
         "part": ((30, 150, 2, 4, 0, False, False), (0, 180, 1, 3, 0, False, False))}


def parms_of(kind):
    return tuple(dict(min=float(a), max=float(b), Jmin=c, Jmax=d, eps=e, equiv=f, periodic=g)
                 for a, b, c, d, e, f, g in KINDS[kind])


def check(csca, cg, want, tol):
    assert abs(csca / want["Csca"] - 1) < tol, (csca, want["Csca"])
    scale = np.linalg.norm(want["Csca.g"])
    assert np.linalg.norm(np.array(cg) - want["Csca.g"]) < tol * scale + 1e-12 * want["Csca"], (cg, want["Csca.g"])


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_oracle_integrals_match_reference(c):
    from oracle import oracle as O
    s = setup_for(c["setup"])
    o = oracle_for(s)
    parms = parms_of(c["setup"]["alldir"])
    for r, pol in enumerate("YX"):
        res = oracle_solve(o, s, r, **solver_opts(c["setup"]))
        csca, cg = O.scattering_integrals(o, res["p"], s.prop, s.incpol[1], s.incpol[0], s.wavenum, parms)
        # converged solutions (eps = 1e-10): the printed 10 digits
        check(csca, cg, c["cross"][pol], 2e-9)
    o.close()


@pytest.mark.parametrize("kind", list(KINDS))
def test_library_romberg_matches_oracle(kind):
    """the library's host Romberg2D and grid against the oracle's restatement on random smooth values"""
    import adda_gb300 as A
    from oracle import oracle as O
    parms = parms_of(kind)
    th, ph = A.integr_points(parms[0], True), A.integr_points(parms[1], False)
    np.testing.assert_allclose(th, O.alldir_angles(parms[0], True), rtol=0, atol=1e-12)
    np.testing.assert_allclose(ph, O.alldir_angles(parms[1], False), rtol=0, atol=1e-12)
    rng = np.random.default_rng(3)
    t, p = np.deg2rad(th)[:, None], np.deg2rad(ph)[None, :]
    for dim in (1, 3):
        vals = np.stack([np.exp(np.cos(t) * rng.uniform(0.5, 2)) * (1.2 + np.sin(p + rng.uniform(0, 6)))
                         for _ in range(dim)], axis=2)
        np.testing.assert_allclose(A.romberg2d(parms, vals), O.romberg2d(parms, vals), rtol=1e-14)


def test_romberg_exact_on_polynomials():
    """Romberg with Richardson extrapolation integrates low polynomials in cos(theta) exactly; the periodic
    trapezoid rule integrates trigonometric polynomials of low order exactly"""
    import adda_gb300 as A
    parms = parms_of("default")
    th, ph = A.integr_points(parms[0], True), A.integr_points(parms[1], False)
    x = np.cos(np.deg2rad(th))[:, None]
    p = np.deg2rad(ph)[None, :]
    vals = (1 + 3 * x ** 2 + x ** 5) * (2 + np.cos(3 * p))
    # average over x in [-1,1] of 1 + 3x^2 + x^5 is 2, over phi of 2 + cos(3 phi) is 2
    assert abs(A.romberg2d(parms, vals[:, :, None])[0] - 4) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_gpu_integrals(c):
    import adda_gb300 as A
    from oracle import oracle as O
    s = setup_for(c["setup"])
    ctx = A.Context.from_setup(s, nrhs_max=2)
    opts = solver_opts(c["setup"])
    res = ctx.solve(np.stack(s.einc), prec="fp64", **opts)
    parms = parms_of(c["setup"]["alldir"])
    csca, cg = ctx.scattering_integrals(2, s.prop, s.incpol[1], s.incpol[0], parms)
    o = oracle_for(s)
    for r, pol in enumerate("YX"):
        # GPU fields + host Romberg against the oracle's fields + Romberg on the same polarisation
        oc, og = O.scattering_integrals(o, res["p"][r], s.prop, s.incpol[1], s.incpol[0], s.wavenum, parms)
        assert abs(csca[r] / oc - 1) < 1e-12
        assert np.linalg.norm(cg[r] - og) < 1e-12 * (np.linalg.norm(og) + oc)
        # and against the reference's printed values (converged solves)
        check(csca[r], cg[r], c["cross"][pol], 1e-8)
    o.close()

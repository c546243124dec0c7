"""The oracle (CPU restatement of the hot path) against the reference's own outputs: the published sample run and
the reference build run on command lines from its differential test suite (tests/golden/reference_runs.json)."""
import numpy as np
import pytest

from helpers import golden, oracle_for, oracle_solve, setup_for, solver_opts

CASES = golden()["cases"]


def close10(a, b, floor):
    """agreement to the 10 significant digits the reference prints (%.10g), with an absolute floor for values that
    are rounding noise (Cabs of a non-absorbing particle)"""
    return abs(a - b) <= max(6e-10 * abs(b), floor)


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_inputs_match_reference(c):
    s = setup_for(c["setup"])
    assert s.n == c["ndip"]
    assert list(s.box) == c["box"]
    assert list(s.grid) == c["grid"]
    cc = [complex(*v) for v in c["cc"]]
    # CoupleConstant printed once (isotropic, same for both polarisations) or once per polarisation
    for i, v in enumerate(cc):
        got = s.cc[min(i, 1)][0]
        assert abs(got - v) <= 6e-10 * abs(v)
    # anisotropic prescriptions (cldr, so): the three diagonal components
    for i, v3 in enumerate(c.get("cc3", [])):
        for a, v in enumerate(v3):
            got = s.cc[min(i, 1)][a]
            assert abs(got - complex(*v)) <= 6e-10 * abs(complex(*v))


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_solve_matches_reference(c):
    s = setup_for(c["setup"])
    o = oracle_for(s)
    opts = solver_opts(c["setup"])
    for pi, pol in enumerate("YX"):
        r = oracle_solve(o, s, pi, **opts)
        ref_hist = np.array(c["resid"][pol])
        # WKB start on the 16^3 m=1.5 sphere: the reference's own two polarisations (the same problem, the particle
        # being symmetric under x<->y) start with identical histories and stop after 45 and 42 iterations with Cext
        # 1.0e-6 apart; the oracle follows each history to 1e-10 until the residual reaches 1e-2 and then drifts the
        # same way, so the iteration count gets 10% and Cext the reference's own 1e-6 spread (3e-6)
        wkb_amp = c["setup"].get("init") == "wkb" and c["ndip"] > 1000
        if wkb_amp:
            assert abs(r["niter"] - (len(ref_hist) - 1)) <= 0.1 * len(ref_hist), (pol, r["niter"], len(ref_hist))
            n = min(len(ref_hist), len(r["resid"]))
            early = ref_hist[:n] > 1e-2
            np.testing.assert_allclose(r["resid"][:n][early], ref_hist[:n][early], rtol=1e-8)
            for q in ("Cext", "Cabs"):
                want = c["cross"][pol][q]
                assert abs(r[q] - want) <= max(3e-6 * abs(want), 1e-12), (q, r[q], want)
            continue
        assert r["niter"] == len(ref_hist) - 1, (pol, r["niter"], len(ref_hist) - 1)
        # RE_ values are printed with 11 significant digits; rounding differences between two FFT call orders grow
        # by about 10x per iteration in BiCGStab and CGNR (QMR_CS, BiCG_CS and CSYM are far tamer: measured, they
        # follow the reference to 1e-8 over the whole history), so for those two the history is compared while the
        # residual is above 1e-3 (BiCGStab) or 1e-1 (CGNR, whose first 1e-8 difference appears at 0.05) and the
        # cross sections with a method-dependent bar
        it = c["setup"].get("iter", "qmr")
        # FCD on the 16^3 sphere: the (measured) history difference grows from 1e-11 at iteration 10 to 1e-8 at
        # iteration 24 (residual 6e-3) -- the same rounding amplification, with equal iteration counts
        fcd = c["setup"].get("interaction") == "fcd" and c["ndip"] > 1000
        early = ref_hist > {"bicgstab": 1e-3, "cgnr": 1e-1}.get(it, 1e-2 if fcd else 0)
        np.testing.assert_allclose(r["resid"][early], ref_hist[early], rtol=1e-8)
        np.testing.assert_allclose(r["resid"], ref_hist, rtol=0.25 if (it == "cgnr" or fcd) else 2e-2)
        for q in ("Cext", "Cabs"):
            want = c["cross"][pol][q]
            if it == "bicgstab":
                assert abs(r[q] - want) <= max(2e-7 * abs(want), 1e-12), (q, r[q], want)
            elif it == "cgnr":
                assert abs(r[q] - want) <= max(1e-8 * abs(want), 1e-12), (q, r[q], want)
            elif fcd:
                assert abs(r[q] - want) <= max(1e-7 * abs(want), 1e-12), (q, r[q], want)
            else:
                assert close10(r[q], want, 1e-12), (q, r[q], want)
    o.close()


def test_published_sample():
    """sample/run000_sphere_g16_m1.5 (ADDA v1.3b4, Windows, FFTW3): Cext 135.0449047 after 22 QMR iterations.
    The spread between FFT implementations at eps=1e-5 is a few 1e-9 (the manual prints 135.0449041)."""
    smp = golden()["sample"]
    c = [x for x in CASES if x["name"] == "sample_default"][0]
    s = setup_for(c["setup"])
    assert abs(s.cc[0][0] - complex(0.005259037197, 1.843854148e-05)) < 1e-12
    o = oracle_for(s)
    r = oracle_solve(o, s, 0)
    assert r["niter"] == smp["niter_Y"]
    np.testing.assert_allclose(r["resid"][:5], smp["resid_Y_first"], rtol=1e-9)
    assert abs(r["Cext"] / smp["Cext_Y"] - 1) < 1e-8
    assert abs(r["Cabs"]) < 1e-14

"""Surface mode on the CPU: a particle near a substrate (-surf h msub | -surf h inf, -int_surf img|som) pinned on the
reference's own runs (tests/golden/reference_surface.json, made by tests/golden/make_surface.py):

- the product's incident field near the substrate (adda_gb300_plane_wave_surf, GenerateB.c:96-140,257-323) equals
  the reference's -store_beam output for beams from above, from below and onto a perfect reflector;
- the oracle's surface path (reflected Green's tensor, R matrix, the reflected part of the matvec, the general-beam
  Cext) solved to the reference's -eps 10 gives the reference's Cext and Cabs for both polarisations, with the
  image-dipole relation and with the Sommerfeld integrals of the reference's own somnec (golden tables)."""
import json
import os

import numpy as np
import pytest

from helpers import oracle_for, oracle_solve

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "reference_surface.json")))
CASES = GOLD["cases"]


def surface_setup(c):
    import adda_gb300 as A
    st = dict(c["setup"])
    st["m"] = complex(*st["m"])
    msub = None if c["msub"] is None else complex(*c["msub"])
    table = None
    if c["relation"] == "som":
        table = np.load(os.path.join(HERE, "golden", "som_%s.npy" % c["name"]))
    return A.Setup(prop=c["prop"], surface=dict(h=c["hsub"], msub=msub, relation=c["relation"], table=table), **st)


@pytest.mark.parametrize("c", [c for c in CASES if "beam_Y" in c], ids=lambda c: c["name"])
def test_surface_beam_matches_reference(c):
    s = surface_setup(c)
    for k, pol in enumerate(("Y", "X")):
        ref = np.array(c["beam_" + pol]).view(np.complex128)
        got = s.einc[k]
        assert got.shape == ref.shape
        # the reference prints 10 significant digits
        assert np.max(np.abs(got - ref)) < 2e-9 * max(1.0, np.max(np.abs(ref))), (c["name"], pol)


@pytest.mark.parametrize("c", CASES, ids=lambda c: c["name"])
def test_oracle_surface_cross_sections_match_reference(c):
    s = surface_setup(c)
    o = oracle_for(s)
    iters = 0
    for k, pol in enumerate(("Y", "X")):
        r = oracle_solve(o, s, k, eps=1e-10)
        iters += r["niter"]
        ce, ca = o.cross_beam(r["p"], s.einc[k], s.inc_scale)
        assert abs(ce / c["Cext_" + pol] - 1) < 3e-9, (c["name"], pol, ce, c["Cext_" + pol])
        assert abs(ca / c["Cabs_" + pol] - 1) < 3e-9, (c["name"], pol, ca, c["Cabs_" + pol])
    assert iters == c["iterations_total"]


def test_surface_setup_validation():
    import adda_gb300 as A
    with pytest.raises(A.AddaError):   # a perfect reflector lit from below
        A.Setup(grid=8, m=1.5, surface=dict(h=2.0, msub=None))
    with pytest.raises(A.AddaError):   # propagation along the surface
        A.Setup(grid=8, m=1.5, prop=[1, 0, 0], surface=dict(h=2.0, msub=2.0, relation="img"))

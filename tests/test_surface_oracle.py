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


@pytest.mark.parametrize("name", ["img_above", "som_above", "img_ell10"])
def test_oracle_surface_operator_is_complex_symmetric(name):
    """reciprocity: the reflected tensor satisfies GR(-rho, zs) = GR(rho, zs)^T, so A = I + S(D+R)S stays complex
    symmetric (y.(A x) = x.(A y) without conjugation) -- what the solvers' bilinear forms and the her folding rely on"""
    c = [c for c in CASES if c["name"] == name][0]
    s = surface_setup(c)
    o = oracle_for(s)
    o.set_cc(s.cc[0].reshape(1, 3))
    rng = np.random.default_rng(5)
    x = rng.standard_normal(3 * s.n) + 1j * rng.standard_normal(3 * s.n)
    y = rng.standard_normal(3 * s.n) + 1j * rng.standard_normal(3 * s.n)
    ax, _ = o.matvec(x)
    ay, _ = o.matvec(y)
    assert abs(np.dot(y, ax) - np.dot(x, ay)) < 1e-12 * abs(np.dot(y, ax))
    # and her = conj(A conj(.)) for a complex-symmetric A
    ah, _ = o.matvec(x, her=True)
    ac, _ = o.matvec(np.conj(x))
    assert np.linalg.norm(ah - np.conj(ac)) < 1e-13 * np.linalg.norm(ah)


def test_oracle_rmatrix_matches_numpy_construction():
    """InitRmatrix (fft.c:818-887) rebuilt with numpy from the image-relation tensor: GR on the (i, j>=0, k) grid,
    mirrored to negative y with the xy/yz parity, heights at z = k, 3-D FFT, -1/Ngrid, y <= gY/2 kept"""
    c = [c for c in CASES if c["name"] == "img_ell10"][0]
    s = surface_setup(c)
    bX, bY, bZ = s.box
    gX, gY, gZ = s.grid
    k, j, i = np.meshgrid(np.arange(2 * bZ - 1), np.arange(bY), np.arange(1 - bX, bX), indexing="ij")
    q = np.stack([i, j, k + s.surface["zsum_shift"]], -1).astype(float)
    rr = np.sqrt((q ** 2).sum(-1))
    v = q / rr[..., None]
    qm = np.stack([v[..., 0] ** 2, v[..., 0] * v[..., 1], v[..., 0] * v[..., 2], v[..., 1] ** 2,
                   v[..., 1] * v[..., 2], v[..., 2] ** 2], -1)
    rr = rr * s.gridspace
    kr = s.wavenum * rr
    m = s.surface["msub"]
    scale = ((1 - m * m) / (1 + m * m) * np.exp(1j * kr) / rr ** 3)[..., None]
    t1, t2, t3 = (3 - kr ** 2)[..., None], (-3 * kr)[..., None], (kr ** 2 - 1)[..., None]
    diag = np.array([1, 0, 0, 1, 0, 1], bool)
    g = np.where(diag, (t1 * qm + t3) + 1j * (kr[..., None] + t2 * qm), (t1 + 1j * t2) * qm) * scale
    g[..., [2, 4, 5]] *= -1                                    # [k][j][i + bX - 1][6]
    full = np.zeros((gX, gY, gZ, 6), np.complex128)
    for ii in range(1 - bX, bX):
        sl = np.transpose(g[:, :, ii + bX - 1, :], (1, 0, 2))  # [j][k][6]
        full[ii % gX, :bY, :2 * bZ - 1] = sl
        sign = np.array([1, -1, 1, 1, -1, 1])
        full[ii % gX, gY - np.arange(1, bY), :2 * bZ - 1] = sl[1:] * sign
    rf = -np.fft.fftn(full, axes=(0, 1, 2)) / (gX * gY * gZ)
    want = np.transpose(rf[:, :gY // 2 + 1, :, :], (0, 2, 1, 3)).reshape(-1)  # [x][z][y<gY/2+1][6]
    got = oracle_for(s).rmatrix()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12


def test_substrate_of_index_one_vanishes():
    """msub = 1: no reflected wave from above, full transmission from below (the beam is the free plane wave), and a
    zero reflection coefficient (the operator is the free-space one)"""
    import adda_gb300 as A
    for prop in ([1, 2, -3], [0.3, -0.2, 1]):
        s = A.Setup(grid=8, m=1.5 + 0.1j, prop=prop, surface=dict(h=2.0, msub=1.0, relation="img"))
        free = A.Setup(grid=8, m=1.5 + 0.1j, prop=prop)
        for k in range(2):
            assert np.max(np.abs(s.einc[k] - free.einc[k])) < 1e-14
        assert s.inc_scale == 1.0
    o_s, o_f = oracle_for(s), oracle_for(free)
    for o in (o_s, o_f):
        o.set_cc(s.cc[0].reshape(1, 3))
    x = np.random.default_rng(6).standard_normal(3 * s.n) + 0j
    ys, _ = o_s.matvec(x)
    yf, _ = o_f.matvec(x)
    assert np.linalg.norm(ys - yf) < 1e-14 * np.linalg.norm(yf)

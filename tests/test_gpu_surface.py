"""Surface mode on the GPU (particle near a substrate: reflected interaction R, fft.c:818-887 / matvec.c:249-303),
through the C ABI, against the oracle and the reference's own runs (tests/golden/reference_surface.json):

- the FP64 R matrix (image relation built on the device, Sommerfeld table combined on the device, and a tensor given
  by the caller) equals the oracle's;
- FP64 and FP32 matvecs (plain and Hermitian, one and two RHS, the generic and the power-of-two transforms, small L2
  chunks) equal the oracle's;
- FP64 and mixed solves give the reference's Cext and Cabs through adda_gb300_cross_sections_beam, with the
  reference's iteration counts in FP64."""
import os

import numpy as np
import pytest

from helpers import oracle_for, oracle_solve, rel
from test_gpu_parity import random_vec
from test_surface_oracle import CASES, surface_setup

pytestmark = pytest.mark.gpu
BY = {c["name"]: c for c in CASES}


def context(s, nrhs=2, surface=None):
    import adda_gb300 as A
    if surface is None:
        return A.Context.from_setup(s, nrhs_max=nrhs)
    c = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs, surface=surface)
    c.init_dmatrix()
    for r in range(min(nrhs, 2)):
        c.set_cc(r, s.cc[r].reshape(1, 3))
    return c


def host_tensor(s):
    """the image-relation reflected tensor on the caller's grid [k<2bZ-1][j<bY][i+bX-1][6] (ReflTerm_img,
    interaction.c:1092-1153), evaluated here in numpy for the HOST relation"""
    bX, bY, bZ = s.box
    k, j, i = np.meshgrid(np.arange(2 * bZ - 1), np.arange(bY), np.arange(1 - bX, bX), indexing="ij")
    q = np.stack([i, j, k + s.surface["zsum_shift"]], -1).astype(float)
    rr = np.sqrt((q ** 2).sum(-1))
    v = q / rr[..., None]
    qm = np.stack([v[..., 0] ** 2, v[..., 0] * v[..., 1], v[..., 0] * v[..., 2], v[..., 1] ** 2, v[..., 1] * v[..., 2],
                   v[..., 2] ** 2], -1)
    rr = rr * s.gridspace
    kr = s.wavenum * rr
    m = s.surface["msub"]
    rcn = -1 if m is None else (1 - m * m) / (1 + m * m)
    scale = (rcn * np.exp(1j * kr) / rr ** 3)[..., None]
    t1, t2, t3 = (3 - kr ** 2)[..., None], (-3 * kr)[..., None], (kr ** 2 - 1)[..., None]
    diag = np.array([1, 0, 0, 1, 0, 1], bool)
    g = np.where(diag, (t1 * qm + t3) + 1j * (kr[..., None] + t2 * qm), (t1 + 1j * t2) * qm) * scale
    g[..., [2, 4, 5]] *= -1
    return np.ascontiguousarray(g)


@pytest.mark.parametrize("name", list(BY))
def test_rmatrix_matches_oracle(name):
    s = surface_setup(BY[name])
    g = context(s).rmatrix()
    o = oracle_for(s).rmatrix()
    assert g.shape == o.shape
    assert rel(g, o) < 1e-12, rel(g, o)


def test_rmatrix_host_tensor_equals_image_relation():
    s = surface_setup(BY["img_above"])
    sf = dict(s.surface, relation="host", data=host_tensor(s))
    assert rel(context(s, surface=sf).rmatrix(), context(s).rmatrix()) < 1e-13


@pytest.mark.parametrize("name", list(BY))
def test_matvec_matches_oracle(name):
    s = surface_setup(BY[name])
    ctx = context(s, 2)
    o = oracle_for(s)
    x = random_vec(s.n, 2, 11)
    for her in (False, True):
        y64, ip = ctx.matvec(x, "fp64", her)
        y32, _ = ctx.matvec(x, "fp32", her)
        for r in range(2):
            o.set_cc(s.cc[r].reshape(1, 3))
            want, _ = o.matvec(x[r], her)
            assert rel(y64[r], want) < 1e-13, (name, her, r, rel(y64[r], want))
            assert rel(y32[r], want) < 3e-6, (name, her, r, rel(y32[r], want))
            assert abs(ip[r] / np.vdot(y64[r], y64[r]).real - 1) < 1e-12


def test_matvec_power_of_two_grid_and_small_chunks():
    """box 32 (grid 64: compile-time transforms) with the FP32 chunk forced to 1 MB (many x-slab chunks)"""
    import adda_gb300 as A
    s = A.Setup(grid=32, m=1.5 + 0.1j, prop=[1, 2, -3], surface=dict(h=8.0, msub=2.0 + 0.5j, relation="img"))
    o = oracle_for(s)
    x = random_vec(s.n, 2, 12)
    os.environ["ADDA_GB300_CHUNK_MB"] = "1"
    try:
        ctx = context(s, 2)
    finally:
        del os.environ["ADDA_GB300_CHUNK_MB"]
    for her in (False, True):
        y64, _ = ctx.matvec(x, "fp64", her)
        y32, _ = ctx.matvec(x, "fp32", her)
        for r in range(2):
            o.set_cc(s.cc[r].reshape(1, 3))
            want, _ = o.matvec(x[r], her)
            assert rel(y64[r], want) < 1e-13
            assert rel(y32[r], want) < 3e-6


@pytest.mark.parametrize("grid", [64, 128])
def test_matvec_register_k2b_surface(grid):
    """FP32 surface matvec through the register-form K2b (gY = 128 and 256, the bench lattice) against the oracle"""
    import adda_gb300 as A
    s = A.Setup(grid=grid, m=1.33 + 0.01j, dpl=15, prop=[0, 0, -1],
                surface=dict(h=0.6 * grid * 2 * np.pi / 15, msub=1.5, relation="img"))
    ctx = context(s, 2)
    o = oracle_for(s)
    x = random_vec(s.n, 2, 13)
    y32, _ = ctx.matvec(x, "fp32")
    for r in range(2):
        o.set_cc(s.cc[r].reshape(1, 3))
        want, _ = o.matvec(x[r])
        assert rel(y32[r], want) < 3e-6, (grid, r, rel(y32[r], want))


def test_matvec_register_k2b_surface_y512():
    """the same through the register-form K2b with a 512-point y axis (a 4 x 256 x 4 box), plain and Hermitian"""
    import adda_gb300 as A
    d = 2 * np.pi / 15
    s = A.Setup(grid=4, shape="box", pars=(64, 1), m=1.33 + 0.01j, dpl=15, prop=[0, 0, -1],
                surface=dict(h=3 * d, msub=1.5, relation="img"))
    assert s.grid[1] == 512
    ctx = context(s, 2)
    o = oracle_for(s)
    x = random_vec(s.n, 2, 17)
    for her in (False, True):
        y32, _ = ctx.matvec(x, "fp32", her)
        for r in range(2):
            o.set_cc(s.cc[r].reshape(1, 3))
            want, _ = o.matvec(x[r], her)
            assert rel(y32[r], want) < 3e-6, (her, r, rel(y32[r], want))


@pytest.mark.parametrize("name", list(BY))
def test_solve_gives_reference_cross_sections(name):
    c = BY[name]
    s = surface_setup(c)
    ctx = context(s, 2)
    e = np.stack(s.einc)
    res = ctx.solve(e, method="qmr", prec="fp64", eps=1e-10)
    assert sum(st["niter"] for st in res["stats"]) == c["iterations_total"]
    ce, ca = ctx.cross_sections_beam(e, s.inc_scale)
    for k, pol in enumerate(("Y", "X")):
        assert abs(ce[k] / c["Cext_" + pol] - 1) < 3e-9, (pol, ce[k], c["Cext_" + pol])
        assert abs(ca[k] / c["Cabs_" + pol] - 1) < 3e-9, (pol, ca[k], c["Cabs_" + pol])
    mixed = ctx.solve(e, method="qmr", prec="mixed", eps=1e-10)
    assert all(st["status"] == "ok" for st in mixed["stats"])
    ce2, ca2 = ctx.cross_sections_beam(e, s.inc_scale)
    for k, pol in enumerate(("Y", "X")):
        assert abs(ce2[k] / c["Cext_" + pol] - 1) < 1e-7 and abs(ca2[k] / c["Cabs_" + pol] - 1) < 1e-7


@pytest.mark.parametrize("method", ["bicgstab", "cgnr", "bcgs2"])
def test_other_methods_match_oracle(method):
    s = surface_setup(BY["som_above"])
    ctx = context(s, 2)
    o = oracle_for(s)
    res = ctx.solve(np.stack(s.einc), method=method, prec="fp64", eps=1e-8)
    for k in range(2):
        r = oracle_solve(o, s, k, method=method, eps=1e-8)
        assert res["stats"][k]["niter"] == r["niter"]
        assert rel(res["p"][k], r["p"]) < 1e-8


def test_surface_create_errors():
    import adda_gb300 as A
    s = surface_setup(BY["img_above"])
    # zsum_shift -1: the lowest layer (z = 0) would sit below the substrate
    for bad in (dict(s.surface, zsum_shift=-1.0), dict(s.surface, relation="som", data=None),
                dict(s.surface, msub=None, relation="som", data=np.zeros(4))):
        with pytest.raises(A.AddaError):
            A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, 1, surface=bad)


def test_free_space_post_processing_refused_in_surface_mode():
    """the free-space scattering formulas (CalcFieldFree) do not apply near a substrate: those entry points refuse"""
    import adda_gb300 as A
    s = surface_setup(BY["img_above"])
    ctx = context(s, 2)
    ctx.solve(np.stack(s.einc), prec="fp64", eps=1e-6)
    with pytest.raises(A.AddaError):
        ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    with pytest.raises(A.AddaError):
        ctx.scattered_fields(np.array([[0.0, 0.0, 1.0]]))
    with pytest.raises(A.AddaError):
        ctx.vjp_chi(0, s.prop, s.incpol[0], np.zeros(s.n, np.complex128))


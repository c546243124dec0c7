"""Adjoint VJP of Cext and Cabs with respect to per-dipole susceptibility (the inhomogeneous-cube differentiation workload at small size):
checked against central finite differences of GPU FP64 solves (step 1e-6 on chi) and against perturbed solves of
the CPU oracle, and through a torch.autograd.Function wrapper."""
import numpy as np
import pytest

from helpers import oracle_for, setup_for

pytestmark = pytest.mark.gpu


def smooth_field(box, seed, sigma=2.0):
    """seeded Gaussian-smoothed random field on the box, standardised, mapped to (0,1) by the normal CDF"""
    from scipy.ndimage import gaussian_filter
    from scipy.stats import norm
    g = np.random.default_rng(seed).standard_normal(box[::-1])
    g = gaussian_filter(g, sigma, mode="wrap")
    g = (g - g.mean()) / g.std()
    return norm.cdf(g)


def chi_field(s):
    u1 = smooth_field(s.box, 20261204).ravel()
    u2 = smooth_field(s.box, 20261205).ravel()
    m = 1.3 + 0.4 * u1 + 0.05j * u2   # every cell of the box is a dipole (shape box), z-major order
    return (m * m - 1) / (4 * np.pi)


@pytest.fixture(scope="module")
def problem():
    import adda_gb300 as A
    s = setup_for(dict(grid=10, shape="box", m=1.5, dpl=12))
    assert s.n == 1000
    chi = chi_field(s)
    ctx = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max=2)
    ctx.init_dmatrix()
    return s, chi, ctx


def cross_for(ctx, s, chi, eps=1e-12):
    from autograd_dda import cc_from_chi
    cc, _ = cc_from_chi(s, chi)
    ctx.set_cc_dipole(0, cc)
    ctx.set_cc_dipole(1, cc)
    ctx.solve(s.einc[0][None], prec="fp64", eps=eps)
    ce, ca = ctx.cross_sections(s.prop[None], s.incpol[0][None])
    return ce[0], ca[0]


def test_vjp_vs_finite_differences(problem):
    from autograd_dda import cc_from_chi
    s, chi, ctx = problem
    cc, f = cc_from_chi(s, chi)
    ctx.set_cc_dipole(0, cc)
    ctx.set_cc_dipole(1, cc)
    ctx.solve(s.einc[0][None], prec="fp64", eps=1e-12)
    ge, ga = ctx.vjp_chi(0, s.prop, s.incpol[0], f, eps=1e-12)
    h = 1e-6
    for j in np.random.default_rng(20261206).choice(s.n, 6, replace=False):
        for part, dz in ((0, h), (1, 1j * h)):
            cp = chi.copy()
            cm = chi.copy()
            cp[j] += dz
            cm[j] -= dz
            ep, ap = cross_for(ctx, s, cp)
            em, am = cross_for(ctx, s, cm)
            fd_e, fd_a = (ep - em) / (2 * h), (ap - am) / (2 * h)
            scale_e = np.abs(ge).max()
            scale_a = np.abs(ga).max()
            assert abs(ge[j, part] - fd_e) <= 1e-5 * scale_e, (j, part, ge[j, part], fd_e)
            assert abs(ga[j, part] - fd_a) <= 1e-5 * scale_a, (j, part, ga[j, part], fd_a)


def test_vjp_vs_oracle_perturbed(problem):
    """the gradient against perturbed solves of the CPU oracle (FP64 restatement of the reference's solver)"""
    from autograd_dda import cc_from_chi
    from oracle import oracle as O
    s, chi, ctx = problem
    cc, f = cc_from_chi(s, chi)
    ctx.set_cc_dipole(0, cc)
    ctx.set_cc_dipole(1, cc)
    ctx.solve(s.einc[0][None], prec="fp64", eps=1e-12)
    ge, ga = ctx.vjp_chi(0, s.prop, s.incpol[0], f, eps=1e-12)
    o = oracle_for(s)
    h = 1e-6
    for j in (3, 517):
        vals = []
        for sgn in (1, -1):
            c2 = chi.copy()
            c2[j] += sgn * h
            cc2, _ = cc_from_chi(s, c2)
            o.set_cc_dipole(cc2)
            r = o.solve(s.einc[0], method=O.QMR_CS, eps=1e-12)
            vals.append(o.cross(r["p"], s.prop, s.incpol[0]))
        fd_e = (vals[0][0] - vals[1][0]) / (2 * h)
        fd_a = (vals[0][1] - vals[1][1]) / (2 * h)
        assert abs(ge[j, 0] - fd_e) <= 1e-5 * np.abs(ge).max()
        assert abs(ga[j, 0] - fd_a) <= 1e-5 * np.abs(ga).max()


def test_autograd_function(problem):
    import torch

    from autograd_dda import DdaCross
    s, chi, ctx = problem
    cr = torch.tensor(chi.real, requires_grad=True)
    ci = torch.tensor(chi.imag, requires_grad=True)
    ce, ca = DdaCross.apply(cr, ci, ctx, s, 0, 1e-12)
    (ce + 0.5 * ca).backward()
    j = 321
    h = 1e-6
    vals = []
    for sgn in (1, -1):
        c2 = chi.copy()
        c2[j] += sgn * 1j * h
        e, a = cross_for(ctx, s, c2)
        vals.append(e + 0.5 * a)
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(ci.grad[j].item() - fd) <= 1e-5 * float(ci.grad.abs().max())

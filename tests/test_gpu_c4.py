"""The differentiation workload at its stated size (tests/c4_workload.py): the 48^3 inhomogeneous cube (110,592
dipoles, grid 96^3), every dipole with its own refractive index from the seeded smooth fields.

- The adjoint VJP of Cext and Cabs with respect to every dipole's chi (one adjoint solve), obtained through the
  ctypes-loaded torch.autograd.Function (tests/autograd_dda.py), against central finite differences (step 1e-6 on
  chi, its real and imaginary part) at the 256 seeded dipoles. The 1024 perturbed FP64 solves run as right-hand
  sides of batched solves, each with its own per-dipole polarisabilities, and start from the unperturbed solution:
  they solve for the solution's change, to 1e-9 of the size of their own starting residual (a solve from zero to a
  residual of 1e-12 would leave errors comparable to the change itself); the cross-section differences are formed
  from the difference of the two polarisation vectors before summing (two full FP64 sums over 110,592 dipoles
  differ by rounding more than a step of 1e-6 at one dipole changes them).
- The same VJP against perturbed solves of the CPU oracle (the reference's algorithm in FP64) at one dipole.
- The forward solve of the field quantised to 14 materials against the reference's own run of it through
  -shape read (tests/golden/reference_c4_quantised.json): cross sections to 1e-8, iterations within 10 %.
"""
import json
import os

import numpy as np
import pytest

import c4_workload as W

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
NB = 512        # perturbed right-hand sides per batched solve
TOL_ABS = 1e-5  # |VJP - FD| <= TOL_ABS * max|gradient| + TOL_REL * |gradient|
TOL_REL = 1e-4
FD_TOL = 1e-9   # the perturbed solves stop at this fraction of their starting residual


def lattice():
    import adda_gb300 as A
    u1, u2 = W.fields()
    m = W.refractive_index(u1, u2)
    s = A.Setup(grid=W.BOX, shape="box", m=complex(m[np.argmax(np.abs(m))]), dpl=W.default_dpl(m))
    assert s.n == W.BOX ** 3 and tuple(s.grid) == (96, 96, 96)
    return s, W.chi_of(m)


@pytest.fixture(scope="module")
def c4():
    import torch

    import adda_gb300 as A
    from autograd_dda import DdaCross, cc_from_chi
    s, chi = lattice()
    ctx = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max=NB)
    ctx.init_dmatrix()
    # gradients through the autograd wrapper: one forward + adjoint per output
    grads = []
    for w_ext, w_abs in ((1.0, 0.0), (0.0, 1.0)):
        cr = torch.tensor(chi.real, requires_grad=True)
        ci = torch.tensor(chi.imag, requires_grad=True)
        ce, ca = DdaCross.apply(cr, ci, ctx, s, 0, 1e-12)
        (w_ext * ce + w_abs * ca).backward()
        grads.append(np.stack([cr.grad.numpy(), ci.grad.numpy()], axis=1))
    cc, _ = cc_from_chi(s, chi)
    # the unperturbed solution
    ctx.set_cc_dipole(0, cc)
    res = ctx.solve(s.einc[0][None], prec="fp64", eps=1e-12)
    return dict(s=s, chi=chi, ctx=ctx, cc=cc, x0=res["x"][0], ge=grads[0], ga=grads[1])


def pert_cc(s, chi, j, dz):
    """the LDR polarisability of dipole j with chi_j + dz (3 components)"""
    import adda_gb300 as A
    m = np.sqrt(1 + 4 * np.pi * (chi[j] + dz))
    return A.polarizability(m, s.kd, s.gridspace, s.prop, s.incpol[0], "ldr")


def absorb_weight(cc, k):
    """AbsCross's weight -Im(1/cc) - 2k^3/3 per component"""
    return -np.imag(1 / cc) - 2 * k ** 3 / 3


def _abs2(a):
    return a.abs() ** 2 if hasattr(a, "abs") else np.abs(a) ** 2


def cross_differences(xp, xm, S0, w0, E, k, sp_j, sm_j, wp_j, wm_j, j):
    """(Cext(P+) - Cext(P-), Cabs(P+) - Cabs(P-)) formed from the difference of the two polarisation vectors before
    any sum, so that FP64 rounding of the full sums does not enter. xp, xm: solutions [n,3]; S0, w0: the unperturbed
    sqrt(cc) and absorption weights [n,3]; sp_j/sm_j, wp_j/wm_j: those of dipole j with +/- the step.
    Cext = 4 pi k sum Im(P . conj(Einc)) (crosssec.c:823-845; equal to the forward-amplitude form for a plane wave),
    Cabs = 4 pi k sum w |P|^2 (crosssec.c:866-882). Works on numpy arrays or torch tensors."""
    Pp = xp * S0
    Pm = xm * S0
    Pp[j] = xp[j] * sp_j
    Pm[j] = xm[j] * sm_j
    D, Sm = Pp - Pm, Pp + Pm
    dext = 4 * np.pi * k * float((D * E.conj()).imag.sum())
    sw = float((w0 * (D * Sm.conj()).real).sum())
    sw += float(((wp_j - w0[j]) * _abs2(Pp[j])).sum())
    sw -= float(((wm_j - w0[j]) * _abs2(Pm[j])).sum())
    return dext, 4 * np.pi * k * sw


def fd_batch(c, dirs):
    """central differences (dCext, dCabs)/(2h) for dirs = [(j, +dz), (j, -dz), ...] (pairs adjacent): the perturbed
    solves as right-hand sides of one FP64 solve from the unperturbed solution, to FD_TOL of the smallest starting
    residual, and the differences of their polarisations"""
    import torch
    s, ctx, n = c["s"], c["ctx"], c["s"].n
    R = len(dirs)
    cc0 = c["cc"]
    for r, (j, dz) in enumerate(dirs):
        cc = cc0.copy()
        cc[j] = pert_cc(s, c["chi"], j, dz)
        ctx.set_cc_dipole(r, cc)
    d_e = torch.from_numpy(np.ascontiguousarray(s.einc[0]).view(np.float64)).cuda().repeat(R)
    x0 = torch.from_numpy(np.ascontiguousarray(c["x0"]).view(np.float64)).cuda()
    d_x = x0.repeat(R)
    # the starting residuals (relative residual after one iteration from x0) set the tolerance
    st = ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), None, method="qmr", prec="fp64", eps=1e-300,
                          maxiter=1, init="x0")
    eps = FD_TOL * min(x["resid"] for x in st)
    c["last_eps"] = eps
    d_x = x0.repeat(R)
    st = ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), None, method="qmr", prec="fp64", eps=eps,
                          maxiter=3000, init="x0")
    assert all(x["status"] == "ok" for x in st), [x for x in st if x["status"] != "ok"][:3]
    x = d_x.view(torch.complex128).view(R, n, 3)
    S0 = torch.from_numpy(np.sqrt(cc0)).cuda()
    w0 = torch.from_numpy(absorb_weight(cc0, s.wavenum)).cuda()
    E = torch.from_numpy(np.ascontiguousarray(s.einc[0]).reshape(n, 3)).cuda()
    out = []
    for r in range(0, R, 2):
        j, dz = dirs[r]
        ccp, ccm = pert_cc(s, c["chi"], j, dz), pert_cc(s, c["chi"], j, -dz)
        dext, dabs = cross_differences(
            x[r], x[r + 1], S0, w0, E, s.wavenum,
            torch.from_numpy(np.sqrt(ccp)).cuda(), torch.from_numpy(np.sqrt(ccm)).cuda(),
            torch.from_numpy(absorb_weight(ccp, s.wavenum)).cuda(),
            torch.from_numpy(absorb_weight(ccm, s.wavenum)).cuda(), j)
        out.append((dext / (2 * abs(dz)), dabs / (2 * abs(dz))))
    return out, max(x["niter"] for x in st)


def test_c4_vjp_vs_central_differences(c4):
    h = W.FD_STEP
    js = W.fd_dipoles(c4["s"].n)
    dirs, keys = [], []
    for j in js:
        for part, dz in ((0, h), (1, 1j * h)):
            dirs += [(int(j), dz), (int(j), -dz)]
            keys.append((int(j), part))
    fd_e = np.zeros((len(js), 2))
    fd_a = np.zeros((len(js), 2))
    row = {int(j): k for k, j in enumerate(js)}
    for b0 in range(0, len(dirs), NB):
        res, _ = fd_batch(c4, dirs[b0:b0 + NB])
        for (j, part), (de, da) in zip(keys[b0 // 2:(b0 + NB) // 2], res):
            fd_e[row[j], part] = de
            fd_a[row[j], part] = da
    for g, fd, name in ((c4["ge"], fd_e, "Cext"), (c4["ga"], fd_a, "Cabs")):
        gj = g[js]
        err = np.abs(gj - fd)
        bound = TOL_ABS * np.abs(g).max() + TOL_REL * np.abs(gj)
        i, part = np.unravel_index(np.argmax(err / bound), err.shape)
        assert (err <= bound).all(), (name, int(js[i]), part, err[i, part], bound[i, part], gj[i, part], fd[i, part])


def test_c4_vjp_vs_oracle_perturbed(c4):
    """d/dRe chi at one dipole from two perturbed FP64 solves of the CPU oracle, started from the oracle's own
    unperturbed solution, differenced like the GPU's"""
    from helpers import oracle_for
    from oracle import oracle as O
    s, chi, h = c4["s"], c4["chi"], W.FD_STEP
    j = int(W.fd_dipoles(s.n)[7])
    cc0 = c4["cc"]
    o = oracle_for(s)
    o.set_cc_dipole(cc0)
    base = o.solve(s.einc[0], method=O.QMR_CS, eps=1e-12)
    xs, ccs = [], []
    for sgn in (1, -1):
        cc = cc0.copy()
        cc[j] = pert_cc(s, chi, j, sgn * h)
        ccs.append(cc[j].copy())
        o.set_cc_dipole(cc)
        r = o.solve(s.einc[0], method=O.QMR_CS, eps=1e-14, maxiter=400, init_field=O.IF_X0, x0=base["x"])
        xs.append(r["x"].reshape(s.n, 3))
    o.close()
    dext, dabs = cross_differences(xs[0], xs[1], np.sqrt(cc0), absorb_weight(cc0, s.wavenum),
                                   s.einc[0].reshape(s.n, 3), s.wavenum, np.sqrt(ccs[0]), np.sqrt(ccs[1]),
                                   absorb_weight(ccs[0], s.wavenum), absorb_weight(ccs[1], s.wavenum), j)
    fd_e, fd_a = dext / (2 * h), dabs / (2 * h)
    assert abs(c4["ge"][j, 0] - fd_e) <= TOL_ABS * np.abs(c4["ge"]).max() + TOL_REL * abs(fd_e), (c4["ge"][j, 0], fd_e)
    assert abs(c4["ga"][j, 0] - fd_a) <= TOL_ABS * np.abs(c4["ga"]).max() + TOL_REL * abs(fd_a), (c4["ga"][j, 0], fd_a)


def test_c4_quantised_field_vs_reference():
    import adda_gb300 as A
    run = json.load(open(os.path.join(HERE, "golden", "reference_c4_quantised.json")))["run"]
    u1, u2 = W.fields()
    mat, levels = W.quantised(u1, u2)
    s = A.Setup(grid=W.BOX, shape="box", m=complex(levels[np.argmax(np.abs(levels))]), dpl=W.default_dpl(levels))
    assert s.n == run["ndip"] and list(s.box) == run["box"] and list(s.grid) == run["grid"]
    assert abs(s.dpl / run["dpl"] - 1) < 1e-5  # the log prints dpl to 6 digits
    ctx = A.Context(s.box, s.pos, mat, s.gridspace, s.wavenum, s.grid, nrhs_max=2)
    ctx.init_dmatrix()
    for r in range(2):
        cc = np.stack([A.polarizability(m, s.kd, s.gridspace, s.prop, s.incpol[r], "ldr") for m in levels])
        ctx.set_cc(r, cc.reshape(len(levels), 3))
    res = ctx.solve(np.stack(s.einc), prec="fp64", eps=1e-10)
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    for r, pol in enumerate("YX"):
        assert res["stats"][r]["status"] == "ok"
        assert abs(ce[r] / run["cross"][pol]["Cext"] - 1) < 1e-8, (pol, ce[r], run["cross"][pol])
        assert abs(ca[r] / run["cross"][pol]["Cabs"] - 1) < 1e-8, (pol, ca[r], run["cross"][pol])
        assert abs(res["stats"][r]["niter"] / run["niter"][pol] - 1) <= 0.1
    ctx.close()

"""GPU parity: the sm_103a kernels (through the C ABI) against the oracle and the reference's golden outputs.

Tolerances:
  - FP64 D matrix and matvec: 1e-13 relative L2 against the oracle (same arithmetic, different FFT orderings);
    FP32 matvec: 5e-6.
  - Solves at eps=1e-10: cross sections within 1e-9 of the oracle / the reference (the FP64 parity bar).
  - Solves at eps=1e-5: a solution that only meets residual 1e-5 is itself 0.3-1.6e-6 away from the converged cross
    section, and 1-ulp differences in the matvec move the QMR_CS/BiCGStab iteration count by several iterations
    near the threshold (checked on the CPU: 1e-16 noise moves the 16^3 sphere between 43 and 49 iterations). So
    cross sections are compared with 2e-6 relative, iteration counts within +-6, and residual histories while the
    residual is above 1e-2.
  - Mixed precision: the FP64-recomputed residual meets eps, and Cext/Cabs are within 1e-6 of the converged
    (eps=1e-10) FP64 oracle (the refinement stops below eps for that, see final_eps in the C ABI).
"""
import numpy as np
import pytest

from helpers import case, golden, oracle_for, oracle_solve, rel, setup_for, solver_opts

pytestmark = pytest.mark.gpu


def random_vec(n, R, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((R, 3 * n)) + 1j * rng.standard_normal((R, 3 * n)))


def cube_setup(box, grid, m=1.3 + 0.05j, dpl=12.0):
    """a fully occupied box (every lattice cell is a dipole) with an explicit FFT grid, to exercise radices 7/11/13"""
    import math

    import adda_gb300 as A
    bx, by, bz = box
    z, y, x = np.meshgrid(np.arange(bz), np.arange(by), np.arange(bx), indexing="ij")
    pos = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.uint16)

    class S:
        pass

    s = S()
    s.box, s.grid, s.pos, s.mat, s.n = tuple(box), tuple(grid), pos, np.zeros(len(pos), np.uint8), len(pos)
    s.gridspace, s.wavenum = 2 * math.pi / dpl, 1.0
    s.kd = s.gridspace
    s.prop, py, px = A.rotation()
    s.incpol = [py, px]
    s.cc = [A.polarizability(m, s.kd, s.gridspace, s.prop, e, "ldr") for e in s.incpol]
    s.einc = [A.plane_wave(s.box, s.pos, s.gridspace, s.wavenum, s.prop, e) for e in s.incpol]
    return s


SETUPS = {
    "sphere16": lambda: setup_for(dict(grid=16, m=1.5, dpl=10)),
    "ell24_grid48x32x40": lambda: setup_for(case("ell24")["setup"]),
    "box12_grid24": lambda: setup_for(case("box12")["setup"]),
    "grid30_60cubed": lambda: setup_for(case("grid30")["setup"]),
    "cube_7x11x13_radix7_11_13": lambda: cube_setup((7, 11, 13), (14, 22, 26)),
    "cube_5x3x9_radix5_3": lambda: cube_setup((5, 3, 9), (10, 6, 18)),
    "grid2_tiny": lambda: setup_for(case("grid2")["setup"]),
    # power-of-two axes of 64..512 take the compile-time kernels (register/column FFTs in FP32): one axis of 512
    # at a time on thin boxes, and 64/128/256 together, each checked against the oracle
    "thin_x512": lambda: cube_setup((256, 3, 2), (512, 6, 4)),
    "thin_y512": lambda: cube_setup((2, 256, 3), (4, 512, 6)),
    "thin_z512": lambda: cube_setup((3, 2, 256), (6, 4, 512)),
    "box_64x128x256": lambda: cube_setup((32, 64, 128), (64, 128, 256)),
    "box_256x64x128": lambda: cube_setup((128, 32, 64), (256, 64, 128)),
    # FCD interaction terms (with their Ci/Si) in D
    "int_fcd": lambda: setup_for(case("int_fcd")["setup"]),
    "int_fcd_st": lambda: setup_for(case("int_fcd_st")["setup"]),
    "ell_fcd": lambda: setup_for(case("ell_fcd_eps8")["setup"]),
    # static non-local interaction terms (erf / incomplete gamma) in D
    "int_nloc": lambda: setup_for(case("int_nloc")["setup"]),
    "int_nloc_av": lambda: setup_for(case("int_nloc_av")["setup"]),
    "int_nloc_small": lambda: setup_for(case("int_nloc_small")["setup"]),
}


def context(s, R=2):
    import adda_gb300 as A
    c = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max=R,
                  interaction=getattr(s, "interaction", "poi"), nloc_rp=getattr(s, "nloc_rp", 0.0))
    c.init_dmatrix()
    for r in range(R):
        c.set_cc(r, s.cc[r % 2].reshape(1, 3))
    return c


@pytest.mark.parametrize("name", list(SETUPS))
def test_dmatrix_fp64(name):
    s = SETUPS[name]()
    o = oracle_for(s)
    c = context(s)
    assert c.grid == tuple(s.grid)
    d_gpu = c.dmatrix()
    d_ref = o.dmatrix()
    assert d_gpu.shape == d_ref.shape
    assert rel(d_gpu, d_ref) < 1e-13


@pytest.mark.parametrize("name", list(SETUPS))
@pytest.mark.parametrize("her", [False, True])
def test_matvec_fp64_and_fp32(name, her):
    s = SETUPS[name]()
    o = oracle_for(s)
    c = context(s, R=2)
    x = random_vec(s.n, 2, 7)
    y, ip = c.matvec(x, "fp64", her)
    yf, ipf = c.matvec(x, "fp32", her)
    for r in range(2):
        o.set_cc(s.cc[r % 2].reshape(1, 3))
        yr, ipr = o.matvec(x[r], her)
        assert rel(y[r], yr) < 1e-13
        assert abs(ip[r] / ipr - 1) < 1e-12
        assert rel(yf[r], yr) < 5e-6
        assert abs(ipf[r] / ipr - 1) < 1e-5


def test_matvec_per_dipole_cc():
    """inhomogeneous medium: every dipole its own polarisability (per-dipole S = diag(sqrt(cc)))"""
    import adda_gb300 as A
    s = setup_for(dict(grid=16, m=1.5, dpl=10))
    rng = np.random.default_rng(3)
    m = 1.3 + 0.4 * rng.random(s.n) + 0.05j * rng.random(s.n)
    cc = np.stack([A.polarizability(mi, s.kd, s.gridspace, s.prop, s.incpol[0], "ldr") for mi in m])
    o = oracle_for(s)
    o.set_cc_dipole(cc)
    c = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max=1)
    c.init_dmatrix()
    c.set_cc_dipole(0, cc)
    x = random_vec(s.n, 1, 11)[0]
    y, _ = c.matvec(x, "fp64")
    yr, _ = o.matvec(x)
    assert rel(y, yr) < 1e-13


SOLVE_CASES = ["c1_qmr", "c1_bicgstab", "mgn", "mgn_eps10", "mgn_init_zero", "mgn_init_inc", "mgn_bicgstab",
               "mgn_maxiter3", "ell_orient", "pol_ldr_prop", "prop_ell", "ell24", "box12", "grid6", "grid18",
               "sample_default", "c2_small", "mgn_bicg", "mgn_cgnr", "mgn_csym", "c1_bicg", "c1_cgnr", "c1_csym",
               "ell_bicg_eps8", "ell_csym_eps8", "mgn_qmr2", "c1_qmr2", "ell_qmr2_eps8",
               "mgn_bcgs2", "c1_bcgs2", "ell_bcgs2_eps8", "pol_cldr", "pol_fcd", "pol_igt_so", "pol_lak", "pol_so",
               "int_fcd", "int_fcd_st", "c1_fcd", "ell_fcd_eps8", "mgn_wkb", "c1_wkb", "ell_wkb_eps8",
               "int_nloc", "int_nloc_av", "int_nloc_small", "int_nloc0", "c1_nloc_av"]


@pytest.mark.parametrize("name", SOLVE_CASES)
def test_solve_fp64_vs_reference(name):
    import adda_gb300 as A
    c0 = case(name)
    s = setup_for(c0["setup"])
    opts = solver_opts(c0["setup"])
    ctx = A.Context.from_setup(s, nrhs_max=2)
    if opts["init"] == "wkb":  # -init_field wkb: x_0 from the host WKB field (CalcFieldWKB + InitFieldfromE)
        from helpers import wkb_x0
        opts["init"] = "x0"
        opts["x0"] = np.stack([wkb_x0(s, r) for r in range(2)])
    res = ctx.solve(np.stack(s.einc), prec="fp64", hist_cap=2000, **opts)
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    tight = opts["eps"] < 1e-8
    for r, pol in enumerate("YX"):
        st = res["stats"][r]
        ref_hist = np.array(c0["resid"][pol])
        nref = len(ref_hist) - 1
        assert abs(st["niter"] - nref) <= (0 if tight else 6), (st, nref)
        if c0["maxiter_warning"]:
            assert st["status"] == "maxiter"
            assert st["niter"] == opts["maxiter"]
        else:
            assert st["status"] == "ok"
            assert st["resid"] <= opts["eps"]
        h = res["hist"][r][: st["niter"] + 1]
        # CGNR and CSYM amplify rounding differences between two FFT call orders from a residual of ~5e-2 on
        # (measured: CGNR oracle vs reference, CSYM GPU vs reference on c1 at iteration 28; both still end within
        # 6 iterations and 2e-6 in the cross sections, and match the oracle at eps=1e-10)
        early = ref_hist[: len(h)] > (1e-1 if opts["method"] in ("cgnr", "csym") else 1e-2)
        np.testing.assert_allclose(h[: len(ref_hist)][early], ref_hist[: len(h)][early], rtol=1e-7)
        tol = 1e-9 if tight else 2e-6
        if opts.get("x0") is not None and s.n > 1000:
            tol = 3e-6  # WKB start on the 16^3 m=1.5 sphere: the reference's own Y and X runs differ by 1.0e-6
        for q, v in (("Cext", ce[r]), ("Cabs", ca[r])):
            want = c0["cross"][pol][q]
            assert abs(v - want) <= max(tol * abs(want), 1e-12), (pol, q, v, want)


@pytest.mark.parametrize("method", ["qmr", "bicgstab", "bicg", "cgnr", "csym", "qmr2", "bcgs2"])
def test_solve_fp64_vs_oracle_tight(method):
    """at eps=1e-10 the GPU FP64 solve and the oracle agree on Cext/Cabs to 1e-9 and per dipole to 1e-8"""
    import adda_gb300 as A
    s = setup_for(case("ell24")["setup"])
    o = oracle_for(s)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    res = ctx.solve(np.stack(s.einc), method=method, prec="fp64", eps=1e-10)
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    for r in range(2):
        ro = oracle_solve(o, s, r, method=method, eps=1e-10)
        assert rel(res["p"][r], ro["p"]) < 1e-8
        assert abs(ce[r] / ro["Cext"] - 1) < 1e-9
        assert abs(ca[r] / ro["Cabs"] - 1) < 1e-9


@pytest.mark.parametrize("prec", ["mixed", "mixed_f64vec", "mixed_f32vec"])
@pytest.mark.parametrize("method", ["qmr", "bicgstab"])
@pytest.mark.parametrize("name", ["c1_qmr", "ell24", "c2_small"])
def test_solve_mixed(name, method, prec):
    """mixed precision: the FP64 recomputed residual meets eps; cross sections within 1e-6 of the converged FP64
    oracle (Cabs relative to max(Cabs, Cext): for a real index it is zero up to rounding)"""
    import adda_gb300 as A
    c0 = case(name)
    s = setup_for(c0["setup"])
    o = oracle_for(s)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    res = ctx.solve(np.stack(s.einc), method=method, prec=prec, eps=1e-5)
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    for r in range(2):
        st = res["stats"][r]
        assert st["status"] == "ok", st
        assert st["resid"] <= 1e-5
        assert st["matvecs_fp64"] >= 1
        rc = oracle_solve(o, s, r, method=method, eps=1e-10)
        assert abs(ce[r] / rc["Cext"] - 1) < 1e-6, (ce[r], rc["Cext"])
        assert abs(ca[r] - rc["Cabs"]) < 1e-6 * max(abs(rc["Cabs"]), abs(rc["Cext"])), (ca[r], rc["Cabs"])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_solve_from_x0(prec):
    """init_field X0: started from the converged solution the solve stops at once; started from the WKB field it
    converges to the same cross sections as from the default start"""
    import adda_gb300 as A
    from helpers import wkb_x0
    s = setup_for(case("ell24")["setup"])
    ctx = A.Context.from_setup(s, nrhs_max=2)
    ref = ctx.solve(np.stack(s.einc), prec="fp64", eps=1e-10)
    ce0, _ = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    res = ctx.solve(np.stack(s.einc), prec=prec, eps=1e-5, init="x0", x0=ref["x"])
    assert all(st["niter"] == 0 and st["resid"] <= 1e-5 for st in res["stats"]), res["stats"]
    assert rel(res["x"], ref["x"]) < 1e-12
    res = ctx.solve(np.stack(s.einc), prec=prec, eps=1e-8, init="x0",
                    x0=np.stack([wkb_x0(s, r) for r in range(2)]))
    ce, _ = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    for r in range(2):
        assert res["stats"][r]["status"] == "ok" and res["stats"][r]["resid"] <= 1e-8
        assert abs(ce[r] / ce0[r] - 1) < 1e-7


@pytest.mark.parametrize("method", ["bicg", "cgnr", "csym", "qmr2", "bcgs2"])
@pytest.mark.parametrize("name", ["c1_qmr", "ell24"])
def test_solve_mixed_other_methods(name, method):
    """BiCG_CS, CGNR, CSYM, QMR_CS_2 and BCGS2 in mixed precision (double-float vectors): FP64 residual meets eps,
    cross sections within 1e-6 of the converged FP64 oracle"""
    import adda_gb300 as A
    s = setup_for(case(name)["setup"])
    o = oracle_for(s)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    res = ctx.solve(np.stack(s.einc), method=method, prec="mixed", eps=1e-5)
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    for r in range(2):
        st = res["stats"][r]
        assert st["status"] == "ok" and st["resid"] <= 1e-5, st
        rc = oracle_solve(o, s, r, method="qmr", eps=1e-10)
        assert abs(ce[r] / rc["Cext"] - 1) < 1e-6, (ce[r], rc["Cext"])
        assert abs(ca[r] - rc["Cabs"]) < 1e-6 * max(abs(rc["Cabs"]), abs(rc["Cext"])), (ca[r], rc["Cabs"])


def test_cross_sections_from_pvec():
    """the device cross-section reduction against the oracle's formula on the same polarisations"""
    import adda_gb300 as A
    s = setup_for(case("prop_ell")["setup"])
    o = oracle_for(s)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    res = ctx.solve(np.stack(s.einc), prec="fp64", eps=1e-8)
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    for r in range(2):
        o.set_cc(s.cc[r].reshape(1, 3))
        e, a = o.cross(res["p"][r], s.prop, s.incpol[r])
        assert abs(ce[r] / e - 1) < 1e-12
        assert abs(ca[r] / a - 1) < 1e-12


def test_solve_rhs_batch_equals_single():
    """solving both polarisations together gives the same results as solving them one at a time"""
    import adda_gb300 as A
    s = setup_for(case("ell_orient")["setup"])
    ctx = A.Context.from_setup(s, nrhs_max=2)
    both = ctx.solve(np.stack(s.einc), prec="fp64", eps=1e-6)
    for r in range(2):
        c1 = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max=1)
        c1.init_dmatrix()
        c1.set_cc(0, s.cc[r].reshape(1, 3))
        one = c1.solve(s.einc[r][None], prec="fp64", eps=1e-6)
        assert one["stats"][0]["niter"] == both["stats"][r]["niter"]
        assert rel(one["x"][0], both["x"][r]) < 1e-12


def test_large_matvec_properties():
    """128^3 sphere (256^3 grid): FP32 vs FP64 matvec agreement, linearity and complex symmetry x1.A.x2 = x2.A.x1"""
    s = setup_for(dict(grid=128, m=1.33 + 0.01j, dpl=15))
    assert s.n == 1099136 and s.grid == (256, 256, 256)
    c = context(s, R=2)
    x = random_vec(s.n, 2, 5)
    y64, _ = c.matvec(x, "fp64")
    y32, _ = c.matvec(x, "fp32")
    for r in range(2):
        assert rel(y32[r], y64[r]) < 5e-6
    # both RHS carry different cc (Y and X polarisations); use RHS 0 for the algebraic checks
    z, _ = c.matvec(np.stack([2.0 * x[0] - 1j * x[1], x[1]]), "fp64")
    w, _ = c.matvec(np.stack([x[1], x[1]]), "fp64")
    lin = 2.0 * y64[0] - 1j * w[0]
    assert rel(z[0], lin) < 1e-13
    a = np.dot(x[0], w[0])
    b = np.dot(x[1], y64[0])
    assert abs(a - b) / abs(a) < 1e-12


def test_solve_many_equals_individual():
    """several particles with uneven grids solved concurrently (one stream each) give the same results as one at a
    time (the batching pattern: ellipsoids of different sizes, orientations, both polarisations)"""
    import adda_gb300 as A
    specs = [dict(grid=8, shape="ellipsoid", pars=(0.6, 0.9), m=1.3 + 0.02j, orient=(10, 40, 70)),
             dict(grid=12, shape="ellipsoid", pars=(0.8, 0.5), m=1.6 + 0.01j, orient=(200, 100, 15)),
             dict(grid=16, shape="ellipsoid", pars=(0.7, 0.7), m=1.45 + 0.04j, orient=(5, 150, 300))]
    setups = [setup_for(k) for k in specs]
    ctxs = [A.Context.from_setup(s, nrhs_max=2) for s in setups]
    many = A.solve_many(ctxs, [np.stack(s.einc) for s in setups], prec="fp64", eps=1e-8)
    for s, c, (x, p, st) in zip(setups, ctxs, many):
        one = c.solve(np.stack(s.einc), prec="fp64", eps=1e-8)
        for r in range(2):
            assert st[r]["status"] == "ok"
            assert st[r]["niter"] == one["stats"][r]["niter"]
            assert rel(x[r], one["x"][r]) < 1e-12

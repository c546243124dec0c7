"""Iteration checkpoints on the GPU through the C ABI (adda_gb300_chpoint_save / _load, init_field ADDA_IF_CHPOINT,
solve_params.chp_time), in the reference's chp.<ringid> format (src/iterative.c:165-278):

- the GPU's FP64 state after the reference's number of iterations equals the reference's own file field by field;
- resumed from the reference's file, the GPU continues with the reference's residual history and cross sections;
- a solve stopped by the checkpoint time and resumed from its own checkpoint ends where the uninterrupted solve ends;
- the oracle resumes from a GPU-written checkpoint like from its own;
- the drop-in's -chpoint / -chp_load path (stand-in host) writes and reads the same files."""
import os
import subprocess

import numpy as np
import pytest

from helpers import case, oracle_for, oracle_solve, parse_chpoint, rel, setup_for
from test_chpoint_oracle import CASES, CHP, compare_state, ref_file, setup

pytestmark = pytest.mark.gpu

METHODS = ["qmr", "bicgstab", "bicg", "cgnr", "csym", "qmr2", "bcgs2"]


def context(s, nrhs=1):
    import adda_gb300 as A
    return A.Context.from_setup(s, nrhs_max=nrhs)


@pytest.mark.parametrize("c", CASES, ids=[c["method"] for c in CASES])
def test_gpu_state_matches_reference_file(c):
    s = setup()
    ctx = context(s)
    nsave = len(c["resid_before"]) - 1
    res = ctx.solve(s.einc[0][None], method=c["method"], prec="fp64", eps=CHP["eps"], maxiter=nsave,
                    full_steps=True, hist_cap=64)
    assert res["stats"][0]["status"] == "maxiter" and res["stats"][0]["niter"] == nsave
    np.testing.assert_allclose(res["hist"][0][:nsave + 1], c["resid_before"], rtol=1e-9)
    # GPU FFTs against the reference's FFTW-order rounding: every field within 1e-9
    compare_state(ctx.chpoint_save(0), ref_file(c["method"]), c["method"], 1e-9)


@pytest.mark.parametrize("c", CASES, ids=[c["method"] for c in CASES])
def test_gpu_resumes_reference_file(c):
    s = setup()
    ctx = context(s)
    ctx.chpoint_load(0, ref_file(c["method"]))
    res = ctx.solve(s.einc[0][None], method=c["method"], prec="fp64", eps=CHP["eps"], init="chpoint", hist_cap=256)
    st = res["stats"][0]
    want = np.array(c["resid_after"])
    first = c["first_loaded"]
    assert st["status"] == "ok" and st["niter"] == first - 1 + len(want), (st, first, len(want))
    assert st["matvecs_fp64"] == len(want) * {"bicgstab": 2, "cgnr": 2, "bcgs2": 4}.get(c["method"], 1)
    assert abs(res["hist"][0][first - 1] / c["resid_before"][-1] - 1) < 1e-9
    np.testing.assert_allclose(res["hist"][0][first:first + len(want)], want, rtol=1e-8)
    ce, ca = ctx.cross_sections(s.prop[None], s.incpol[0][None])
    assert abs(ce[0] / c["cross"]["Cext"] - 1) < 1e-9 and abs(ca[0] / c["cross"]["Cabs"] - 1) < 1e-9


@pytest.mark.parametrize("method", METHODS)
def test_gpu_stop_and_resume_equals_uninterrupted(method):
    """chp_time stops both RHS after the first graph batch (status chpoint); their checkpoints, loaded back, finish
    the solve with the iterates of the uninterrupted one"""
    s = setup_for(case("ell24")["setup"])
    ctx = context(s, 2)
    e = np.stack(s.einc)
    full = ctx.solve(e, method=method, prec="fp64", eps=1e-8, check_every=2, hist_cap=2000)
    part = ctx.solve(e, method=method, prec="fp64", eps=1e-8, check_every=2, chp_time=1e-9, hist_cap=2000)
    for r in range(2):
        assert part["stats"][r]["status"] == "chpoint" and part["stats"][r]["niter"] == 2, part["stats"][r]
    chp = [ctx.chpoint_save(r) for r in range(2)]
    for r in range(2):
        head, _, _ = parse_chpoint(chp[r], method)
        assert head[2] == 3 and head[1] == 3 * s.n   # niter = 3: two iterations done
        ctx.chpoint_load(r, chp[r])
    res = ctx.solve(e, method=method, prec="fp64", eps=1e-8, init="chpoint", check_every=2, hist_cap=2000)
    for r in range(2):
        assert res["stats"][r]["niter"] == full["stats"][r]["niter"]
        assert res["stats"][r]["status"] == full["stats"][r]["status"] == "ok"
        n = full["stats"][r]["niter"]
        # the dot products carried into the first resumed iteration are recomputed from the loaded vectors (same
        # partition and order as the fused ones; QMR_CS_2's delta divides by ro^2 instead of |v~|^2, which moves late
        # residuals of 1e-8 by ~1e-16 absolute)
        np.testing.assert_allclose(res["hist"][r][3:n + 1], full["hist"][r][3:n + 1], rtol=1e-10, atol=1e-14)
        assert rel(res["x"][r], full["x"][r]) < 1e-10


@pytest.mark.parametrize("method", METHODS)
def test_oracle_resumes_gpu_checkpoint(method):
    s = setup()
    ctx = context(s)
    ctx.solve(s.einc[0][None], method=method, prec="fp64", eps=CHP["eps"], maxiter=2, full_steps=True)
    chp = ctx.chpoint_save(0)
    o = oracle_for(s)
    ref = oracle_solve(o, s, 0, method=method, eps=CHP["eps"])
    got = oracle_solve(o, s, 0, method=method, eps=CHP["eps"], chp_in=chp)
    assert got["niter"] == ref["niter"]
    np.testing.assert_allclose(got["resid"][1:], ref["resid"][3:], rtol=1e-8)
    assert abs(got["Cext"] / ref["Cext"] - 1) < 1e-10


def test_chpoint_errors():
    import adda_gb300 as A
    s = setup()
    ctx = context(s)
    with pytest.raises(RuntimeError):
        ctx.chpoint_save(0)                       # no FP64 solve yet
    with pytest.raises(RuntimeError):
        ctx.chpoint_load(0, ref_file("qmr")[:-16])  # too short
    with pytest.raises(RuntimeError):
        ctx.chpoint_load(0, ref_file("qmr") + b"\0")  # too long
    other = setup_for(case("mgn")["setup"])     # another lattice: different vector size
    with pytest.raises(RuntimeError):
        context(other).chpoint_load(0, ref_file("qmr"))
    ctx.chpoint_load(0, ref_file("qmr"))
    with pytest.raises(RuntimeError):             # a QMR_CS state for BiCGStab
        ctx.solve(s.einc[0][None], method="bicgstab", prec="fp64", init="chpoint")
    ctx.chpoint_load(0, ref_file("qmr"))
    with pytest.raises(RuntimeError):             # FP64 only
        ctx.solve(s.einc[0][None], method="qmr", prec="mixed", init="chpoint")
    ctx.solve(s.einc[0][None], method="qmr", prec="mixed")
    with pytest.raises(RuntimeError):             # no state after a mixed solve
        ctx.chpoint_save(0)
    assert A.lib() is not None


def test_dropin_chpoint_save_and_load(tmp_path):
    """-chpoint 0s (type always) with -maxiter 4 writes chp.0 equal to the oracle's state; -chp_load resumes it and
    prints the history from RE_005 on"""
    import adda_gb300 as A
    from test_gpu_dropin import build_mock
    A.lib()
    exe = build_mock()
    d = str(tmp_path / "chp")
    out = tmp_path / "res.bin"
    grid, m = CHP["setup"]["grid"], CHP["setup"]["m"]
    base = [exe, str(grid), str(m[0]), str(m[1]), "15", "qmr", "10", str(out)]
    p = subprocess.run(base + ["chpoint", d, "always", "0", "4"], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "Checkpoint (iteration) saved" in p.stdout
    assert open(os.path.join(d, "chp.log")).read().startswith("Info about the run")
    raw = open(os.path.join(d, "chp.0"), "rb").read()
    s = setup_for(dict(grid=grid, m=complex(*m), dpl=15))
    o = oracle_for(s)
    r = oracle_solve(o, s, 0, eps=1e-10, maxiter=4, chp_save=True)
    compare_state(raw, r["chp"], "qmr", 1e-9)
    p = subprocess.run(base + ["chp_load", d], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "Checkpoint (iteration) loaded" in p.stdout and "RE_005" in p.stdout and "RE_004" not in p.stdout
    full = oracle_solve(o, s, 0, eps=1e-10)
    resumed = np.frombuffer(open(out, "rb").read()[20:], np.complex128)[:3 * s.n]
    assert rel(resumed, full["p"]) < 1e-8

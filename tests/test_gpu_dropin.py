"""The drop-in layer (the reference's InitDmatrix / MatVec / IterativeSolver signatures over the C ABI) driven by a
stand-in host that defines the reference's globals: its pvec and MatVec match the C-ABI results, and its FP64 solve
matches the oracle's cross section."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from helpers import oracle_for, oracle_solve, setup_for

pytestmark = pytest.mark.gpu

BUILD = os.path.join(ROOT, "a-dda_gb300", "_build")


def build_mock():
    exe = os.path.join(BUILD, "mock_host")
    inc = os.path.join(ROOT, "include")
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-fcommon", "-I", inc, "-o", exe,
                    os.path.join(ROOT, "tests", "dropin", "mock_host.c"),
                    os.path.join(ROOT, "tests", "dropin", "mock_crosssec.c"),
                    os.path.join(ROOT, "a-dda_gb300", "csrc", "dropin", "adda_dropin.c"),
                    "-L" + BUILD, "-ladda_gb300", "-Wl,-rpath," + BUILD, "-Wl,--wrap=CalcField", "-Wl,--wrap=CalcAlldir",
                    "-Wl,--wrap=CalcScatGrid", "-lm"], check=True)
    return exe


@pytest.mark.parametrize("method", ["qmr", "bicgstab", "bicg", "cgnr", "csym", "qmr2", "bcgs2"])
def test_dropin_solve_and_matvec(tmp_path, method):
    import adda_gb300 as A
    A.lib()
    exe = build_mock()
    out = tmp_path / "res.bin"
    p = subprocess.run([exe, "16", "1.5", "0", "10", method, "10", str(out)], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "RE_000" in p.stdout and "Final (recalculated) residual norm" in p.stdout
    raw = open(out, "rb").read()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    niter = int(np.frombuffer(raw[8:12], np.int32)[0])
    ip = float(np.frombuffer(raw[12:20], np.float64)[0])
    vec = np.frombuffer(raw[20:], np.complex128)
    pv, y, fields = vec[:3 * n], vec[3 * n:6 * n], vec[6 * n:6 * n + 9].reshape(3, 3)
    e2 = np.frombuffer(raw[20 + 16 * (6 * n + 9):20 + 16 * (6 * n + 9) + 160], np.float64)
    egrid = np.frombuffer(raw[20 + 16 * (6 * n + 9) + 160:], np.complex128).reshape(3, 2)
    s = setup_for(dict(grid=16, m=1.5, dpl=10))
    assert n == s.n
    o = oracle_for(s)
    r = oracle_solve(o, s, 0, method=method, eps=1e-10)
    ce, _ = o.cross(pv, s.prop, s.incpol[0])
    assert abs(ce / r["Cext"] - 1) < 1e-9
    # at eps = 1e-10 the Lanczos-type methods move by a few iterations under rounding differences (BiCG_CS: 69 vs
    # 74 measured); CGNR/CSYM have their own stagnation exits
    assert abs(niter - r["niter"]) <= max(3, 0.1 * r["niter"]) or method in ("cgnr", "csym")
    o.set_cc(s.cc[0].reshape(1, 3))
    yr, ipr = o.matvec(s.einc[0])
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < 1e-13
    assert abs(ip / ipr - 1) < 1e-12
    # CalcField through the link-time wrapper, on the GPU, against the oracle's field of the same polarisations
    for d, n_ in enumerate([s.prop, (0.6, 0.0, 0.8), (0.0, -1.0, 0.0)]):
        eo = o.field(pv, np.asarray(n_, dtype=float))
        assert np.linalg.norm(fields[d] - eo) <= 1e-12 * np.linalg.norm(eo), (d, fields[d], eo)
    # CalcAlldir through its wrapper: |E|^2 on a 5 x 4 grid of beam-frame directions in one GPU batch
    k = 0
    for th in (180, 120, 90, 60, 0):
        for ph in (0, 90, 180, 270):
            t, f = np.deg2rad(th), np.deg2rad(ph)
            dirn = np.cos(t) * s.prop + np.sin(t) * (np.cos(f) * s.incpol[1] + np.sin(f) * s.incpol[0])
            eo = o.field(pv, dirn)
            assert abs(e2[k] / np.sum(np.abs(eo) ** 2) - 1) < 1e-12, (th, ph, e2[k])
            k += 1
    # CalcScatGrid through its wrapper: E projected on Eper = robs x prop/|..| and Epar = robs x Eper (pairs)
    for k, (th, ph) in enumerate(((30, 10), (90, 200), (150, 300))):
        t, f = np.deg2rad(th), np.deg2rad(ph)
        dirn = np.cos(t) * s.prop + np.sin(t) * (np.cos(f) * s.incpol[1] + np.sin(f) * s.incpol[0])
        per = np.cross(dirn, s.prop)
        per /= np.linalg.norm(per)
        par = np.cross(dirn, per)
        eo = o.field(pv, dirn)
        want = np.array([eo @ per, eo @ par])
        assert np.linalg.norm(egrid[k] - want) <= 1e-12 * np.linalg.norm(eo), (th, ph, egrid[k], want)


def _run_mock(tmp_path, extra, eps="10"):
    exe = build_mock()
    out = tmp_path / "res.bin"
    p = subprocess.run([exe, "16", "1.5", "0", "10", "qmr", eps, str(out), *extra], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    raw = open(out, "rb").read()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    niter = int(np.frombuffer(raw[8:12], np.int32)[0])
    return p.stdout, n, niter, np.frombuffer(raw[20:], np.complex128)[:3 * n]


def test_dropin_init_field_wkb(tmp_path):
    """-init_field wkb: the drop-in computes the WKB field on the host, turns it into x_0 (InitFieldfromE) and the
    GPU solve from there ends at the oracle's solution from the same start"""
    import adda_gb300 as A
    from helpers import wkb_x0
    A.lib()
    out, n, niter, pv = _run_mock(tmp_path, ["wkb"])
    assert "x_0 = result of WKB" in out
    s = setup_for(dict(grid=16, m=1.5, dpl=10))
    o = oracle_for(s)
    r = oracle_solve(o, s, 0, eps=1e-10, init="x0", x0=wkb_x0(s, 0))
    # the starting residual is the oracle's to the printed digits
    re0 = float(out.split("RE_000 = ")[1].split()[0])
    assert abs(re0 / r["resid"][0] - 1) < 1e-9, (re0, r["resid"][0])
    assert abs(niter - r["niter"]) <= max(3, 0.1 * r["niter"])
    ce, _ = o.cross(pv, s.prop, s.incpol[0])
    assert abs(ce / r["Cext"] - 1) < 1e-9


def test_dropin_init_field_read(tmp_path):
    """-init_field read: a field file holding the converged internal field E = chi_inv p makes the solve stop at
    iteration 0 with the same polarisation"""
    import adda_gb300 as A
    A.lib()
    s = setup_for(dict(grid=16, m=1.5, dpl=10))
    o = oracle_for(s)
    r = oracle_solve(o, s, 0, eps=1e-12)
    chi_inv = 4 * np.pi / (s.gridspace ** 3 * (1.5 ** 2 - 1))
    f = tmp_path / "field.bin"
    (chi_inv * r["p"]).astype(np.complex128).tofile(f)
    out, n, niter, pv = _run_mock(tmp_path, ["read", str(f)])
    assert "x_0 = from file " + str(f) in out
    assert niter == 0, out
    assert np.linalg.norm(pv - r["p"]) <= 1e-10 * np.linalg.norm(r["p"])


def test_dropin_surface(tmp_path):
    """-surf 2 2 0.5 -int_surf img through the drop-in: the reflected tensor comes from the host's ReflTerm_int
    (HOST relation); pvec and the surface matvec equal the oracle's (Y polarisation, beam from the substrate)"""
    import adda_gb300 as A
    A.lib()
    exe = build_mock()
    out = tmp_path / "res.bin"
    p = subprocess.run([exe, "8", "1.5", "0.1", "15", "qmr", "10", str(out), "surf", "2", "2", "0.5"],
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    raw = open(out, "rb").read()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    vec = np.frombuffer(raw[20:], np.complex128)
    pv, y = vec[:3 * n], vec[3 * n:6 * n]
    s = A.Setup(grid=8, m=1.5 + 0.1j, dpl=15, surface=dict(h=2.0, msub=2 + 0.5j, relation="img"))
    assert n == s.n
    o = oracle_for(s)
    r = oracle_solve(o, s, 0, eps=1e-10)
    assert np.linalg.norm(pv - r["p"]) / np.linalg.norm(r["p"]) < 1e-9
    o.set_cc(s.cc[0].reshape(1, 3))
    yr, _ = o.matvec(s.einc[0])
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < 1e-13


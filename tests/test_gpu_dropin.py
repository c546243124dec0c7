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
                    "-L" + BUILD, "-ladda_gb300", "-Wl,-rpath," + BUILD, "-Wl,--wrap=CalcField", "-lm"], check=True)
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
    pv, y, fields = vec[:3 * n], vec[3 * n:6 * n], vec[6 * n:].reshape(3, 3)
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

"""The 128^3 sphere workload at full size against the reference's own run of it (tests/golden/reference_c2.json,
made by tests/golden/make_reference_c2.py): inputs on the CPU, solves on the GPU.

At eps = 1e-5 a solution is only determined to the residual: the reference's two methods themselves differ by up to
4e-6 in Cext and 1e-5 in Cabs for the X polarisation (5377.4954 QMR_CS against 5377.4755 BiCGStab), and its QMR_CS
run is 6e-6 from the converged Cabs. The mixed solves are therefore held to two bars: within 1e-6 of the converged
cross sections of the reference's own solve to residual 1e-8 (reference_c2_converged.json, the spec accuracy
bar), and within 1e-5 of its runs at eps 1e-5. They must meet the FP64 residual, and take between 0.85 and 1.3 times
the reference's iterations to 1e-5 (the mixed refinement stops at 0.3 eps for QMR_CS and 0.1 eps for BiCGStab, for
the accuracy of the cross sections).
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REF = json.load(open(os.path.join(HERE, "golden", "reference_c2.json")))


def setup():
    import adda_gb300 as A
    return A.Setup(grid=128, m=1.33 + 0.01j, dpl=15)


def test_c2_inputs_match_reference():
    s = setup()
    runs = list(REF["runs"].values())
    conv = os.path.join(HERE, "golden", "reference_c2_converged.json")
    if os.path.exists(conv):
        runs += list(json.load(open(conv))["runs"].values())
    for run in runs:
        assert run["ndip"] == s.n
        assert tuple(run["box"]) == tuple(s.box)
        assert tuple(run["grid"]) == tuple(s.grid)
        for pol, cc in zip("YX", run["cc"]):
            got = s.cc[0 if pol == "Y" else 1][0]
            assert abs(got - complex(*cc)) <= 1e-9 * abs(got)


def test_c2_converged_reference_is_converged():
    """the two methods of the reference's residual-1e-8 runs agree to 1e-8 (so their mean is a converged bar for 1e-6
    checks), and each is within 1e-5 of the same method's eps-1e-5 run"""
    conv = os.path.join(HERE, "golden", "reference_c2_converged.json")
    if not os.path.exists(conv):
        pytest.skip("no converged fixture")
    c = json.load(open(conv))
    assert c["converged"]["spread"]["Cext"] < 1e-8 and c["converged"]["spread"]["Cabs"] < 1e-8
    for m, run in c["runs"].items():
        assert run["resid_final"]["Y"] <= 1e-8
        for q in ("Cext", "Cabs"):
            assert abs(run["cross"]["Y"][q] / REF["runs"][m]["cross"]["Y"][q] - 1) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["qmr", "bicgstab"])
def test_c2_mixed_solve_matches_reference(method):
    import torch

    import adda_gb300 as A
    s = setup()
    ctx = A.Context.from_setup(s, nrhs_max=2)
    d_e = torch.from_numpy(np.ascontiguousarray(np.stack(s.einc)).view(np.float64)).cuda()
    d_x = torch.empty_like(d_e)
    d_p = torch.empty_like(d_e)
    st = ctx.solve_device(d_e.data_ptr(), 2, d_x.data_ptr(), d_p.data_ptr(), method=method, prec="mixed", eps=1e-5)
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    ref = REF["runs"][method]
    for r, pol in enumerate("YX"):
        assert st[r]["status"] == "ok" and st[r]["resid"] <= 1e-5
        assert abs(ce[r] / ref["cross"][pol]["Cext"] - 1) < 1e-5, (pol, ce[r], ref["cross"][pol])
        assert abs(ca[r] / ref["cross"][pol]["Cabs"] - 1) < 1e-5, (pol, ca[r], ref["cross"][pol])
        assert 0.85 < st[r]["niter"] / ref["niter"][pol] < 1.3, (pol, st[r]["niter"], ref["niter"][pol])
    conv = os.path.join(HERE, "golden", "reference_c2_converged.json")
    if os.path.exists(conv):
        c = json.load(open(conv))["converged"]
        for r in range(2):
            assert abs(ce[r] / c["Cext"] - 1) < 1e-6, (r, ce[r], c["Cext"])
            assert abs(ca[r] / c["Cabs"] - 1) < 1e-6, (r, ca[r], c["Cabs"])
    ctx.close()

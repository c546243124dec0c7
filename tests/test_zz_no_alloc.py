"""adda_gb300_cross_sections_noalloc: the cross sections computed without any allocation (partial sums in the
library's static device array), for callers that cannot call cudaMalloc at that point (a framework owning all device
memory through its own pool allocator, a plugin whose host forbids device allocation after start-up). Checked
through the C ABI against the context-based adda_gb300_cross_sections on two calls in a row that differ (the static
array keeps the previous call's contents: the second call has one right-hand side and doubled polarisations, so
Cext doubles and Cabs quadruples), in per-material mode with and without a material array and in per-dipole mode,
plus the size limit. Runs alone in a fresh process or after the other tests."""
import ctypes

import numpy as np
import pytest

from helpers import case, setup_for

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the bar of the existing cross-section test (same sums, different block partition)


def _dev(t):
    return ctypes.c_void_p(t.data_ptr())


def _call(L, R, s, d_p, d_pos, d_mat, d_cc, nmat, per_dip, d_prop, d_inc, d_ce, d_ca):
    return L.adda_gb300_cross_sections_noalloc(R, s.n, _dev(d_p), _dev(d_pos), _dev(d_mat) if d_mat is not None
                                               else None, _dev(d_cc), nmat, per_dip, *s.box, s.gridspace, s.wavenum,
                                               _dev(d_prop), _dev(d_inc), _dev(d_ce), _dev(d_ca), None)


@pytest.mark.parametrize("per_dip,with_mat", [(0, True), (0, False), (1, False)])
def test_noalloc_matches_context_cross_sections(per_dip, with_mat):
    import torch

    import adda_gb300 as A
    L = A.lib()
    s = setup_for(case("prop_ell")["setup"])
    ctx = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max=2)
    ctx.init_dmatrix()
    cc = np.stack([s.cc[0], s.cc[1]])                       # [2][3], one material
    if per_dip:
        ccd = np.stack([np.tile(s.cc[r], (s.n, 1)) for r in range(2)])   # [2][N][3]
        for r in range(2):
            ctx.set_cc_dipole(r, ccd[r])
    else:
        for r in range(2):
            ctx.set_cc(r, cc[r].reshape(1, 3))
    res = ctx.solve(np.stack(s.einc), prec="fp64", eps=1e-8)
    prop = np.stack([s.prop, s.prop])
    inc = np.stack(s.incpol)
    ce_ref, ca_ref = ctx.cross_sections(prop, inc)
    dev = "cuda"
    d_p = torch.from_numpy(np.ascontiguousarray(res["p"]).view(np.float64)).to(dev)
    d_pos = torch.from_numpy(np.ascontiguousarray(s.pos.astype(np.int16))).to(dev)
    d_mat = torch.from_numpy(np.ascontiguousarray(s.mat.astype(np.int8))).to(dev) if with_mat else None
    cc_in = ccd if per_dip else cc.reshape(2, 1, 3)
    d_cc = torch.from_numpy(np.ascontiguousarray(cc_in).view(np.float64)).to(dev)
    d_prop = torch.from_numpy(prop.copy()).to(dev)
    d_inc = torch.from_numpy(inc.copy()).to(dev)
    # call 0: both right-hand sides as solved; call 1: only the first, with its polarisations doubled (Cext is
    # linear in P, Cabs quadratic), so stale partial sums of call 0 would show
    for call, (R, scale) in enumerate([(2, 1.0), (1, 2.0)]):
        d_ce = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
        d_ca = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
        d_pc = d_p * scale if scale != 1.0 else d_p
        rc = _call(L, R, s, d_pc, d_pos, d_mat, d_cc, 1, per_dip, d_prop, d_inc, d_ce, d_ca)
        assert rc == 0, L.adda_gb300_last_error().decode()
        torch.cuda.synchronize()
        ce, ca = d_ce.cpu().numpy(), d_ca.cpu().numpy()
        for r in range(R):
            assert abs(ce[r] / (scale * ce_ref[r]) - 1) < TOL, (call, r, ce[r], ce_ref[r])
            assert abs(ca[r] / (scale * scale * ca_ref[r]) - 1) < TOL, (call, r, ca[r], ca_ref[r])
        assert np.isnan(ce[R:]).all() and np.isnan(ca[R:]).all()   # nothing written beyond nrhs


def test_noalloc_rejects_too_many_rhs():
    import torch

    import adda_gb300 as A
    L = A.lib()
    s = setup_for(case("mgn")["setup"])
    t = torch.zeros(16, dtype=torch.float64, device="cuda")
    too_many = 65
    rc = L.adda_gb300_cross_sections_noalloc(too_many, s.n, _dev(t), _dev(t), None, _dev(t), 1, 0, *s.box,
                                             s.gridspace, s.wavenum, _dev(t), _dev(t), _dev(t), _dev(t), None)
    assert rc == -1
    assert "ADDA_GB300_NOALLOC_MAX_RHS" in L.adda_gb300_last_error().decode()

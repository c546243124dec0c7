"""The differentiation workload's inputs (tests/c4_workload.py) on the CPU: the seeded smooth fields, the refractive
index range, the quantisation onto 14 materials and the finite-difference dipoles; and its agreement with the
reference's own reading of the quantised field (dipole count, box, grid, dpl, the 28 coupling constants)."""
import json
import os

import numpy as np

import c4_workload as W

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fields_and_index_range():
    u1, u2 = W.fields()
    assert u1.shape == u2.shape == (W.BOX ** 3,)
    for u in (u1, u2):
        assert 0 < u.min() and u.max() < 1 and abs(u.mean() - 0.5) < 0.05
    m = W.refractive_index(u1, u2)
    assert 1.3 < m.real.min() and m.real.max() < 1.7 and 0 < m.imag.min() and m.imag.max() < 0.05
    # smooth: neighbouring cells along x are strongly correlated (sigma = 4 dipoles)
    g = u1.reshape(W.BOX, W.BOX, W.BOX)
    assert np.corrcoef(g[:, :, :-1].ravel(), g[:, :, 1:].ravel())[0, 1] > 0.9
    assert abs(W.chi_of(m[0]) - (m[0] ** 2 - 1) / (4 * np.pi)) < 1e-15


def test_quantised_materials_and_fd_dipoles():
    u1, u2 = W.fields()
    mat, levels = W.quantised(u1, u2)
    assert mat.max() == 13 and len(levels) == 14 and len(np.unique(mat)) == 14
    m = W.refractive_index(u1, u2)
    assert np.abs(levels[mat] - m).max() < 0.4 / 7 / 2 + 0.05 / 2 / 2 + 1e-12
    js = W.fd_dipoles(W.BOX ** 3)
    assert len(js) == 256 and len(np.unique(js)) == 256 and js.max() < W.BOX ** 3


def test_quantised_geometry_matches_reference_run(adda):
    run = json.load(open(os.path.join(HERE, "golden", "reference_c4_quantised.json")))["run"]
    u1, u2 = W.fields()
    _, levels = W.quantised(u1, u2)
    s = adda.Setup(grid=W.BOX, shape="box", m=complex(levels[np.argmax(np.abs(levels))]), dpl=W.default_dpl(levels))
    assert s.n == run["ndip"] and list(s.box) == run["box"] and list(s.grid) == run["grid"]
    assert abs(s.dpl / run["dpl"] - 1) < 1e-5  # the log prints dpl to 6 digits
    # the coupling constants the reference printed per material (Y polarisation, then X)
    for r in range(2):
        for k, m in enumerate(levels):
            cc = adda.polarizability(m, s.kd, s.gridspace, s.prop, s.incpol[r], "ldr")[0]
            ref = complex(*run["cc"][14 * r + k])
            assert abs(cc / ref - 1) < 1e-9, (r, k, cc, ref)

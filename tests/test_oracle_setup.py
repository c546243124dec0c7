"""The oracle's numpy restatement of the reference host's inputs (oracle/setup.py, used by bench.py's CPU arm so that
it never loads the GPU library) builds the same lattice, grid, plane waves and LDR coupling constants as the
library's host code, and the bench workload's sizes and coupling constant agree with the reference's own run of it."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle import setup as OS

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("grid,m,dpl", [(16, 1.5, 10.0), (24, 1.33 + 0.01j, 15.0), (128, 1.33 + 0.01j, 15.0)])
def test_sphere_workload_matches_library_setup(adda, grid, m, dpl):
    s = adda.Setup(grid=grid, m=m, dpl=dpl)
    w = OS.SphereWorkload(grid, m, dpl, O.lib().or_fftfit)
    assert tuple(w.box) == tuple(s.box) and tuple(w.grid) == tuple(s.grid) and w.n == s.n
    assert np.array_equal(w.pos, s.pos)
    for r in range(2):
        assert np.allclose(w.cc[r], s.cc[r], rtol=1e-14, atol=0)
        assert np.allclose(w.einc[r], s.einc[r], rtol=0, atol=1e-14)


@pytest.mark.parametrize("shape,pars,box", [("ellipsoid", (0.7, 0.8), 24), ("box", (0.5, 1.0), 10),
                                            ("ellipsoid", (0.55, 0.93), 32)])
def test_lattice_shapes_match_library(adda, shape, pars, box):
    s = adda.Setup(grid=box, shape=shape, pars=pars, m=1.4)
    b = OS.fit_box(shape, box, pars)
    assert tuple(b) == tuple(s.box)
    assert np.array_equal(OS.lattice(shape, b, pars), s.pos)


def test_bench_workload_matches_reference_run():
    ref = json.load(open(os.path.join(HERE, "golden", "reference_c2.json")))["runs"]["qmr"]
    w = OS.SphereWorkload(128, 1.33 + 0.01j, 15.0, O.lib().or_fftfit)
    assert w.n == ref["ndip"] and list(w.box) == ref["box"] and list(w.grid) == ref["grid"]
    for r, pol in enumerate("YX"):
        got = w.cc[r][0]
        assert abs(got - complex(*ref["cc"][r])) <= 1e-9 * abs(got)

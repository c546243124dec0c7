"""The C-ABI library loads without a GPU and exports every entry point include/adda_gb300.h declares; the host-side
setup functions (no GPU) behave like the reference's; GPU entry points fail cleanly when no GPU is present."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, have_gpu


def declared():
    txt = open(os.path.join(ROOT, "include", "adda_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(adda_gb300_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(adda):
    L = ctypes.CDLL(adda.LIB_PATH)
    names = declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(adda.EXPORTS)


def test_fftfit_matches_reference_rule(adda):
    # fftFit (fft.c:528-562): even, divisible by divis, 2^a 3^b 5^c 7^d (11|13)^{0,1}
    for x, d, want in [(32, 1, 32), (34, 1, 36), (44, 1, 44), (46, 1, 48), (50, 2, 50), (54, 2, 54), (242, 1, 250),
                       (256, 2, 256), (512, 1, 512), (14, 1, 14), (22, 1, 22), (26, 1, 26), (286, 1, 288)]:
        assert adda.fft_fit(x, d) == want, (x, d)


def test_particle_counts(adda):
    # occupied-dipole counts printed by the reference for the benchmark workloads (log / prognosis)
    for shape, grid, pars, n in [("sphere", 16, None, 2176), ("sphere", 128, None, 1099136),
                                 ("ellipsoid", 24, (0.7, 0.8), 4032), ("box", 48, None, 110592)]:
        box, pos, mat = adda.make_particle(shape, grid, pars)
        assert len(pos) == n
        # z-major, then y, then x: the order the device lattice requires
        key = (pos[:, 2].astype(np.int64) * box[1] + pos[:, 1]) * box[0] + pos[:, 0]
        assert np.all(np.diff(key) > 0)


def test_rotation_default_and_prop(adda):
    prop, py, px = adda.rotation()
    np.testing.assert_allclose(prop, [0, 0, 1])
    np.testing.assert_allclose(py, [0, 1, 0])
    np.testing.assert_allclose(px, [1, 0, 0])
    prop, py, px = adda.rotation(10, 20, 30, prop0=(1, 2, 3))
    for v in (prop, py, px):
        assert abs(np.linalg.norm(v) - 1) < 1e-14
    assert abs(prop @ py) < 1e-14 and abs(prop @ px) < 1e-14 and abs(px @ py) < 1e-14


@pytest.mark.skipif(have_gpu(), reason="checks the no-GPU error path")
def test_create_fails_loudly_without_gpu(adda):
    box, pos, mat = adda.make_particle("sphere", 8)
    with pytest.raises(adda.AddaError):
        adda.Context(box, pos, mat, 0.5, 1.0)


def test_create_group_rejects_bad_arguments(adda):
    """adda_gb300_create_group checks its description before touching a device (EINVAL = -1)"""
    L = adda.lib()
    box, pos, mat = adda.make_particle("sphere", 8)
    pr = adda.Problem(box[0], box[1], box[2], 0, 0, 0, 0, None, None, 0.5, 1.0, 2, 0, 0, 0.0)
    nd = (ctypes.c_size_t * 1)(len(pos))
    pp = (ctypes.c_void_p * 1)(pos.ctypes.data)
    h = ctypes.c_void_p()
    assert L.adda_gb300_create_group(ctypes.byref(pr), 0, nd, pp, None, ctypes.byref(h)) == -1    # no particle
    assert L.adda_gb300_create_group(ctypes.byref(pr), 1, None, pp, None, ctypes.byref(h)) == -1  # no counts
    bad = adda.Problem(0, box[1], box[2], 0, 0, 0, 0, None, None, 0.5, 1.0, 2, 0, 0, 0.0)
    assert L.adda_gb300_create_group(ctypes.byref(bad), 1, nd, pp, None, ctypes.byref(h)) == -1   # empty box
    assert not h.value


def test_host_functions_reject_bad_arguments(adda):
    """the host-side entry points return the reference's error cases as status codes instead of aborting"""
    L = adda.lib()
    prop = np.array([0.0, 0.0, 1.0])
    pol = np.array([0.0, 1.0, 0.0])
    cc = np.zeros(6)
    p = prop.ctypes.data_as(ctypes.c_void_p)
    q = pol.ctypes.data_as(ctypes.c_void_p)
    c = cc.ctypes.data_as(ctypes.c_void_p)
    assert L.adda_gb300_polarizability(99, 1.5, 0.0, 0.6, 0.1, p, q, 0, c) == -1       # unknown -pol
    assert L.adda_gb300_polarizability_nloc(9, 1.5, 0.0, 0.1, -1.0, c) == -1          # negative Gaussian width
    assert L.adda_gb300_polarizability_nloc(0, 1.5, 0.0, 0.1, 0.2, c) == -1           # not an nloc relation
    by, bz = ctypes.c_int(), ctypes.c_int()
    assert L.adda_gb300_fit_box(7, None, 16, ctypes.byref(by), ctypes.byref(bz)) != 0  # unknown shape
    # alldir parameters the reference's ScanIntegrParms rejects
    for bad in (dict(min=10.0, max=5.0), dict(Jmin=0), dict(Jmax=1, Jmin=2), dict(eps=-1.0), dict(max=190.0)):
        prm = dict(adda.ALLDIR_DEFAULT[0])
        prm.update(bad)
        with pytest.raises(adda.AddaError):
            adda.integr_points(prm, True)
    assert len(adda.integr_points(adda.ALLDIR_DEFAULT[0], True)) == 65      # 2^6 + 1 values of cos(theta)
    assert len(adda.integr_points(adda.ALLDIR_DEFAULT[1], False)) == 32     # 2^5 + 1 - 1 (min == max direction)

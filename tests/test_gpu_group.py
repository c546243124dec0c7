"""Several particles in one group context (adda_gb300_create_group): every stage of the matvec and of the solve runs
once for all particles' right-hand sides. Checked against one context per particle: the FP64 matvec of random
vectors (1e-13), FP64 solves of both polarisations to residual 1e-10 (solutions 1e-8, cross sections 1e-9), the
mixed solve (cross sections within 1e-6 of the FP64 single-particle solves), the zero padding of the smaller
particles' vectors, and the refusal of the single-lattice features (VJP, checkpoints)."""
import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu


def _setups():
    import adda_gb300 as A
    return [A.Setup(grid=16, m=1.5, dpl=10),
            A.Setup(grid=12, shape="ellipsoid", pars=(0.8, 0.6), m=1.33 + 0.01j, dpl=10),
            A.Setup(grid=10, shape="box", m=1.3 + 0.05j, dpl=10)]


def _stack(g, setups, per_particle):
    return np.concatenate([g.group_pad(per_particle(q, s), q) for q, s in enumerate(setups)])


def test_group_matvec_equals_single_particles():
    import adda_gb300 as A
    setups = _setups()
    g = A.Context.group(setups, rhs_per_particle=2)
    rng = np.random.default_rng(3)
    xs = [rng.standard_normal((2, 3 * s.n)) + 1j * rng.standard_normal((2, 3 * s.n)) for s in setups]
    y, _ = g.matvec(_stack(g, setups, lambda q, s: xs[q]), "fp64")
    for q, s in enumerate(setups):
        c = A.Context.from_setup(s, nrhs_max=2)
        y1, _ = c.matvec(xs[q], "fp64")
        for k in range(2):
            r = 2 * q + k
            assert rel(y[r][:3 * s.n], y1[k]) < 1e-13, (q, k)
            assert not np.any(y[r][3 * s.n:]), "padding of a smaller particle must stay zero"
        c.close()
    g.close()


def _einc(g, setups):
    # incident fields with the common box's centre as phase reference
    return np.concatenate([np.stack([g.group_plane_wave(q, s.prop, e) for e in s.incpol]) for q, s in enumerate(setups)])


@pytest.mark.parametrize("method", ["qmr", "bicgstab"])
def test_group_solve_equals_single_particles(method):
    import adda_gb300 as A
    setups = _setups()
    g = A.Context.group(setups, rhs_per_particle=2)
    E = _einc(g, setups)
    props = np.stack([s.prop for s in setups for _ in range(2)])
    incs = np.stack([e for s in setups for e in s.incpol])
    res = g.solve(E, method=method, prec="fp64", eps=1e-10)
    ce, ca = g.cross_sections(props, incs)
    resm = g.solve(E, method=method, prec="mixed", eps=1e-5)
    cem, cam = g.cross_sections(props, incs)
    for q, s in enumerate(setups):
        c = A.Context.from_setup(s, nrhs_max=2)
        r1 = c.solve(np.stack(s.einc), method=method, prec="fp64", eps=1e-10)
        ce1, ca1 = c.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
        for k in range(2):
            r = 2 * q + k
            assert res["stats"][r]["status"] == "ok" and resm["stats"][r]["status"] == "ok", (q, k)
            # the same solution up to the constant phase between the two reference points
            j = int(np.argmax(np.abs(s.einc[k])))
            ph = E[r][j] / s.einc[k][j]
            assert abs(abs(ph) - 1) < 1e-12 and np.allclose(E[r][:3 * s.n], ph * s.einc[k], rtol=0, atol=1e-12)
            assert rel(res["x"][r][:3 * s.n], ph * r1["x"][k]) < 1e-8, (q, k)
            assert not np.any(res["x"][r][3 * s.n:]) and not np.any(res["p"][r][3 * s.n:])
            assert abs(ce[r] / ce1[k] - 1) < 1e-9 and abs(ca[r] - ca1[k]) < 1e-9 * max(abs(ca1[k]), abs(ce1[k]))
            assert abs(cem[r] / ce1[k] - 1) < 1e-6, (q, k, cem[r], ce1[k])
            assert abs(cam[r] - ca1[k]) < 1e-6 * max(abs(ca1[k]), abs(ce1[k])), (q, k, cam[r], ca1[k])
        c.close()
    g.close()


def test_group_refuses_single_lattice_features():
    import adda_gb300 as A
    setups = _setups()
    g = A.Context.group(setups, rhs_per_particle=2)
    g.solve(_einc(g, setups), method="qmr", prec="fp64", eps=1e-6)
    with pytest.raises(A.AddaError):
        g.vjp_chi(0, setups[0].prop, setups[0].incpol[0], np.ones(g.n, complex))
    with pytest.raises(A.AddaError):
        g.chpoint_save(0)
    g.close()

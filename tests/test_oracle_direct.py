"""The oracle's FFT-based matvec against a dense O(N^2) evaluation of A = I + S.D.S for a small particle, with the
point-dipole Green's tensor (interaction.c:290-331) written out independently in numpy."""
import numpy as np

from helpers import oracle_for, setup_for


def green(r, k):
    """G(r) for one offset vector r (real units), as a 3x3 complex matrix"""
    rr = np.linalg.norm(r)
    q = r / rr
    kr = k * rr
    ev = np.exp(1j * kr) / rr ** 3
    qq = np.outer(q, q)
    return ev * ((3 - kr * kr - 3j * kr) * qq + (kr * kr - 1 + 1j * kr) * np.eye(3))


def dense_matrix(s, cc):
    n = s.n
    pos = s.pos.astype(float) * s.gridspace
    A = np.eye(3 * n, dtype=complex)
    sq = np.sqrt(cc)
    for i in range(n):
        for j in range(n):
            if i != j:
                A[3 * i:3 * i + 3, 3 * j:3 * j + 3] -= sq[:, None] * green(pos[i] - pos[j], s.wavenum) * sq[None, :]
    return A


def test_oracle_matvec_equals_dense():
    s = setup_for(dict(grid=6, shape="ellipsoid", pars=(0.7, 1.4), m=1.4 + 0.1j, dpl=9))
    assert 20 < s.n < 200
    o = oracle_for(s)
    o.set_cc(s.cc[0].reshape(1, 3))
    A = dense_matrix(s, s.cc[0])
    rng = np.random.default_rng(1)
    x = rng.standard_normal(3 * s.n) + 1j * rng.standard_normal(3 * s.n)
    y, ip = o.matvec(x)
    yd = A @ x
    assert np.linalg.norm(y - yd) / np.linalg.norm(yd) < 1e-13
    assert abs(ip / np.vdot(yd, yd).real - 1) < 1e-12
    yh, _ = o.matvec(x, her=True)
    yhd = A.conj().T @ x
    assert np.linalg.norm(yh - yhd) / np.linalg.norm(yhd) < 1e-13
    assert np.allclose(A, A.T)  # complex symmetric

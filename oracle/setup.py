"""The reference host's inputs to the hot path for the bench workload, restated in numpy.

TEST INFRASTRUCTURE (oracle): used by bench.py's CPU leg (`--impl reference`, `cpu_baseline`) and by tests/ to
build the particle, the incident plane waves and the coupling constants without loading the GPU library, so that the
timed CPU run touches nothing but the oracle. Restated from the reference (ADDA 1.3b6, paths within its project):

    sphere / ellipsoid lattice   MakeParticle box loop, jagged = 1     src/make_particle.c:1979-2030 (shape tests
                                                                      SH_SPHERE :1752, SH_ELLIPSOID)
    box sizes                    InitShape + FitBox_yz                 src/make_particle.c:1283-1308,1912-1919
    FFT grid                     ParSetup: fftFit(2*box), gridZ even   src/comm.c:489-491 (fftFit: the oracle's own)
    incident frame               prop_0 = (0,0,1), incPolY/X           src/param.c:1988-1989,2116-2131
    plane wave                   GenerateB, free space                 src/GenerateB.c:324-328
    LDR coupling constant        CoupleConstant / pol3coef             src/calculator.c:118-132,214-222
"""
import math

import numpy as np

# LDR coefficients of the reference (src/const.h:234-236)
LDR_B1, LDR_B2, LDR_B3 = 1.8915316, -0.1648469, 1.7700004


def fit_box(shape, box_x, pars=None):
    """(boxX, boxY, boxZ): FitBox_yz with jagged = 1, 2*floor((ratio*boxX + 1)/2) and at least 2"""
    yx, zx = (1.0, 1.0) if shape == "sphere" or pars is None else pars

    def fit(v):
        return max(2, 2 * int(math.floor((v * box_x + 1) / 2)))
    return box_x, fit(yx), fit(zx)


def lattice(shape, box, pars=None):
    """positions [N,3] uint16 of the occupied cells, z outermost and x fastest (the reference's order); the cell centre
    relative to the box centre, in units of boxX, must satisfy the shape test"""
    bX, bY, bZ = box
    k, j, i = np.meshgrid(np.arange(bZ), np.arange(bY), np.arange(bX), indexing="ij")
    xr = (i - bX // 2 + 0.5) / bX
    yr = (j - bY // 2 + 0.5) / bX
    zr = (k - bZ // 2 + 0.5) / bX
    if shape == "sphere":
        inside = xr * xr + yr * yr + zr * zr <= 0.25
    elif shape == "ellipsoid":
        a, b = pars
        inside = xr * xr + yr * yr / (a * a) + zr * zr / (b * b) <= 0.25
    elif shape == "box":
        a, b = pars if pars is not None else (1.0, 1.0)
        inside = (np.abs(yr) <= a / 2) & (np.abs(zr) <= b / 2)
    else:
        raise ValueError(shape)
    return np.stack([i[inside], j[inside], k[inside]], axis=1).astype(np.uint16)


def plane_wave(box, pos, gridspace, wavenum, prop, pol):
    """Einc = pol * exp(i k r.prop) at the dipole centres (origin at the box centre): complex [3N]"""
    c = (np.asarray(box, float) - 1) / 2
    r = (pos.astype(np.float64) - c) * gridspace
    ph = wavenum * (r @ np.asarray(prop, float))
    e = (np.cos(ph) + 1j * np.sin(ph))[:, None] * np.asarray(pol, float)[None, :]
    return e.reshape(-1)


def ldr_cc(m, kd, gridspace, prop, pol):
    """LDR polarisability (Draine & Goodman) without avgpol: CM / (1 - CM/V (M0 + 2i kd^3/3)),
    M0 = (b1 + (b2 + b3 S) m^2) kd^2, S = sum_i prop_i^2 pol_i^2"""
    m = complex(m)
    vol = gridspace ** 3
    S = float(np.sum(np.asarray(prop, float) ** 2 * np.asarray(pol, float) ** 2))
    cm = 3 / (4 * math.pi) * vol * (m * m - 1) / (m * m + 2)
    M = (LDR_B1 + (LDR_B2 + LDR_B3 * S) * m * m) * kd * kd + 2j * kd ** 3 / 3
    return cm / (1 - cm / vol * M)


class SphereWorkload:
    """'-grid g -m m -dpl dpl' (sphere, LDR, default orientation, lambda = 2 pi): the inputs of both polarisations
    (Y first, then X, as the reference solves them)"""

    def __init__(self, grid, m, dpl, fftfit):
        self.box = fit_box("sphere", grid)
        self.pos = lattice("sphere", self.box)
        self.n = len(self.pos)
        self.mat = np.zeros(self.n, np.uint8)
        self.grid = (fftfit(2 * self.box[0], 1), fftfit(2 * self.box[1], 1), fftfit(2 * self.box[2], 2))
        self.m = complex(m)
        self.wavenum = 1.0
        self.gridspace = 2 * math.pi / dpl
        self.kd = 2 * math.pi / dpl
        self.prop = np.array([0.0, 0.0, 1.0])
        self.incpol = [np.array([0.0, 1.0, 0.0]), np.array([1.0, 0.0, 0.0])]
        self.cc = [np.full(3, ldr_cc(self.m, self.kd, self.gridspace, self.prop, e)) for e in self.incpol]
        self.einc = [plane_wave(self.box, self.pos, self.gridspace, self.wavenum, self.prop, e) for e in self.incpol]

"""The differentiation workload: an inhomogeneous cube of 48^3 dipoles (-shape box -grid 48, grid 96^3) in which
every dipole has its own refractive index from two seeded, Gaussian-smoothed random fields.

    u = Phi(standardised(gaussian_filter(N(0,1) on the 48^3 lattice, sigma = 4 dipoles, periodic)))
    m_re = 1.3 + 0.4 u1 (seed 20261204), m_im = 0.05 u2 (seed 20261205), chi = (m^2 - 1)/(4 pi)
    finite-difference dipoles: 256 drawn with seed 20261206, step 1e-6 on chi

dpl follows the reference's default, 10 max|m| (make_particle.c:1347-1353). The reference holds at most 15
materials (const.h:106), so it cannot run the continuous field; quantised() maps the field onto 14 materials (7
levels of m_re x 2 of m_im, each at its bin centre), which the reference runs through -shape read (golden fixture
reference_c4_quantised.json, made by golden/make_c4_quantised.py). Arrays are in the lattice order of the box:
z outermost, x fastest.
"""
import numpy as np

BOX = 48
SIGMA = 4.0
SEEDS = (20261204, 20261205)
FD_SEED, FD_COUNT, FD_STEP = 20261206, 256, 1e-6
LEVELS_RE, LEVELS_IM = 7, 2


def smooth_field(box, seed, sigma=SIGMA):
    """seeded Gaussian-smoothed white noise on the box (periodic), standardised, mapped to (0,1) by the normal CDF;
    shape (bz, by, bx)"""
    from scipy.ndimage import gaussian_filter
    from scipy.stats import norm
    g = np.random.default_rng(seed).standard_normal(tuple(box)[::-1])
    g = gaussian_filter(g, sigma, mode="wrap")
    g = (g - g.mean()) / g.std()
    return norm.cdf(g)


def fields(box=(BOX, BOX, BOX)):
    """(u1, u2) flattened in lattice order"""
    return smooth_field(box, SEEDS[0]).ravel(), smooth_field(box, SEEDS[1]).ravel()


def refractive_index(u1, u2):
    return 1.3 + 0.4 * u1 + 0.05j * u2


def chi_of(m):
    return (m * m - 1) / (4 * np.pi)


def default_dpl(m):
    """the reference's default dipoles per wavelength: 10 max|m|"""
    return 10 * float(np.max(np.abs(m)))


def quantised(u1, u2):
    """material index (0-based) per dipole and the 14 refractive indices (bin centres)"""
    q1 = np.minimum((u1 * LEVELS_RE).astype(int), LEVELS_RE - 1)
    q2 = np.minimum((u2 * LEVELS_IM).astype(int), LEVELS_IM - 1)
    mat = q1 + LEVELS_RE * q2
    lv1 = (np.arange(LEVELS_RE) + 0.5) / LEVELS_RE
    lv2 = (np.arange(LEVELS_IM) + 0.5) / LEVELS_IM
    levels = np.array([refractive_index(lv1[k % LEVELS_RE], lv2[k // LEVELS_RE])
                       for k in range(LEVELS_RE * LEVELS_IM)])
    return mat.astype(np.uint8), levels


def fd_dipoles(n):
    return np.sort(np.random.default_rng(FD_SEED).choice(n, FD_COUNT, replace=False))

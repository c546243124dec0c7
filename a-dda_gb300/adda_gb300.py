"""Python front end of libadda_gb300.so (ctypes over the C ABI in include/adda_gb300.h).

The host side mirrors the reference's command-line driven setup for the hot path: a particle from -grid/-shape,
-m, -dpl, -pol, -orient (param.c defaults: lambda = 2*pi, so k = 1; dpl = 10*|m|), the incident plane waves of
both polarisations, and then the device context that owns the interaction matrix, the matvec and the solver.
No CPU fallback exists: every compute call goes through the CUDA library and fails loudly without it.
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libadda_gb300.so")

SHAPES = {"sphere": 0, "ellipsoid": 1, "box": 2}
POLS = {"ldr": 0, "cm": 1, "rrc": 2, "dgf": 3, "cldr": 4, "fcd": 5, "igt_so": 6, "lak": 7, "so": 8, "nloc": 9,
        "nloc_av": 10}
ITERS = {"qmr": 0, "bicgstab": 1, "bicg": 2, "cgnr": 3, "csym": 4, "qmr2": 5, "bcgs2": 6}
PREC = {"fp64": 0, "fp32": 1, "mixed": 2, "mixed_f32vec": 3, "mixed_f64vec": 4}
INIT = {"auto": 0, "zero": 1, "inc": 2, "x0": 3, "chpoint": 4}
STATUS = {0: "ok", 1: "breakdown", 2: "stagnation", 3: "maxiter", 4: "chpoint"}


class AddaError(RuntimeError):
    pass


class Problem(ctypes.Structure):
    _fields_ = [("boxX", ctypes.c_int), ("boxY", ctypes.c_int), ("boxZ", ctypes.c_int),
                ("gridX", ctypes.c_int), ("gridY", ctypes.c_int), ("gridZ", ctypes.c_int),
                ("ndip", ctypes.c_size_t), ("position", ctypes.c_void_p), ("material", ctypes.c_void_p),
                ("gridspace", ctypes.c_double), ("wavenum", ctypes.c_double), ("nrhs_max", ctypes.c_int),
                ("device", ctypes.c_int), ("interaction", ctypes.c_int), ("nloc_rp", ctypes.c_double),
                ("surface", ctypes.c_int), ("zsum_shift", ctypes.c_double), ("msub_re", ctypes.c_double),
                ("msub_im", ctypes.c_double), ("msub_inf", ctypes.c_int), ("refl", ctypes.c_int),
                ("refl_data", ctypes.c_void_p), ("int_tables", ctypes.c_void_p), ("so_m_re", ctypes.c_double),
                ("so_m_im", ctypes.c_double)]


INTERACTIONS = {"poi": 0, "fcd": 1, "fcd_st": 2, "nloc": 3, "nloc_av": 4, "igt_so": 5, "so": 6}
INT_TABLES = 11928  # doubles of the igt_so / so integral tables
# -int_surf: image dipole (GPU), image + Sommerfeld integrals from a table, or a tensor supplied by the caller
REFL = {"img": 0, "som": 1, "host": 2}


class SolveParams(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("precision", ctypes.c_int), ("eps", ctypes.c_double),
                ("maxiter", ctypes.c_int), ("init_field", ctypes.c_int), ("check_every", ctypes.c_int),
                ("inner_eps", ctypes.c_double), ("max_refine", ctypes.c_int), ("chp_time", ctypes.c_double),
                ("full_steps", ctypes.c_int), ("final_eps", ctypes.c_double)]


class IntegrParms(ctypes.Structure):
    """one angle's block of alldir_params.dat (degrees)"""
    _fields_ = [("min", ctypes.c_double), ("max", ctypes.c_double), ("Jmin", ctypes.c_int), ("Jmax", ctypes.c_int),
                ("eps", ctypes.c_double), ("equiv", ctypes.c_int), ("periodic", ctypes.c_int)]


# the reference's alldir_params.dat defaults: theta, phi
ALLDIR_DEFAULT = (dict(min=0.0, max=180.0, Jmin=2, Jmax=6, eps=0.0, equiv=False, periodic=False),
                  dict(min=0.0, max=360.0, Jmin=2, Jmax=5, eps=0.0, equiv=True, periodic=True))


def _parms(parms):
    arr = (IntegrParms * 2)()
    for i, p in enumerate(parms):
        arr[i] = IntegrParms(p["min"], p["max"], p["Jmin"], p["Jmax"], p["eps"], int(p["equiv"]), int(p["periodic"]))
    return arr


def integr_points(p, in_cos):
    """grid angles (degrees) of one alldir block: equal steps in cos for theta, in the angle for phi"""
    arr = _parms([p, p])
    n = lib().adda_gb300_integr_points(ctypes.byref(arr[0]), int(in_cos), None)
    if n < 1:
        raise AddaError("integr_points: inconsistent integration parameters")
    out = np.zeros(n)
    lib().adda_gb300_integr_points(ctypes.byref(arr[0]), int(in_cos), _p(out))
    return out


def romberg2d(parms, values, poles=False):
    """the reference's Romberg2D average of values [ntheta][nphi][dim] on the alldir (or orientation) grid; poles:
    full-range orientation averaging, where beta = 0 and 180 are single orientations"""
    v = np.ascontiguousarray(values, dtype=np.float64)
    res = np.zeros(v.shape[2])
    lib().adda_gb300_romberg2d_ex(_parms(parms), v.shape[2], _p(v), _p(res), int(poles))
    return res


class RhsStats(ctypes.Structure):
    _fields_ = [("niter", ctypes.c_int), ("status", ctypes.c_int), ("resid", ctypes.c_double),
                ("refinements", ctypes.c_int), ("matvecs_fp64", ctypes.c_int), ("matvecs_fp32", ctypes.c_int)]


EXPORTS = ["adda_gb300_fft_fit", "adda_gb300_fit_box", "adda_gb300_make_particle", "adda_gb300_rotation",
           "adda_gb300_plane_wave", "adda_gb300_plane_wave_surf", "adda_gb300_wkb_field", "adda_gb300_polarizability",
           "adda_gb300_polarizability_dchi", "adda_gb300_polarizability_nloc",
           "adda_gb300_create", "adda_gb300_create_group", "adda_gb300_destroy",
           "adda_gb300_get_grid", "adda_gb300_init_dmatrix", "adda_gb300_dmatrix_len", "adda_gb300_get_dmatrix",
           "adda_gb300_set_cc", "adda_gb300_set_cc_sqrt", "adda_gb300_set_cc_dipole", "adda_gb300_matvec", "adda_gb300_matvec_device",
           "adda_gb300_solve", "adda_gb300_solve_device", "adda_gb300_solve_many", "adda_gb300_vjp_chi",
           "adda_gb300_chpoint_size", "adda_gb300_chpoint_save", "adda_gb300_chpoint_load",
           "adda_gb300_rmatrix_len", "adda_gb300_get_rmatrix", "adda_gb300_cross_sections_beam",
           "adda_gb300_cross_sections", "adda_gb300_scattered_fields", "adda_gb300_integr_points",
           "adda_gb300_romberg2d", "adda_gb300_romberg2d_ex", "adda_gb300_scattering_integrals",
           "adda_gb300_cross_sections_noalloc", "adda_gb300_time_matvec", "adda_gb300_read_int_tables",
           "adda_gb300_get_fft_shape", "adda_gb300_set_fft_shape", "adda_gb300_get_l2_chunk", "adda_gb300_set_stream",
           "adda_gb300_last_solve_ms", "adda_gb300_last_error", "adda_gb300_kernel_launches"]

_lib = None


def build(force=False, out=None, defines=()):
    """compile the library (out/defines: a variant build in another directory with extra -D macros)"""
    import importlib.util
    spec = importlib.util.spec_from_file_location("adda_gb300_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force, out=out, defines=defines)


def lib():
    """Load the CUDA library (building it first if it is missing or older than its sources)."""
    global _lib
    if _lib is None:
        build()
        _lib = load_library(LIB_PATH)
    return _lib


def load_library(path):
    """a libadda_gb300.so with the C ABI's argument and result types bound"""
    L = ctypes.CDLL(path)
    P, I, D, SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
    sig = {
        "adda_gb300_fft_fit": ([I, I], I),
        "adda_gb300_fit_box": ([I, P, I, P, P], I),
        "adda_gb300_make_particle": ([I, P, I, I, I, P, P], SZ),
        "adda_gb300_rotation": ([P, D, D, D, P, P, P], None),
        "adda_gb300_plane_wave": ([SZ, P, I, I, I, D, D, P, P, P], None),
        "adda_gb300_plane_wave_surf": ([SZ, P, I, I, I, D, D, P, P, P, I, D, D, D, I, P, P], I),
        "adda_gb300_rmatrix_len": ([P], SZ),
        "adda_gb300_get_rmatrix": ([P, P], I),
        "adda_gb300_cross_sections_beam": ([P, I, P, D, P, P], I),
        "adda_gb300_wkb_field": ([I, I, I, SZ, P, P, I, P, D, P, P], I),
        "adda_gb300_polarizability": ([I, D, D, D, D, P, P, I, P], I),
        "adda_gb300_polarizability_dchi": ([I, D, D, D, D, P, P, I, P], I),
        "adda_gb300_polarizability_nloc": ([I, D, D, D, D, P], I),
        "adda_gb300_vjp_chi": ([P, P, I, P, P, P, P, P], I),
        "adda_gb300_create": ([P, P], I),
        "adda_gb300_create_group": ([P, I, P, P, P, P], I),
        "adda_gb300_destroy": ([P], I),
        "adda_gb300_get_grid": ([P, P], I),
        "adda_gb300_init_dmatrix": ([P], I),
        "adda_gb300_dmatrix_len": ([P], SZ),
        "adda_gb300_get_dmatrix": ([P, P], I),
        "adda_gb300_set_cc": ([P, I, I, P], I),
        "adda_gb300_set_cc_sqrt": ([P, I, I, P], I),
        "adda_gb300_set_cc_dipole": ([P, I, P], I),
        "adda_gb300_matvec": ([P, I, I, P, P, P, I], I),
        "adda_gb300_matvec_device": ([P, I, I, P, P, P, I], I),
        "adda_gb300_solve": ([P, P, I, P, P, P, P, P, I], I),
        "adda_gb300_solve_device": ([P, P, I, P, P, P, P], I),
        "adda_gb300_solve_many": ([I, P, P, P, P, P, P, P], I),
        "adda_gb300_chpoint_size": ([P, I], SZ),
        "adda_gb300_integr_points": ([P, I, P], I),
        "adda_gb300_romberg2d": ([P, I, P, P], D),
        "adda_gb300_romberg2d_ex": ([P, I, P, P, I], D),
        "adda_gb300_scattering_integrals": ([P, I, P, P, P, P, P, P], I),
        "adda_gb300_chpoint_save": ([P, I, P, SZ], I),
        "adda_gb300_chpoint_load": ([P, I, P, SZ], I),
        "adda_gb300_time_matvec": ([P, I, I, I, SZ, P], I),
        "adda_gb300_cross_sections": ([P, I, P, P, P, P], I),
        "adda_gb300_scattered_fields": ([P, I, I, P, P], I),
        "adda_gb300_cross_sections_noalloc": ([I, SZ, P, P, P, P, I, I, I, I, I, D, D, P, P, P, P, P], I),
        "adda_gb300_read_int_tables": ([ctypes.c_char_p, P], I),
        "adda_gb300_get_fft_shape": ([P, I, P], I),
        "adda_gb300_set_fft_shape": ([P, I, P], I),
        "adda_gb300_get_l2_chunk": ([P, I], I),
        "adda_gb300_set_stream": ([P, P], I),
        "adda_gb300_last_error": ([], ctypes.c_char_p),
        "adda_gb300_last_solve_ms": ([P], D),
        "adda_gb300_kernel_launches": ([], ctypes.c_uint64),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(rc, what):
    if rc != 0:
        raise AddaError("%s failed (%d): %s" % (what, rc, lib().adda_gb300_last_error().decode()))


def kernel_launches():
    return int(lib().adda_gb300_kernel_launches())


# ---------------------------------------------------------------------------------------------------------------------
# host-side inputs (no GPU)

def read_int_tables(directory):
    """the integral tables of -int igt_so / so (the reference's input/tables/t1f.dat .. t10f.dat) as one array"""
    out = np.zeros(INT_TABLES)
    if lib().adda_gb300_read_int_tables(os.fsencode(directory), _p(out)):
        raise AddaError("read_int_tables: missing or short table files in " + str(directory))
    return out


def fft_fit(x, divis=1):
    return lib().adda_gb300_fft_fit(int(x), int(divis))


def make_particle(shape="sphere", grid=16, pars=None):
    """Particle lattice as MakeParticle builds it: returns (box, position [N,3] uint16, material [N] uint8)."""
    L = lib()
    sh = SHAPES[shape]
    pp = None if pars is None else np.ascontiguousarray(pars, dtype=np.float64)
    by, bz = ctypes.c_int(), ctypes.c_int()
    _check(L.adda_gb300_fit_box(sh, _p(pp), int(grid), ctypes.byref(by), ctypes.byref(bz)), "fit_box")
    box = (int(grid), by.value, bz.value)
    n = L.adda_gb300_make_particle(sh, _p(pp), *box, None, None)
    pos = np.zeros((n, 3), np.uint16)
    mat = np.zeros(n, np.uint8)
    L.adda_gb300_make_particle(sh, _p(pp), *box, _p(pos), _p(mat))
    return box, pos, mat


def rotation(alpha=0.0, beta=0.0, gamma=0.0, prop0=None):
    prop, py, px = np.zeros(3), np.zeros(3), np.zeros(3)
    p0 = None if prop0 is None else np.ascontiguousarray(prop0, dtype=np.float64)
    lib().adda_gb300_rotation(_p(p0), alpha, beta, gamma, _p(prop), _p(py), _p(px))
    return prop, py, px


def plane_wave(box, pos, gridspace, wavenum, prop, pol):
    e = np.zeros(len(pos) * 3, np.complex128)
    pos = np.ascontiguousarray(pos, dtype=np.uint16)
    lib().adda_gb300_plane_wave(len(pos), _p(pos), *box, gridspace, wavenum, _p(np.ascontiguousarray(prop, float)),
                                _p(np.ascontiguousarray(pol, float)), _p(e))
    return e


def plane_wave_surf(box, pos, gridspace, wavenum, prop, incpol_y, incpol_x, which, hsub, msub):
    """the incident field of a particle whose centre is hsub above a substrate of index msub (None: perfectly
    reflecting), which = 0 (Y, s-polarised) or 1 (X, p-polarised); returns (einc, inc_scale)"""
    e = np.zeros(len(pos) * 3, np.complex128)
    pos = np.ascontiguousarray(pos, dtype=np.uint16)
    sc = np.zeros(1)
    f = [_p(np.ascontiguousarray(v, float)) for v in (prop, incpol_y, incpol_x)]
    m = complex(0 if msub is None else msub)
    _check(lib().adda_gb300_plane_wave_surf(len(pos), _p(pos), *box, gridspace, wavenum, *f, which, hsub, m.real,
                                            m.imag, 1 if msub is None else 0, _p(e), _p(sc)), "plane_wave_surf")
    return e, float(sc[0])


def polarizability(m, kd, gridspace, prop, incpol, relation="ldr", avgpol=False, rp=0.0):
    """CoupleConstant: the three diagonal components; rp is the Gaussian width of -pol nloc|nloc_av <Rp>"""
    cc = np.zeros(3, np.complex128)
    if relation in ("nloc", "nloc_av"):
        _check(lib().adda_gb300_polarizability_nloc(POLS[relation], complex(m).real, complex(m).imag, gridspace, rp,
                                                    _p(cc)), "polarizability_nloc")
        return cc
    _check(lib().adda_gb300_polarizability(POLS[relation], complex(m).real, complex(m).imag, kd, gridspace,
                                           _p(np.ascontiguousarray(prop, float)),
                                           _p(np.ascontiguousarray(incpol, float)), int(avgpol), _p(cc)),
           "polarizability")
    return cc


VOLUME_RATIO = {"sphere": lambda p: math.pi / 6, "ellipsoid": lambda p: math.pi / 6 * p[0] * p[1],
                "box": lambda p: p[0] * p[1]}


def wkb_field(box, pos, mat, ref_index, kd, einc):
    """internal field in the WKB approximation for incidence along +z (CalcFieldWKB, iterative.c:1227-1322):
    ref_index per material; einc [3N] complex -> field [3N] complex"""
    pos = np.ascontiguousarray(pos, dtype=np.uint16).reshape(-1, 3)
    m = None if mat is None else np.ascontiguousarray(mat, dtype=np.uint8)
    ri = np.ascontiguousarray(np.atleast_1d(np.asarray(ref_index, dtype=np.complex128)))
    e = np.ascontiguousarray(einc, dtype=np.complex128)
    out = np.zeros_like(e)
    _check(lib().adda_gb300_wkb_field(int(box[0]), int(box[1]), int(box[2]), len(pos), _p(pos), _p(m), len(ri),
                                      _p(ri), kd, _p(e), _p(out)), "wkb_field")
    return out


def field_to_x0(field, cc, ref_index, gridspace, mat=None):
    """starting vector x_0 = E/(cc_sqrt*chi_inv) of a field E [3N] (InitFieldfromE, iterative.c:1325-1338):
    chi_inv = 4pi/(d^3 (m^2-1)) per material, cc [nmat,3] the polarizabilities"""
    ri = np.atleast_1d(np.asarray(ref_index, dtype=np.complex128))
    cc = np.asarray(cc, dtype=np.complex128).reshape(len(ri), 3)
    chi_inv = 4 * np.pi / (gridspace ** 3 * (ri * ri - 1))
    mult = 1 / (np.sqrt(cc) * chi_inv[:, None])                       # [nmat,3]
    idx = np.zeros(len(field) // 3, np.int64) if mat is None else np.asarray(mat, dtype=np.int64)
    return (np.asarray(field).reshape(-1, 3) * mult[idx]).reshape(-1)


def polarizability_dchi(m, kd, gridspace, prop, incpol, relation="ldr", avgpol=False):
    """d(1/alpha)/dchi, chi = (m^2-1)/(4 pi)"""
    out = np.zeros(1, np.complex128)
    _check(lib().adda_gb300_polarizability_dchi(POLS[relation], complex(m).real, complex(m).imag, kd, gridspace,
                                                _p(np.ascontiguousarray(prop, float)),
                                                _p(np.ascontiguousarray(incpol, float)), int(avgpol), _p(out)),
           "polarizability_dchi")
    return out[0]


class Setup:
    """The inputs the reference host would build for
    '-grid g -shape s [pars] -m re im [-dpl d | -size s] -pol p [avgpol] -orient a b c -prop px py pz'
    (lambda = 2*pi, so k = 1): lattice, grid, both polarisations' cc, Einc, propagation and polarisation vectors.
    dpl defaults to 10*|m|; with -size it follows from the volume correction (make_particle.c:2178-2191).
    Order of the RHS: Y polarisation first, then X (calculator.c:309-330)."""

    def __init__(self, grid=16, shape="sphere", pars=None, m=1.5, dpl=None, size=None, pol="ldr", orient=(0, 0, 0),
                 avgpol=False, prop=None, lam=2 * math.pi, interaction="poi", nloc_rp=0.0, pol_rp=0.0, surface=None,
                 int_tables=None):
        self.interaction = interaction
        self.int_tables = int_tables  # -int igt_so | so: the integral tables (read_int_tables)
        self.nloc_rp = float(nloc_rp)
        self.pol, self.avgpol, self.pol_rp, self.prop0 = pol, avgpol, pol_rp, prop
        self.box, self.pos, self.mat = make_particle(shape, grid, pars)
        self.n = len(self.pos)
        self.grid = (fft_fit(2 * self.box[0]), fft_fit(2 * self.box[1]), fft_fit(2 * self.box[2], 2))
        self.m = complex(m)
        if size is not None:
            vr = VOLUME_RATIO[shape](pars if pars is not None else (1.0, 1.0))
            self.dpl = lam * (self.n / vr) ** (1.0 / 3) / size
        else:
            self.dpl = float(dpl) if dpl else 10 * abs(self.m)
        self.wavenum = 2 * math.pi / lam
        self.gridspace = lam / self.dpl
        self.kd = 2 * math.pi / self.dpl
        self.prop, py, px = rotation(*orient, prop0=prop)
        self.incpol = [py, px]
        self.cc = [polarizability(self.m, self.kd, self.gridspace, self.prop, e, pol, avgpol, pol_rp)
                   for e in self.incpol]
        self.einc = [plane_wave(self.box, self.pos, self.gridspace, self.wavenum, self.prop, e) for e in self.incpol]
        # -surf h msub | -surf h inf with -int_surf img|som (table: the Sommerfeld integrals, see Context)
        self.surface = None
        self.inc_scale = 1.0
        if surface is not None:
            h, msub = float(surface["h"]), surface.get("msub")
            rel = surface.get("relation", "img" if msub is None else "som")
            zsum = 2 * (h / self.gridspace - (self.box[2] - 1) / 2.0)
            self.surface = dict(zsum_shift=zsum, msub=None if msub is None else complex(msub), relation=rel,
                                data=surface.get("table"))
            beams = [plane_wave_surf(self.box, self.pos, self.gridspace, self.wavenum, self.prop, py, px, w, h, msub)
                     for w in (0, 1)]
            self.einc = [b[0] for b in beams]
            self.inc_scale = beams[0][1]


# ---------------------------------------------------------------------------------------------------------------------
# device context

# the reference's avg_params.dat defaults for the Euler angles beta (equal steps in cos) and gamma
AVG_DEFAULT = (dict(min=0.0, max=180.0, Jmin=2, Jmax=4, eps=1e-3, equiv=False, periodic=False),
               dict(min=0.0, max=360.0, Jmin=2, Jmax=4, eps=1e-3, equiv=True, periodic=True))


def orient_avg_cross_sections(ctx, s, parms=AVG_DEFAULT, full_alpha=True, method="qmr", prec="mixed", eps=1e-5,
                              maxiter=100000):
    """-orient avg for the cross sections (calculate_one_orientation and its Romberg integration over the Euler
    angles, src/calculator.c:293-358,690-710; CalculateE.c:737-751): for every (beta, gamma) of the avg_params grid
    (alpha = 0) the two incident polarisations are solved, the unpolarised Cext and Cabs are the means of the two, and
    the two-level Romberg scheme averages them over the orientations (full_alpha: the first Euler angle covers
    0..360, so beta = 0 and 180 are single orientations). The reference evaluates the orientations one after another
    as the adaptive integration asks for them; here all of them are solved up front as right-hand sides of batched
    solves (ctx.nrhs_max at a time), with each orientation's own polarisability (LDR averaged over the incident
    polarisation, as the reference forces for -orient avg, param.c:2136-2139: it still depends on the direction).
    s: the Setup the context was made from. Returns (Cext, Cabs) and the per-orientation values [nbeta][ngamma][2]."""
    betas, gammas = integr_points(parms[0], True), integr_points(parms[1], False)
    jobs = []  # (ib, ig, prop, incpol)
    for ib, b in enumerate(betas):
        for ig, g in enumerate(gammas):
            prop, py, px = rotation(0.0, b, g, prop0=s.prop0)
            jobs += [(ib, ig, prop, py), (ib, ig, prop, px)]
    R = ctx.nrhs_max
    vals = np.zeros((len(betas), len(gammas), 2))
    for k0 in range(0, len(jobs), R):
        batch = jobs[k0:k0 + R]
        for r, (_, _, prop, inc) in enumerate(batch):
            ctx.set_cc(r, polarizability(s.m, s.kd, s.gridspace, prop, inc, s.pol, True, s.pol_rp).reshape(1, 3))
        einc = np.stack([plane_wave(s.box, s.pos, s.gridspace, s.wavenum, prop, inc) for _, _, prop, inc in batch])
        ctx.solve(einc, method=method, prec=prec, eps=eps, maxiter=maxiter)
        ce, ca = ctx.cross_sections(np.stack([b[2] for b in batch]), np.stack([b[3] for b in batch]))
        for r, (ib, ig, _, _) in enumerate(batch):
            vals[ib, ig, 0] += 0.5 * ce[r]
            vals[ib, ig, 1] += 0.5 * ca[r]
    res = romberg2d(parms, vals, poles=full_alpha)
    return res[0], res[1], vals


def solve_many(ctxs, eincs, method="qmr", prec="mixed", eps=1e-5, maxiter=100000, init="auto", check_every=0):
    """solve several contexts (particles) concurrently; eincs[i]: [nrhs_i, 3N_i] complex. Returns per context
    (x, p, stats)."""
    L = lib()
    n = len(ctxs)
    es = [np.ascontiguousarray(e, dtype=np.complex128).reshape(-1, 3 * c.n) for c, e in zip(ctxs, eincs)]
    xs = [np.empty_like(e) for e in es]
    ps = [np.empty_like(e) for e in es]
    sts = [(RhsStats * e.shape[0])() for e in es]
    P = ctypes.c_void_p
    arr = lambda vals: (P * n)(*vals)
    nr = (ctypes.c_int * n)(*[e.shape[0] for e in es])
    sp = SolveParams(ITERS[method], PREC[prec], eps, maxiter, INIT[init], check_every, 0.0, 0, 0.0, 0)
    _check(L.adda_gb300_solve_many(n, arr([c.h.value for c in ctxs]), ctypes.byref(sp), nr,
                                   arr([e.ctypes.data for e in es]), arr([x.ctypes.data for x in xs]),
                                   arr([p.ctypes.data for p in ps]), arr([ctypes.addressof(s) for s in sts])),
           "solve_many")
    out = []
    for x, p, st in zip(xs, ps, sts):
        out.append((x, p, [dict(niter=s.niter, status=STATUS.get(s.status, s.status), resid=s.resid) for s in st]))
    return out


class Context:
    """One particle lattice on one GPU: the interaction matrix, FP64/FP32 matvecs, solver and cross sections."""

    def __init__(self, box, pos, mat, gridspace, wavenum, grid=(0, 0, 0), nrhs_max=2, device=0, interaction="poi",
                 nloc_rp=0.0, library=None, surface=None, int_tables=None, so_m=0.0):
        self.L = library or lib()
        self.pos = np.ascontiguousarray(pos, dtype=np.uint16).reshape(-1, 3)
        self.mat = None if mat is None else np.ascontiguousarray(mat, dtype=np.uint8)
        self.n = len(self.pos)
        self.nrhs_max = nrhs_max
        pr = Problem(box[0], box[1], box[2], grid[0], grid[1], grid[2], self.n, _p(self.pos).value,
                     None if self.mat is None else _p(self.mat).value, gridspace, wavenum, nrhs_max, device,
                     INTERACTIONS[interaction], nloc_rp)
        # igt_so / so: the integral tables and (so) the refractive index of the second-order terms
        self._tables = None
        if int_tables is not None:
            self._tables = np.ascontiguousarray(int_tables, dtype=np.float64)
            pr.int_tables = _p(self._tables).value
            pr.so_m_re, pr.so_m_im = complex(so_m).real, complex(so_m).imag
        # surface: dict(zsum_shift, msub (None = perfect reflector), relation img|som|host, data (complex array))
        self._refl = None
        if surface is not None:
            m = surface.get("msub")
            pr.surface, pr.zsum_shift, pr.refl = 1, surface["zsum_shift"], REFL[surface.get("relation", "img")]
            pr.msub_re, pr.msub_im, pr.msub_inf = (0.0, 0.0, 1) if m is None else (complex(m).real, complex(m).imag, 0)
            if surface.get("data") is not None:
                self._refl = np.ascontiguousarray(surface["data"], dtype=np.complex128)
                pr.refl_data = _p(self._refl).value
        self.h = ctypes.c_void_p()
        _check(self.L.adda_gb300_create(ctypes.byref(pr), ctypes.byref(self.h)), "create")
        g = (ctypes.c_int * 3)()
        self.L.adda_gb300_get_grid(self.h, g)
        self.grid = tuple(g)

    @classmethod
    def group(cls, setups, rhs_per_particle=2, device=0, library=None, box=None):
        """several particles (Setup objects of the same lattice spacing, wavelength and interaction term) solved as
        one batch: one context in the smallest box that holds every particle, rhs_per_particle RHS each (RHS
        r belongs to particle r // rhs_per_particle). Vectors are [R][3 * n] with n the largest particle's dipole count
        (group_pad pads a particle's field); set_cc per RHS, D built, the first rhs_per_particle of each particle's
        cc set. The phase reference of incident and scattered fields is the centre of the common box (self.box):
        incident fields come from group_plane_wave. box: a larger common box (e.g. one whose FFT grid is a power of
        two, for the compile-time transforms)."""
        s0 = setups[0]
        for s in setups:
            if s.gridspace != s0.gridspace or s.wavenum != s0.wavenum or s.interaction != s0.interaction:
                raise ValueError("group: particles need the same lattice spacing, wavelength and interaction term")
        fit = tuple(max(s.box[d] for s in setups) for d in range(3))
        box = fit if box is None else tuple(int(b) for b in box)
        if any(b < f for b, f in zip(box, fit)):
            raise ValueError("group: the common box must hold every particle")
        c = cls.__new__(cls)
        c.L = library or lib()
        c._lat = [(np.ascontiguousarray(s.pos, dtype=np.uint16).reshape(-1, 3),
                   None if s.mat is None else np.ascontiguousarray(s.mat, dtype=np.uint8)) for s in setups]
        c.counts = [len(p) for p, _ in c._lat]
        c.n = max(c.counts)
        c.pos, c.mat = None, None
        c.nparticles, c.rpp = len(setups), rhs_per_particle
        c.box, c.gridspace, c.wavenum = box, s0.gridspace, s0.wavenum
        c.nrhs_max = len(setups) * rhs_per_particle
        c._tables, c._refl = None, None
        pr = Problem(box[0], box[1], box[2], 0, 0, 0, 0, None, None, s0.gridspace, s0.wavenum, c.nrhs_max, device,
                     INTERACTIONS[s0.interaction], getattr(s0, "nloc_rp", 0.0))
        P_ = len(setups)
        nd = (ctypes.c_size_t * P_)(*c.counts)
        pp = (ctypes.c_void_p * P_)(*[_p(p).value for p, _ in c._lat])
        mm = (ctypes.c_void_p * P_)(*[None if m is None else _p(m).value for _, m in c._lat])
        c.h = ctypes.c_void_p()
        _check(c.L.adda_gb300_create_group(ctypes.byref(pr), P_, nd, pp, mm, ctypes.byref(c.h)), "create_group")
        g = (ctypes.c_int * 3)()
        c.L.adda_gb300_get_grid(c.h, g)
        c.grid = tuple(g)
        c.init_dmatrix()
        for q, s in enumerate(setups):
            for k in range(min(rhs_per_particle, len(s.cc))):
                c.set_cc(q * rhs_per_particle + k, s.cc[k].reshape(1, 3))
        return c

    def group_plane_wave(self, q, prop, pol):
        """the incident plane wave at particle q's dipoles, phase reference the common box's centre, padded"""
        pos = self._lat[q][0]
        return self.group_pad(plane_wave(self.box, pos, self.gridspace, self.wavenum, prop, pol), q)

    def group_pad(self, field, q):
        """particle q's [..., 3 * n_q] complex field padded with zeros to the group's vector length"""
        f = np.asarray(field, dtype=np.complex128)
        out = np.zeros(f.shape[:-1] + (3 * self.n,), np.complex128)
        out[..., :f.shape[-1]] = f
        return out

    @classmethod
    def from_setup(cls, s, nrhs_max=2, device=0, library=None):
        c = cls(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max, device, s.interaction,
                getattr(s, "nloc_rp", 0.0), library, getattr(s, "surface", None), getattr(s, "int_tables", None),
                getattr(s, "m", 0.0))
        c.init_dmatrix()
        for r in range(min(nrhs_max, len(s.cc))):
            c.set_cc(r, s.cc[r].reshape(1, 3))
        return c

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.adda_gb300_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_dmatrix(self):
        _check(self.L.adda_gb300_init_dmatrix(self.h), "init_dmatrix")

    def dmatrix(self):
        n = self.L.adda_gb300_dmatrix_len(self.h)
        out = np.empty(n, np.complex128)
        _check(self.L.adda_gb300_get_dmatrix(self.h, _p(out)), "get_dmatrix")
        return out

    def rmatrix(self):
        """surface mode: the FP64 reflected interaction matrix [x][z][y<gY/2+1][6]"""
        n = self.L.adda_gb300_rmatrix_len(self.h)
        out = np.empty(n, np.complex128)
        _check(self.L.adda_gb300_get_rmatrix(self.h, _p(out)), "get_rmatrix")
        return out

    def set_cc(self, rhs, cc):
        cc = np.ascontiguousarray(cc, dtype=np.complex128).reshape(-1, 3)
        _check(self.L.adda_gb300_set_cc(self.h, rhs, cc.shape[0], _p(cc)), "set_cc")

    def set_cc_dipole(self, rhs, cc):
        cc = np.ascontiguousarray(cc, dtype=np.complex128).reshape(self.n, 3)
        _check(self.L.adda_gb300_set_cc_dipole(self.h, rhs, _p(cc)), "set_cc_dipole")

    def matvec(self, x, prec="fp64", her=False):
        """x: [nrhs, 3N] (or [3N]) complex; returns (y, |y|^2 per RHS)."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        one = x.ndim == 1
        x2 = x.reshape(-1, 3 * self.n)
        y = np.empty_like(x2)
        ip = np.zeros(x2.shape[0])
        _check(self.L.adda_gb300_matvec(self.h, PREC[prec], x2.shape[0], _p(x2), _p(y), _p(ip), int(her)), "matvec")
        return (y[0], ip[0]) if one else (y, ip)

    def solve(self, einc, method="qmr", prec="fp64", eps=1e-5, maxiter=100000, init="auto", check_every=0,
              inner_eps=0.0, max_refine=0, hist_cap=0, x0=None, chp_time=0.0, full_steps=False, out=None,
              final_eps=0.0):
        """einc: [nrhs, 3N] complex. Returns dict with x, p [nrhs,3N], stats per RHS and residual histories
        (hist[r][k] = RE_k). init="x0" starts from x0 [nrhs, 3N] (see field_to_x0 for a field read from file or from
        wkb_field); init="chpoint" resumes every RHS from chpoint_load. chp_time > 0 stops after that many seconds
        (status "chpoint", state kept for chpoint_save); full_steps: BiCGStab without its half-step exit.
        out: optional (x, p) complex128 [nrhs, 3N] C-contiguous host arrays (e.g. views of pinned memory) that receive
        the solution and the polarisations directly. final_eps (mixed): the FP64 residual the refinement stops at (0:
        0.3*eps, 0.1*eps for BiCGStab/BCGS2, for cross sections within about 1e-6 of the converged ones)."""
        e = np.ascontiguousarray(einc, dtype=np.complex128).reshape(-1, 3 * self.n)
        R = e.shape[0]
        if out is not None:
            x, p = out
            for a in (x, p):
                if a.dtype != np.complex128 or a.shape != e.shape or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError("out arrays must be C-contiguous complex128 of shape %s" % (e.shape,))
            if init == "x0":
                x[:] = np.asarray(x0, dtype=np.complex128).reshape(R, 3 * self.n)
        elif init == "x0":
            x = np.ascontiguousarray(np.array(x0, dtype=np.complex128).reshape(R, 3 * self.n))
        else:
            x = np.empty_like(e)
        if out is None:
            p = np.empty_like(e)
        st = (RhsStats * R)()
        hist = np.zeros((R, hist_cap)) if hist_cap else None
        sp = SolveParams(ITERS[method], PREC[prec], eps, maxiter, INIT[init], check_every, inner_eps, max_refine,
                         chp_time, int(full_steps), final_eps)
        _check(self.L.adda_gb300_solve(self.h, ctypes.byref(sp), R, _p(e), _p(x), _p(p), st, _p(hist), hist_cap),
               "solve")
        stats = [dict(niter=s.niter, status=STATUS.get(s.status, s.status), resid=s.resid,
                      refinements=s.refinements, matvecs_fp64=s.matvecs_fp64, matvecs_fp32=s.matvecs_fp32)
                 for s in st]
        return dict(x=x, p=p, stats=stats, hist=hist)

    def solve_device(self, d_einc, nrhs, d_x=None, d_p=None, method="qmr", prec="mixed", eps=1e-5, maxiter=100000,
                     init="auto", check_every=0, inner_eps=0.0, max_refine=0, final_eps=0.0):
        """solve on device-resident buffers (raw CUDA pointers as ints, double2 [nrhs][3N]); the solve reads them after
        the work queued on the stream of set_stream (by default the legacy default stream, torch's default)"""
        st = (RhsStats * nrhs)()
        sp = SolveParams(ITERS[method], PREC[prec], eps, maxiter, INIT[init], check_every, inner_eps, max_refine,
                         0.0, 0, final_eps)
        _check(self.L.adda_gb300_solve_device(self.h, ctypes.byref(sp), nrhs, ctypes.c_void_p(d_einc),
                                              ctypes.c_void_p(d_x) if d_x else None,
                                              ctypes.c_void_p(d_p) if d_p else None, st), "solve_device")
        return [dict(niter=s.niter, status=STATUS.get(s.status, s.status), resid=s.resid, refinements=s.refinements,
                     matvecs_fp64=s.matvecs_fp64, matvecs_fp32=s.matvecs_fp32) for s in st]

    def scattering_integrals(self, nrhs, prop, incpolx, incpoly, parms=ALLDIR_DEFAULT):
        """Csca [nrhs] and Csca*g [nrhs,3] (beam frame) of the last solve's RHS 0..nrhs-1 sharing one incident frame,
        from the GPU scattered field on the alldir grid and the reference's Romberg integration"""
        csca = np.zeros(nrhs)
        cg = np.zeros((nrhs, 3))
        vec = [np.ascontiguousarray(v, dtype=np.float64) for v in (prop, incpolx, incpoly)]
        _check(self.L.adda_gb300_scattering_integrals(self.h, nrhs, _parms(parms), *[_p(v) for v in vec], _p(csca),
                                                      _p(cg)), "scattering_integrals")
        return csca, cg

    def chpoint_size(self, method="qmr"):
        """bytes of an iteration checkpoint of that method (the reference's chp.<ringid> format)"""
        return self.L.adda_gb300_chpoint_size(self.h, ITERS[method])

    def chpoint_save(self, rhs=0):
        """the FP64 solver state of right-hand side rhs after the last solve, as the reference's checkpoint bytes"""
        # the method of the last solve is not known here: try the sizes (each method has its own)
        n = max(self.chpoint_size(m) for m in ITERS)
        buf = ctypes.create_string_buffer(n)
        _check(self.L.adda_gb300_chpoint_save(self.h, rhs, buf, n), "chpoint_save")
        head = np.frombuffer(buf.raw[:4], np.int32)[0]
        meth = {5: "qmr", 2: "bicgstab", 1: "bicg", 3: "cgnr", 4: "csym", 6: "qmr2", 0: "bcgs2"}[int(head)]
        return buf.raw[:self.chpoint_size(meth)]

    def chpoint_load(self, rhs, data):
        """keep checkpoint bytes (the reference's chp.<ringid> file) for the next solve with init="chpoint" """
        data = bytes(data)
        _check(self.L.adda_gb300_chpoint_load(self.h, rhs, data, len(data)), "chpoint_load")

    def fft_shape(self, prec="fp32"):
        """the matvec's tile shape (w1, w2, pairs, threads) for fp32 or fp64"""
        v = (ctypes.c_int * 4)()
        _check(self.L.adda_gb300_get_fft_shape(self.h, PREC[prec], v), "get_fft_shape")
        return tuple(v)

    def l2_chunk(self, prec="fp32"):
        """x-slabs per chunk of the matvec's y/z stage"""
        return self.L.adda_gb300_get_l2_chunk(self.h, PREC[prec])

    def set_fft_shape(self, shape, prec="fp32"):
        """fix the matvec's tile shape (fp32: no tuning of it)"""
        _check(self.L.adda_gb300_set_fft_shape(self.h, PREC[prec], (ctypes.c_int * 4)(*shape)), "set_fft_shape")

    def set_stream(self, stream=None):
        """the caller's stream the device-buffer calls order themselves with: a torch.cuda.Stream, a raw
        cudaStream_t as int, or None for the legacy default stream"""
        ptr = getattr(stream, "cuda_stream", stream)
        _check(self.L.adda_gb300_set_stream(self.h, ctypes.c_void_p(ptr) if ptr else None), "set_stream")

    def last_solve_ms(self):
        """device milliseconds of the last solve (CUDA events on the context stream)"""
        return self.L.adda_gb300_last_solve_ms(self.h)

    def time_matvec(self, prec="fp32", nrhs=1, iters=10, flush_bytes=0):
        """average device milliseconds of one matvec (CUDA events on the context stream)"""
        ms = ctypes.c_double(0)
        _check(self.L.adda_gb300_time_matvec(self.h, PREC[prec], nrhs, iters, flush_bytes, ctypes.byref(ms)),
               "time_matvec")
        return ms.value

    def vjp_chi(self, rhs, prop, incpol, dinv_alpha, method="qmr", prec="fp64", eps=1e-10, maxiter=100000):
        """gradients of Cext and Cabs of RHS `rhs` of the last solve w.r.t. each dipole's chi: two [N,2] arrays
        (d/dRe chi, d/dIm chi)"""
        f = np.ascontiguousarray(dinv_alpha, dtype=np.complex128).reshape(self.n)
        ge = np.zeros((self.n, 2))
        ga = np.zeros((self.n, 2))
        sp = SolveParams(ITERS[method], PREC[prec], eps, maxiter, INIT["zero"], 0, 0.0, 0, 0.0, 0)
        _check(self.L.adda_gb300_vjp_chi(self.h, ctypes.byref(sp), rhs, _p(np.ascontiguousarray(prop, float)),
                                         _p(np.ascontiguousarray(incpol, float)), _p(f), _p(ge), _p(ga)), "vjp_chi")
        return ge, ga

    def cross_sections(self, prop, incpol):
        """prop/incpol: [nrhs,3]; returns (Cext[nrhs], Cabs[nrhs]) from the last solve's polarisations."""
        prop = np.ascontiguousarray(prop, dtype=np.float64).reshape(-1, 3)
        inc = np.ascontiguousarray(incpol, dtype=np.float64).reshape(-1, 3)
        R = prop.shape[0]
        ce, ca = np.zeros(R), np.zeros(R)
        _check(self.L.adda_gb300_cross_sections(self.h, R, _p(prop), _p(inc), _p(ce), _p(ca)), "cross_sections")
        return ce, ca

    def cross_sections_beam(self, einc, inc_scale=1.0):
        """Cext (general incident field, the surface-mode formula) and Cabs of the last solve; einc [nrhs, n*3]"""
        e = np.ascontiguousarray(einc, dtype=np.complex128).reshape(-1, 3 * self.n)
        R = e.shape[0]
        ce, ca = np.zeros(R), np.zeros(R)
        _check(self.L.adda_gb300_cross_sections_beam(self.h, R, _p(e), inc_scale, _p(ce), _p(ca)),
               "cross_sections_beam")
        return ce, ca

    def scattered_fields(self, dirs, nrhs=1):
        """scattering amplitudes E(n) of the last solve's first nrhs RHS for unit directions dirs [ndir,3]:
        complex [nrhs, ndir, 3] (CalcFieldFree, crosssec.c:506-596)"""
        d = np.ascontiguousarray(dirs, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((nrhs, d.shape[0], 3), np.complex128)
        _check(self.L.adda_gb300_scattered_fields(self.h, nrhs, d.shape[0], _p(d), _p(out)), "scattered_fields")
        return out

    def mueller_yz(self, prop, incpol_y, incpol_x, thetas_deg):
        """Mueller matrices [ntheta, 4, 4] in the plane of prop and incpol_y, for a last solve whose RHS 0 and 1 are
        the Y and X polarisations: CalcEplaneYZ (CalculateE.c:423-500: observer n = cos(t) prop + sin(t) incpol_y,
        E_per = E.incpol_x, E_par = E.(-sin(t) prop + cos(t) incpol_y)) and ComputeMuellerMatrix (CalculateE.c:83-118,
        Bohren & Huffman 3.16) with s1 = Eper(X), s2 = Epar(Y), s3 = Epar(X), s4 = Eper(Y) (CalculateE.c:244)"""
        prop, py, px = (np.asarray(v, dtype=np.float64) for v in (prop, incpol_y, incpol_x))
        t = np.radians(np.asarray(thetas_deg, dtype=np.float64))
        co, si = np.cos(t)[:, None], np.sin(t)[:, None]
        e = self.scattered_fields(co * prop + si * py, nrhs=2)
        epar = -si * prop + co * py
        per = e @ px                                    # [2, ntheta]
        par = np.einsum("rtc,tc->rt", e, epar)
        return mueller_matrix(per[1], par[0], par[1], per[0])


def mueller_matrix(s1, s2, s3, s4):
    """4x4 Mueller matrices from the amplitude-matrix elements (ComputeMuellerMatrix, CalculateE.c:83-118)"""
    a1, a2, a3, a4 = (np.abs(v) ** 2 for v in (s1, s2, s3, s4))
    m = np.empty(np.shape(s1) + (4, 4))
    m[..., 0, 0] = 0.5 * (a1 + a2 + a3 + a4)
    m[..., 0, 1] = 0.5 * (a2 - a1 + a4 - a3)
    m[..., 0, 2] = (s2 * np.conj(s3) + s1 * np.conj(s4)).real
    m[..., 0, 3] = (s2 * np.conj(s3) - s1 * np.conj(s4)).imag
    m[..., 1, 0] = 0.5 * (a2 - a1 + a3 - a4)
    m[..., 1, 1] = 0.5 * (a2 + a1 - a3 - a4)
    m[..., 1, 2] = (s2 * np.conj(s3) - s1 * np.conj(s4)).real
    m[..., 1, 3] = (s2 * np.conj(s3) + s1 * np.conj(s4)).imag
    m[..., 2, 0] = (s2 * np.conj(s4) + s1 * np.conj(s3)).real
    m[..., 2, 1] = (s2 * np.conj(s4) - s1 * np.conj(s3)).real
    m[..., 2, 2] = (s1 * np.conj(s2) + s3 * np.conj(s4)).real
    m[..., 2, 3] = (s2 * np.conj(s1) + s4 * np.conj(s3)).imag
    m[..., 3, 0] = (s4 * np.conj(s2) + s1 * np.conj(s3)).imag
    m[..., 3, 1] = (s4 * np.conj(s2) - s1 * np.conj(s3)).imag
    m[..., 3, 2] = (s1 * np.conj(s2) - s3 * np.conj(s4)).imag
    m[..., 3, 3] = (s1 * np.conj(s2) - s3 * np.conj(s4)).real
    return m

"""ctypes front end of the C oracle (liboracle.so) and of the reference build under oracle/_ref.

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the
checker or the timed CPU baseline. The GPU product never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "adda")

QMR_CS, BICGSTAB, BICG_CS, CGNR, CSYM, QMR_CS_2, BCGS2 = 0, 1, 2, 3, 4, 5, 6
IF_AUTO, IF_ZERO, IF_INC, IF_X0 = 0, 1, 2, 3
STATUS = {0: "ok", 1: "breakdown", 2: "stagnation", 3: "maxiter"}

_lib = None


def build(force=False):
    """Compile liboracle.so (and, when the reference sources are present, the reference build)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "lib"], check=True)
    return LIB_PATH


def ref_src_dir():
    """Where the reference's sources are read: $ADDA_REF_SRC, else a reference checkout beside this repository
    (<repository>/../reference/src)."""
    return os.environ.get("ADDA_REF_SRC") or os.path.normpath(os.path.join(HERE, "..", "..", "reference", "src"))


def build_reference(ref_src=None):
    """Compile the unmodified reference sequential build with the FFTW-subset shim into oracle/_ref/adda."""
    ref_src = ref_src or ref_src_dir()
    if not os.path.isdir(ref_src):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF_SRC=" + ref_src, "-j8"], check=True)
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        c_p, c_d, c_i, c_sz = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_size_t
        L.or_fftfit.argtypes = [c_i, c_i]
        L.or_fftfit.restype = c_i
        L.or_create.argtypes = [c_i] * 6 + [c_sz, c_p, c_p, c_d, c_d, c_i]
        L.or_create.restype = c_p
        L.or_free.argtypes = [c_p]
        L.or_init_dmatrix.argtypes = [c_p]
        L.or_dmatrix_len.argtypes = [c_p]
        L.or_dmatrix_len.restype = c_sz
        L.or_get_dmatrix.argtypes = [c_p, c_p]
        L.or_set_cc_mat.argtypes = [c_p, c_i, c_p]
        L.or_set_cc_dip.argtypes = [c_p, c_p]
        L.or_matvec.argtypes = [c_p, c_p, c_p, c_p, c_i]
        L.or_solve.argtypes = [c_p, c_i, c_p, c_d, c_i, c_i, c_p, c_p, c_p, c_i, c_p]
        L.or_solve.restype = c_i
        L.or_solve_chp.argtypes = [c_p, c_i, c_p, c_d, c_i, c_i, c_p, c_p, c_p, c_i, c_p, c_p, ctypes.c_size_t, c_p,
                                   c_p]
        L.or_solve_chp.restype = c_i
        L.or_set_interaction.argtypes = [c_p, ctypes.c_int]
        L.or_set_nloc_rp.argtypes = [c_p, ctypes.c_double]
        L.or_set_tables.argtypes = [c_p, c_p, ctypes.c_double, ctypes.c_double]
        L.or_cisi.argtypes = [ctypes.c_double, c_p, c_p]
        L.or_cross.argtypes = [c_p, c_p, c_p, c_p, c_p, c_p]
        L.or_field.argtypes = [c_p, c_p, c_p, c_p]
        L.or_set_surface.argtypes = [c_p, c_d, c_d, c_d, c_i, c_p]
        L.or_rmatrix_len.argtypes = [c_p]
        L.or_rmatrix_len.restype = c_sz
        L.or_get_rmatrix.argtypes = [c_p, c_p]
        L.or_cross_beam.argtypes = [c_p, c_p, c_p, c_d, c_p, c_p]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """One particle lattice on the CPU: D matrix, matvec, QMR_CS/BiCGStab and Cext/Cabs in double precision."""

    def __init__(self, box, grid, position, material, gridspace, wavenum, nthreads=0, interaction="poi", nloc_rp=0.0,
                 surface=None, int_tables=None, so_m=0.0):
        self.L = lib()
        self.position = np.ascontiguousarray(position, dtype=np.uint16).reshape(-1, 3)
        self.material = np.ascontiguousarray(material if material is not None
                                             else np.zeros(len(self.position)), dtype=np.uint8)
        self.n = len(self.position)
        self.box, self.grid = tuple(box), tuple(grid)
        self.h = self.L.or_create(*box, *grid, self.n, _ptr(self.position), _ptr(self.material),
                                  gridspace, wavenum, nthreads)
        self.L.or_set_interaction(self.h, {"poi": 0, "fcd": 1, "fcd_st": 2, "nloc": 3, "nloc_av": 4, "igt_so": 5,
                                           "so": 6}[interaction])
        self.L.or_set_nloc_rp(self.h, nloc_rp)
        if int_tables is not None:
            t = np.ascontiguousarray(int_tables, dtype=np.float64)
            self.L.or_set_tables(self.h, _ptr(t), complex(so_m).real, complex(so_m).imag)
        if surface is not None:  # dict(zsum_shift, msub (None: perfect reflector), relation img|som, data: som table)
            m = surface.get("msub")
            tab = surface.get("data") if surface.get("relation", "img") == "som" else None
            tab = None if tab is None else np.ascontiguousarray(tab, dtype=np.complex128)
            mm = complex(0 if m is None else m)
            self.L.or_set_surface(self.h, surface["zsum_shift"], mm.real, mm.imag, 1 if m is None else 0,
                                  None if tab is None else _ptr(tab))
        self.L.or_init_dmatrix(self.h)

    def close(self):
        if self.h:
            self.L.or_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rmatrix(self):
        n = self.L.or_rmatrix_len(self.h)
        out = np.empty(n, dtype=np.complex128)
        self.L.or_get_rmatrix(self.h, _ptr(out))
        return out

    def cross_beam(self, p, einc, inc_scale=1.0):
        ce, ca = ctypes.c_double(), ctypes.c_double()
        p = np.ascontiguousarray(p, dtype=np.complex128)
        e = np.ascontiguousarray(einc, dtype=np.complex128)
        self.L.or_cross_beam(self.h, _ptr(p), _ptr(e), inc_scale, ctypes.byref(ce), ctypes.byref(ca))
        return ce.value, ca.value

    def dmatrix(self):
        n = self.L.or_dmatrix_len(self.h)
        out = np.empty(n, dtype=np.complex128)
        self.L.or_get_dmatrix(self.h, _ptr(out))
        return out

    def set_cc(self, cc):
        """cc: complex [nmat,3] per material or [ndip,3] per dipole (flag by shape)."""
        cc = np.ascontiguousarray(cc, dtype=np.complex128)
        if cc.ndim == 2 and cc.shape[0] == self.n and cc.shape[0] > 255:
            self.L.or_set_cc_dip(self.h, _ptr(cc))
        else:
            self.L.or_set_cc_mat(self.h, cc.shape[0], _ptr(cc))

    def set_cc_dipole(self, cc):
        cc = np.ascontiguousarray(cc, dtype=np.complex128).reshape(self.n, 3)
        self.L.or_set_cc_dip(self.h, _ptr(cc))

    def matvec(self, x, her=False):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(x)
        ip = ctypes.c_double(0)
        self.L.or_matvec(self.h, _ptr(x), _ptr(y), ctypes.byref(ip), int(her))
        return y, ip.value

    def solve(self, einc, method=QMR_CS, eps=1e-5, maxiter=100000, init_field=IF_AUTO, hist_cap=100000, x0=None,
              chp_in=None, chp_save=False):
        """chp_in: the reference's checkpoint bytes to resume from (resid then starts at the saved iteration);
        chp_save: also return the final state as checkpoint bytes ('chp', like -chp_type always)"""
        einc = np.ascontiguousarray(einc, dtype=np.complex128)
        x = np.empty_like(einc) if x0 is None else np.array(x0, dtype=np.complex128)
        p = np.empty_like(einc)
        hist = np.zeros(hist_cap)
        nit = ctypes.c_int(0)
        cin = None if chp_in is None else ctypes.create_string_buffer(bytes(chp_in), len(chp_in))
        cap = 64 + 8 * 16 + 8 * x.size * 16
        cout = ctypes.create_string_buffer(cap) if chp_save else None
        clen = ctypes.c_size_t(cap)
        st = self.L.or_solve_chp(self.h, method, _ptr(einc), eps, maxiter, init_field, _ptr(x), _ptr(p), _ptr(hist),
                                 hist_cap, ctypes.byref(nit), cin, 0 if chp_in is None else len(chp_in), cout,
                                 ctypes.byref(clen) if chp_save else None)
        if st < 0:
            raise ValueError("checkpoint is for another iterative method or vector size")
        first = 0
        if chp_in is not None:
            first = int(np.frombuffer(bytes(chp_in)[12:16], np.int32)[0]) - 1
        res = dict(status=st, niter=nit.value, x=x, p=p, resid=hist[:min(nit.value + 1 - first, hist_cap)])
        if chp_save:
            res["chp"] = cout.raw[:clen.value]
        return res

    def cross(self, pvec, prop, incpol):
        pvec = np.ascontiguousarray(pvec, dtype=np.complex128)
        prop = np.ascontiguousarray(prop, dtype=np.float64)
        incpol = np.ascontiguousarray(incpol, dtype=np.float64)
        ce, ca = ctypes.c_double(0), ctypes.c_double(0)
        self.L.or_cross(self.h, _ptr(pvec), _ptr(prop), _ptr(incpol), ctypes.byref(ce), ctypes.byref(ca))
        return ce.value, ca.value

    def field(self, pvec, n):
        """scattering amplitude (CalcFieldFree) for the unit direction n: complex [3]"""
        pvec = np.ascontiguousarray(pvec, dtype=np.complex128)
        n = np.ascontiguousarray(n, dtype=np.float64)
        e = np.zeros(3, np.complex128)
        self.L.or_field(self.h, _ptr(pvec), _ptr(n), _ptr(e))
        return e


# ---- integrals over the scattering directions (src/crosssec.c:233-307, 991-1260; src/Romberg.c:175-533) ----
# parms: dict(min, max, Jmin, Jmax, eps, equiv, periodic) per angle, degrees, as in alldir_params.dat
ALLDIR_DEFAULT = (dict(min=0.0, max=180.0, Jmin=2, Jmax=6, eps=0.0, equiv=False, periodic=False),
                  dict(min=0.0, max=360.0, Jmin=2, Jmax=5, eps=0.0, equiv=True, periodic=True))


def alldir_angles(p, in_cos):
    """grid angles in degrees: equal steps in cos for theta (from max down to min), in the angle for phi"""
    if p["min"] == p["max"]:
        return np.array([p["min"]])
    G = 2 ** p["Jmax"] + 1
    n = G - 1 if p["equiv"] else G
    if in_cos:
        lo, hi = np.cos(np.deg2rad(p["max"])), np.cos(np.deg2rad(p["min"]))
        lo = 0.0 if abs(lo) < 1e-15 else lo
        hi = 0.0 if abs(hi) < 1e-15 else hi
        unit = (hi - lo) / (G - 1)
        return np.array([np.rad2deg(np.arccos(lo + unit * i)) for i in range(n)])
    unit = (p["max"] - p["min"]) / (G - 1)
    return np.array([p["min"] + unit * i for i in range(n)])


def _romberg(p, f, dim):
    """one level of the bracketing Romberg scheme (Davis & Rabinowitz 6.3; trapezoid rule when periodic) over the
    points 0..G-1 of a variable; f(i) -> (values[dim], abs error). Returns (average, abs error, rel error)."""
    if p["min"] == p["max"]:
        v, e = f(0)
        return v, e, (0.0 if v[0] == 0 else e / abs(v[0]))
    J, G = p["Jmax"], 2 ** p["Jmax"] + 1
    c1 = [4.0 ** i for i in range(J + 1)]
    c2 = [0.0] + [1 / (c1[i] - 1) for i in range(1, J + 1)]
    c3 = [2 * c1[i] - 1 for i in range(J + 1)]
    M = [np.zeros(dim) for _ in range(J + 1)]
    T = np.zeros(dim)
    abs_err = err = int_err = 0.0
    m0 = 0
    for m in range(J):
        if m == 0:
            T, int_err = f(0)
            T = np.array(T, dtype=float)
            if not p["equiv"]:
                vl, el = f(G - 1)
                int_err = 0.5 * (int_err + el)
                T = 0.5 * (vl + T)
        elif p["periodic"]:
            T = 0.5 * (T + M[0])
        else:
            T = c3[m - 1] * c2[m] * (T - M[0]) + M[0]
            m0 = m
        step = (G - 1) >> m
        acc, e = np.zeros(dim), 0.0
        for j in range(step >> 1, G, step):
            v, ej = f(j)
            acc = acc + v
            e += ej
        sc = 2.0 ** (-m)
        M[m0] = acc * sc
        int_err = 0.5 * (int_err + e * sc)
        if m0 != 0:
            for k in range(m - 1, -1, -1):
                M[k] = c2[m - k] * (c1[m - k] * M[k + 1] - M[k])
        if m >= p["Jmin"] - 1:
            abs_res = 0.5 * abs(M[0][0] + T[0])
            abs_err = 0.5 * abs(M[0][0] - T[0]) + int_err
            err = 0.0 if abs_res == 0 else abs_err / abs_res
            if err < p["eps"]:
                break
    return 0.5 * (M[0] + T), abs_err, err


def romberg2d(parms, values, poles=False, used=None):
    """Romberg2D: average of values [ntheta][nphi][dim] over theta (outer, cos spacing) and phi (inner); poles: the
    outer end points at 180 and 0 degrees use their first inner value alone (orientation averaging over the full
    alpha range, OuterInitT's onepoint, src/Romberg.c:347-360)"""
    values = np.asarray(values, dtype=float)
    nphi = values.shape[1]
    nth = values.shape[0]

    def inner(i):
        full = parms[0]["min"] != parms[0]["max"]
        if poles and full and ((i == 0 and parms[0]["max"] == 180) or (i == nth - 1 and parms[0]["min"] == 0)):
            if used is not None:
                used.add((i, 0))
            return values[i, 0], 0.0

        def g(j):
            if used is not None:
                used.add((i, j if j < nphi else j - nphi))
            return values[i, j if j < nphi else j - nphi], 0.0
        r, e, _ = _romberg(parms[1], g, values.shape[2])
        return r, e
    return _romberg(parms[0], inner, values.shape[2])[0]


def scattering_integrals(o, pvec, prop, incx, incy, wavenum, parms=ALLDIR_DEFAULT):
    """Csca and Csca*g (beam frame) from the oracle's scattering amplitude on the alldir grid (CalcAlldir, ScaCross,
    AsymParm_x/y/z)"""
    th, ph = alldir_angles(parms[0], True), alldir_angles(parms[1], False)
    prop, incx, incy = (np.asarray(v, dtype=float) for v in (prop, incx, incy))
    e2 = np.zeros((len(th), len(ph)))
    for i, t in enumerate(th):
        ct, st = np.cos(np.deg2rad(t)), np.sin(np.deg2rad(t))
        for j, f in enumerate(ph):
            n = ct * prop + st * (np.cos(np.deg2rad(f)) * incx + np.sin(np.deg2rad(f)) * incy)
            e = o.field(pvec, n)
            e2[i, j] = np.sum(np.abs(e) ** 2)
    scale = 4 * np.pi / wavenum ** 2
    csca = romberg2d(parms, e2[:, :, None])[0] * scale
    tr, pr = np.deg2rad(th)[:, None], np.deg2rad(ph)[None, :]
    gx = np.where(th[:, None] == 180, 0.0, e2 * np.sin(tr) * np.cos(pr))
    gy = np.where(th[:, None] == 180, 0.0, e2 * np.sin(tr) * np.sin(pr))
    gz = e2 * np.cos(tr)
    cg = np.array([romberg2d(parms, g[:, :, None])[0] * scale for g in (gx, gy, gz)])
    return csca, cg


def fftfit(x, divis=1):
    return lib().or_fftfit(x, divis)


def run_reference(args, workdir):
    """Run the reference build (oracle/_ref/adda) with a command line; returns (stdout, run directory)."""
    os.makedirs(workdir, exist_ok=True)
    rundir = os.path.join(workdir, "run")
    out = subprocess.run([REF_BIN] + list(args) + ["-dir", rundir], cwd=workdir, capture_output=True, text=True,
                         check=True)
    return out.stdout, rundir

"""Shared helpers for the tests: build the reference-equivalent inputs for a golden case, run the oracle on them."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_runs.json")

SETUP_KEYS = ("grid", "shape", "pars", "m", "dpl", "size", "pol", "orient", "avgpol", "prop", "interaction", "nloc_rp",
              "pol_rp")
INT_TABLES = os.path.join(HERE, "golden", "int_tables.npy")


def int_tables():
    """the reference's igt_so / so integral tables (fixture made by golden/make_int_tables.py)"""
    return np.load(INT_TABLES)


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def case(name):
    for c in golden()["cases"]:
        if c["name"] == name:
            return c
    raise KeyError(name)


def setup_for(kw):
    import adda_gb300 as A
    args = {k: v for k, v in kw.items() if k in SETUP_KEYS}
    if isinstance(args.get("m"), list):
        args["m"] = complex(*args["m"])
    if args.get("interaction") in ("igt_so", "so"):
        args["int_tables"] = int_tables()
    return A.Setup(**args)


def solver_opts(kw):
    return dict(method=kw.get("iter", "qmr"), eps=kw.get("eps", 1e-5), maxiter=kw.get("maxiter", 100000),
                init=kw.get("init", "auto"))


def oracle_for(s, nthreads=0):
    from oracle import oracle as O
    o = O.Oracle(s.box, s.grid, s.pos, s.mat, s.gridspace, s.wavenum, nthreads,
                 interaction=getattr(s, "interaction", "poi"), nloc_rp=getattr(s, "nloc_rp", 0.0),
                 surface=getattr(s, "surface", None), int_tables=getattr(s, "int_tables", None),
                 so_m=getattr(s, "m", 0.0))
    return o


def wkb_x0(s, pol_index):
    """the reference's -init_field wkb starting vector for polarisation pol_index: the WKB field of the product's host
    code turned into x_0 (InitFieldfromE)"""
    import adda_gb300 as A
    e = A.wkb_field(s.box, s.pos, s.mat, [s.m], s.kd, s.einc[pol_index])
    return A.field_to_x0(e, s.cc[pol_index].reshape(1, 3), [s.m], s.gridspace, s.mat)


def oracle_solve(o, s, pol_index, method="qmr", eps=1e-5, maxiter=100000, init="auto", x0=None, chp_in=None,
                 chp_save=False):
    if init == "wkb":
        init, x0 = "x0", wkb_x0(s, pol_index)
    from oracle import oracle as O
    o.set_cc(s.cc[pol_index].reshape(1, 3))
    methods = {"qmr": O.QMR_CS, "bicgstab": O.BICGSTAB, "bicg": O.BICG_CS, "cgnr": O.CGNR, "csym": O.CSYM,
               "qmr2": O.QMR_CS_2, "bcgs2": O.BCGS2}
    r = o.solve(s.einc[pol_index], method=methods[method], eps=eps, maxiter=maxiter,
                init_field={"auto": O.IF_AUTO, "zero": O.IF_ZERO, "inc": O.IF_INC, "x0": O.IF_X0}[init], x0=x0,
                chp_in=chp_in, chp_save=chp_save)
    ce, ca = o.cross(r["p"], s.prop, s.incpol[pol_index])
    r["Cext"], r["Cabs"] = ce, ca
    return r


CHP_SCALARS = {"bcgs2": "cc", "bicg": "c", "bicgstab": "ccc", "cgnr": "d", "csym": "dddccc", "qmr": "ddddcccc",
               "qmr2": "dddcc"}  # d: double, c: doublecomplex, in the order of each method's PHASE_VARS


def parse_chpoint(raw, method):
    """the reference's chp.<ringid> bytes (SaveIterChpoint, iterative.c:165-218): (ind_m, nRows, niter, counter,
    inprodR, prev_err, resid_scale), [scalars], vectors [k][nRows] (xvec, rvec, pvec, then the method's own)"""
    import struct
    head = struct.unpack("<iQiiddd", raw[:44])
    off, sc = 44, []
    for t in CHP_SCALARS[method]:
        if t == "d":
            sc.append(struct.unpack("<d", raw[off:off + 8])[0])
            off += 8
        else:
            sc.append(complex(*struct.unpack("<dd", raw[off:off + 16])))
            off += 16
    return head, sc, np.frombuffer(raw[off:], np.complex128).reshape(-1, head[1])


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

"""Generate tests/golden/reference_surface.json (+ som_<case>.npy): the UNMODIFIED reference (sequential build of
oracle/Makefile) with a particle near a substrate (-surf h m_re m_im | -surf h inf; make_particle.c:2309, fft.c:818-887,
interaction.c:1082-1345, GenerateB.c:96-140,257-323). Records per case the lattice, the substrate, Cext and Cabs of
both polarisations (CrossSec-Y/-X), the total iteration count and, for the image-relation cases, the incident beam at every dipole
(-store_beam).

For the cases with the Sommerfeld-integral relation (-int_surf som) the table of the four Sommerfeld integrals the
reference combines into the reflected Green's tensor (CalcSomTable/SingleSomIntegral, interaction.c:1157-1224) is
computed with the reference's own som_init/evlua (somnec.c, built alone by `make -C oracle som`) on the rectangular
grid the library takes: [k < 2*boxZ-1][j < boxY][i < boxX][4] at rho = hypot(i,j)*d, z = (k + ZsumShift)*d.

Run from the repository root:  python tests/golden/make_surface.py [/path/to/reference/src]
"""
import ctypes
import json
import math
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "a-dda_gb300"))

EPS = ["-eps", "10"]
# name, particle arguments, setup, substrate (h, msub or None for inf, relation), propagation (None = the default +z)
CASES = [
    ("img_above", ["-grid", "8", "-m", "1.5", "0.1"], dict(grid=8, m=[1.5, 0.1]), (2.0, [2.0, 0.5], "img"), [1, 2, -3]),
    ("img_below", ["-grid", "8", "-m", "1.5", "0.1"], dict(grid=8, m=[1.5, 0.1]), (2.0, [2.0, 0.5], "img"), None),
    ("inf_above", ["-grid", "8", "-m", "1.5", "0.1"], dict(grid=8, m=[1.5, 0.1]), (2.0, None, "img"), [1, 2, -3]),
    ("som_above", ["-grid", "8", "-m", "1.5", "0.1"], dict(grid=8, m=[1.5, 0.1]), (2.0, [1.5, 0.2], "som"), [0, 1, -2]),
    ("som_below", ["-grid", "8", "-m", "1.5", "0.1"], dict(grid=8, m=[1.5, 0.1]), (2.5, [1.5, 0.2], "som"), None),
    ("img_ell10", ["-grid", "10", "-shape", "ellipsoid", "0.7", "1.3", "-m", "1.3", "0.05"],
     dict(grid=10, m=[1.3, 0.05], shape="ellipsoid", pars=[0.7, 1.3]), (3.0, [1.3, 0.05], "img"), [1, 0, -1]),
]


class _Cplx(ctypes.Structure):
    _fields_ = [("re", ctypes.c_double), ("im", ctypes.c_double)]


def som_table(libpath, msub, box, gridspace, zsum, wavenum=1.0):
    """the reference's SingleSomIntegral (interaction.c:1157-1172) over the library's rectangular grid"""
    L = ctypes.CDLL(libpath)
    L.som_init.argtypes = [_Cplx]
    L.evlua.argtypes = [ctypes.c_double, ctypes.c_double] + [ctypes.POINTER(_Cplx)] * 4
    m2 = complex(*msub) ** 2
    L.som_init(_Cplx(m2.real, m2.imag))
    scale = wavenum / (2 * math.pi)
    isc = scale ** 3
    bX, bY, bZ = box
    out = np.zeros((2 * bZ - 1, bY, bX, 4), np.complex128)
    v = [_Cplx() for _ in range(4)]
    for k in range(2 * bZ - 1):
        z = (k + zsum) * gridspace
        for j in range(bY):
            for i in range(bX):
                rho = math.hypot(i, j) * gridspace
                if rho == 0:
                    rho = z * 0.00000001
                L.evlua(z * scale, rho * scale, *[ctypes.byref(x) for x in v])
                out[k, j, i] = [complex(x.re, x.im) * isc for x in v]
    return out


def read_beam(path):
    rows = [list(map(float, ln.split())) for ln in open(path).read().splitlines()[1:] if ln.strip()]
    a = np.array(rows)
    return (a[:, 4::2] + 1j * a[:, 5::2]), a[:, :3]


def main(ref_src=None):
    from oracle import oracle as O
    import adda_gb300 as A
    binp = O.build_reference(ref_src)
    if not binp:
        raise SystemExit("reference sources not found at " + (ref_src or O.ref_src_dir()))
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "som", "REF_SRC=" + (ref_src or O.ref_src_dir())], check=True)
    somlib = os.path.join(ROOT, "oracle", "_ref", "libsomnec.so")
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, part, setup, (h, msub, rel), prop in CASES:
            surf = ["-surf", repr(h)] + (["inf"] if msub is None else [repr(msub[0]), repr(msub[1])])
            args = part + surf + ["-int_surf", rel] + (["-prop"] + [str(p) for p in prop] if prop else []) + EPS + \
                ["-sym", "no"]
            rd = os.path.join(tmp, name)
            p = subprocess.run([binp] + args + ["-store_beam", "-dir", rd], cwd=tmp, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError(name + ": " + p.stdout + p.stderr)
            res = dict(name=name, args=args, setup=setup, hsub=h, msub=msub, relation=rel, prop=prop)
            for pol in ("Y", "X"):
                cs = open(os.path.join(rd, "CrossSec-" + pol)).read()
                res["Cext_" + pol] = float(re.search(r"Cext\s*=\s*([-+0-9.eE]+)", cs).group(1))
                res["Cabs_" + pol] = float(re.search(r"Cabs\s*=\s*([-+0-9.eE]+)", cs).group(1))
                e, xyz = read_beam(os.path.join(rd, "IncBeam-" + pol))
                if rel == "img":
                    res["beam_" + pol] = [float("%.12g" % v) for v in e.reshape(-1).view(np.float64)]
            # RE_ lines of both polarisations' solves
            res["iterations_total"] = len(re.findall(r"^RE_\d+", p.stdout, re.M)) - 2
            if rel == "som":
                s = A.Setup(**{k: (complex(*v) if k == "m" else v) for k, v in setup.items()})
                zsum = 2 * (h / s.gridspace - (s.box[2] - 1) / 2.0)
                np.save(os.path.join(HERE, "som_%s.npy" % name), som_table(somlib, msub, s.box, s.gridspace, zsum))
            out.append(res)
            print(name, res["Cext_Y"], res["Cabs_Y"], res["Cext_X"], res["Cabs_X"], res["iterations_total"])
    with open(os.path.join(HERE, "reference_surface.json"), "w") as f:
        json.dump(dict(reference="ADDA 1.3b6 sequential build + FFTW-subset shim", cases=out), f)


if __name__ == "__main__":
    main(*sys.argv[1:])

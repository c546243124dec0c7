"""Generate tests/golden/reference_c4_quantised.json: the UNMODIFIED reference (ADDA 1.3b6 sequential build, compiled
from its own sources by oracle/Makefile with this project's FFTW-subset shim) on the differentiation workload's
refractive-index field quantised to 14 materials (tests/c4_workload.py: the 48^3 cube, 7 levels of m_re x 2 of
m_im), read through -shape read from a geometry file this script writes:

    -shape read c4.geom -m <14 pairs> -iter qmr -eps 10 -sym no

(dpl: the reference's default, 10 max|m|). Recorded: dipole count, box, grid, dpl, the coupling constants, the
iterations, and Cext/Cabs of both polarisations as printed (10 digits). Runs a few minutes on one core. From the
repository root:

    python tests/golden/make_c4_quantised.py [/path/to/reference/src]
"""
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))


def write_geom(path, box, mat):
    import numpy as np
    bx, by, bz = box
    z, y, x = np.meshgrid(np.arange(bz), np.arange(by), np.arange(bx), indexing="ij")
    with open(path, "w") as f:
        f.write("#differentiation workload, quantised to 14 materials\n#box size: %dx%dx%d\nNmat=14\n" % box)
        for xi, yi, zi, m in zip(x.ravel(), y.ravel(), z.ravel(), mat):
            f.write("%d %d %d %d\n" % (xi, yi, zi, int(m) + 1))


def main(argv):
    import c4_workload as W
    from make_golden import parse_run
    from oracle import oracle as O
    binp = O.build_reference(argv[0] if argv else None)
    if not binp:
        raise SystemExit("reference sources not found")
    u1, u2 = W.fields()
    mat, levels = W.quantised(u1, u2)
    box = (W.BOX,) * 3
    margs = []
    for m in levels:
        margs += ["%.17g" % m.real, "%.17g" % m.imag]
    with tempfile.TemporaryDirectory() as tmp:
        geom = os.path.join(tmp, "c4.geom")
        write_geom(geom, box, mat)
        args = ["-shape", "read", "c4.geom", "-m"] + margs + ["-iter", "qmr", "-eps", "10", "-sym", "no"]
        rundir = os.path.join(tmp, "run")
        p = subprocess.run([binp] + args + ["-dir", rundir], cwd=tmp, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(p.stdout + p.stderr)
        res = parse_run(rundir, p.stdout)
        log = open(os.path.join(rundir, "log")).read()
        res["dpl"] = float(re.search(r"Dipoles/lambda:\s*([0-9.eE+-]+)", log).group(1))
        res["niter"] = {pol: len(h) - 1 for pol, h in res["resid"].items()}
        del res["resid"]
    out = dict(reference="ADDA 1.3b6 sequential build + FFTW-subset shim",
               args=args[:3] + ["-m", "<14 levels>"] + args[4 + len(margs):],
               levels=[[m.real, m.imag] for m in levels], run=res)
    with open(os.path.join(HERE, "reference_c4_quantised.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main(sys.argv[1:])

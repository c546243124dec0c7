"""Generate tests/golden/reference_orient_avg.json: the UNMODIFIED reference (sequential build of oracle/Makefile) with
`-orient avg <file>` (orientation averaging, calculator.c:293-358,690-710) on a sphere and an ellipsoid, with the
reference's default integration parameters and with variants (every grid point used, eps = 0; a partial range of the
first Euler angle, where beta = 0 and 180 are no longer single orientations). Records the averaged Cext and Cabs from
CrossSec and the number of orientations the adaptive integration evaluated (log_orient_avg).

Run from the repository root:  python tests/golden/make_orient_avg.py [/path/to/reference/src]
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

M = ["-m", "1.1", "0.1", "-grid", "8"]
ELL = ["-shape", "ellipsoid", "0.5", "1.5"]
# blocks alpha, beta, gamma: min, max, Jmin, Jmax, eps, equiv, periodic (the first one is the reference's default)
PARMS = {
    "default": ((0, 360, 2, 5, 0, True, True), (0, 180, 2, 4, 1e-3, False, False), (0, 360, 2, 4, 1e-3, True, True)),
    "full": ((0, 360, 2, 5, 0, True, True), (0, 180, 2, 3, 0, False, False), (0, 360, 2, 3, 0, True, True)),
    "half_alpha": ((0, 180, 2, 4, 0, False, False), (0, 180, 2, 3, 0, False, False), (0, 360, 2, 3, 0, True, True)),
}
CASES = [
    ("sphere_default", M, dict(grid=8, m=[1.1, 0.1]), "default"),
    ("ell_default", ELL + M, dict(grid=8, m=[1.1, 0.1], shape="ellipsoid", pars=[0.5, 1.5]), "default"),
    ("ell_full", ELL + M, dict(grid=8, m=[1.1, 0.1], shape="ellipsoid", pars=[0.5, 1.5]), "full"),
    ("ell_half_alpha", ELL + M, dict(grid=8, m=[1.1, 0.1], shape="ellipsoid", pars=[0.5, 1.5]), "half_alpha"),
]


def avg_file(path, kind):
    with open(path, "w") as f:
        for name, (lo, hi, jmin, jmax, eps, eq, per) in zip(("alpha", "beta", "gamma"), PARMS[kind]):
            f.write("%s:\nmin=%g\nmax=%g\nJmin=%d\nJmax=%d\neps=%g\nequiv=%s\nperiodic=%s\n\n" % (
                name, lo, hi, jmin, jmax, eps, "true" if eq else "false", "true" if per else "false"))


def main(ref_src=None):
    from oracle import oracle as O
    binp = O.build_reference(ref_src)
    if not binp:
        raise SystemExit("reference sources not found at " + (ref_src or O.ref_src_dir()))
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, args, setup, kind in CASES:
            pf = os.path.join(tmp, name + "_avg.dat")
            avg_file(pf, kind)
            rd = os.path.join(tmp, name)
            full = args + ["-orient", "avg", pf, "-sym", "no"]
            p = subprocess.run([binp] + full + ["-dir", rd], cwd=tmp, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError(name + ": " + p.stdout + p.stderr)
            cs = open(os.path.join(rd, "CrossSec")).read()
            ev = open(os.path.join(rd, "log_orient_avg")).read()
            out.append(dict(name=name, args=full[:-len(["-orient", "avg", pf, "-sym", "no"])] + ["-orient", "avg",
                                                                                                   "-sym", "no"],
                            setup=setup, parms=kind,
                            Cext=float(re.search(r"Cext\s*=\s*([-+0-9.eE]+)", cs).group(1)),
                            Cabs=float(re.search(r"Cabs\s*=\s*([-+0-9.eE]+)", cs).group(1)),
                            evaluations=int(re.search(r"In total (\d+) evaluations", ev).group(1))))
            print(out[-1])
    with open(os.path.join(HERE, "reference_orient_avg.json"), "w") as f:
        json.dump(dict(reference="ADDA 1.3b6 sequential build + FFTW-subset shim", parms=PARMS, cases=out), f,
                  indent=1)


if __name__ == "__main__":
    main(*sys.argv[1:])

"""Generate tests/golden/reference_c2.json: the UNMODIFIED reference (ADDA 1.3b6 sequential build compiled from its
own sources by oracle/Makefile with this project's FFTW-subset shim) on the 128^3 sphere workload,

    -grid 128 -dpl 15 -m 1.33 0.01 -iter {qmr,bicgstab} -eps 5 -sym no

both polarisations. Each run takes about two hours on one core; the two run in parallel. Run from the repository
root:

    python tests/golden/make_reference_c2.py [/path/to/reference/src]
    python tests/golden/make_reference_c2.py --parse QMR_RUNDIR BICGSTAB_RUNDIR   # record finished runs

Recorded per method: dipole count, box, grid, coupling constant, iterations per polarisation, Cext/Cabs of both
polarisations, and the reference's own total wall time (single thread, x86 host of the generating machine).

With --converged it writes tests/golden/reference_c2_converged.json instead: the same workload solved by the
reference to relative residual 1e-8 with both methods (-eps 8, the reference's default symmetry handling: the sphere
is symmetric, so it solves the Y polarisation and X equals it), 1.6-1.7 hours per method on one core, and their
mean as the converged cross sections:

    python tests/golden/make_reference_c2.py --converged [/path/to/reference/src]
    python tests/golden/make_reference_c2.py --parse-converged QMR_RUNDIR BICGSTAB_RUNDIR
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

ARGS = ["-grid", "128", "-dpl", "15", "-m", "1.33", "0.01", "-eps", "5", "-sym", "no"]


def parse(rundir):
    from make_golden import parse_run
    res = parse_run(rundir, "")
    log = open(os.path.join(rundir, "log")).read()
    res["niter"] = {pol: len(h) - 1 for pol, h in res["resid"].items()}
    res["resid_final"] = {pol: h[-1] for pol, h in res["resid"].items()}
    del res["resid"]
    res["wall_s"] = float(re.search(r"Total wall time:\s*([0-9.]+)", log).group(1))
    res["total_iterations"] = int(re.search(r"Total number of iterations: (\d+)", log).group(1))
    return res


def write(runs):
    out = dict(reference="ADDA 1.3b6 sequential build + FFTW-subset shim, one thread",
               args=ARGS, setup=dict(grid=128, m=[1.33, 0.01], dpl=15), runs=runs)
    with open(os.path.join(HERE, "reference_c2.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


TIGHT = ["-grid", "128", "-dpl", "15", "-m", "1.33", "0.01", "-eps", "8"]


def write_converged(runs):
    ce = [r["cross"]["Y"]["Cext"] for r in runs.values()]
    ca = [r["cross"]["Y"]["Cabs"] for r in runs.values()]
    out = dict(reference="ADDA 1.3b6 sequential build + FFTW-subset shim, one thread", args=TIGHT,
               setup=dict(grid=128, m=[1.33, 0.01], dpl=15), runs=runs,
               converged=dict(Cext=sum(ce) / len(ce), Cabs=sum(ca) / len(ca),
                              spread=dict(Cext=abs(ce[0] / ce[1] - 1), Cabs=abs(ca[0] / ca[1] - 1))))
    with open(os.path.join(HERE, "reference_c2_converged.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


def main(argv):
    if argv and argv[0] == "--parse":
        write({"qmr": parse(argv[1]), "bicgstab": parse(argv[2])})
        return
    if argv and argv[0] == "--parse-converged":
        write_converged({"qmr": parse(argv[1]), "bicgstab": parse(argv[2])})
        return
    converged = bool(argv) and argv[0] == "--converged"
    if converged:
        argv = argv[1:]
    from oracle import oracle as O
    binp = O.build_reference(argv[0] if argv else None)
    if not binp:
        raise SystemExit("reference sources not found")
    with tempfile.TemporaryDirectory() as tmp:
        procs = {}
        for m in ("qmr", "bicgstab"):
            procs[m] = subprocess.Popen([binp] + (TIGHT if converged else ARGS) + ["-iter", m, "-dir",
                                        os.path.join(tmp, m)], cwd=tmp, stdout=subprocess.DEVNULL)
        for m, p in procs.items():
            if p.wait() != 0:
                raise RuntimeError(m + " run failed")
        (write_converged if converged else write)({m: parse(os.path.join(tmp, m)) for m in procs})


if __name__ == "__main__":
    main(sys.argv[1:])

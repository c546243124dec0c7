"""Generate the checkpoint fixtures: tests/golden/chpoint/<method>.chp and tests/golden/reference_chpoint.json.

For each of the reference's seven iterative solvers, the UNMODIFIED reference (sequential build of oracle/Makefile)
runs twice on a small sphere (-grid 6 -m 1.5 0.1, one incident polarisation by symmetry, which the reference's
checkpoints require, param.c:2173):

1. `-maxiter 4 -chpoint 0s` (`-maxiter 2` for BCGS2; chp_type ALWAYS, param.c:1011-1015): the iterations, then
   SaveIterChpoint (iterative.c:165-218) writes <chp_dir>/chp.0 -- kept here byte for byte;
2. `-chp_load` from that directory: LoadIterChpoint (iterative.c:222-278) and the solve continues to -eps 10; the
   residual history after the saved iteration and CrossSec-Y are recorded.

Run from the repository root:  python tests/golden/make_chpoint.py [/path/to/reference/src]
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

BASE = ["-grid", "6", "-m", "1.5", "0.1", "-eps", "10"]
SAVE_AFTER = {"bcgs2": 2}  # iterations before the checkpoint; default 4 (BCGS2 takes two BiCG steps per iteration)
METHODS = ["bcgs2", "bicg", "bicgstab", "cgnr", "csym", "qmr", "qmr2"]


def history(log):
    return {int(m.group(1)): float(m.group(2)) for m in re.finditer(r"RE_(\d+) = ([-+0-9.E]+)", log)}


def cross(rundir):
    txt = open(os.path.join(rundir, "CrossSec-Y")).read()
    return {q: float(re.search(q + r"\s*=\s*([-+0-9.eE]+)", txt).group(1)) for q in ("Cext", "Cabs")}


def main(ref_src=None):
    from oracle import oracle as O
    binp = O.build_reference(ref_src)
    if not binp:
        raise SystemExit("reference sources not found at " + (ref_src or O.ref_src_dir()))
    out_dir = os.path.join(HERE, "chpoint")
    os.makedirs(out_dir, exist_ok=True)
    cases = []
    with tempfile.TemporaryDirectory() as tmp:
        for meth in METHODS:
            chp = os.path.join(tmp, meth + "_chp")
            save_args = BASE + ["-iter", meth, "-maxiter", str(SAVE_AFTER.get(meth, 4)), "-chpoint", "0s",
                                "-chp_dir", chp]
            load_args = BASE + ["-iter", meth, "-chp_load", "-chp_dir", chp]
            r1, r2 = os.path.join(tmp, meth + "_save"), os.path.join(tmp, meth + "_load")
            for args, rd in ((save_args, r1), (load_args, r2)):
                p = subprocess.run([binp] + args + ["-dir", rd], cwd=tmp, capture_output=True, text=True)
                if p.returncode != 0:
                    raise RuntimeError(meth + ": " + p.stdout + p.stderr)
                if rd == r1:
                    shutil.copyfile(os.path.join(chp, "chp.0"), os.path.join(out_dir, meth + ".chp"))
            log1, log2 = open(os.path.join(r1, "log")).read(), open(os.path.join(r2, "log")).read()
            assert "Checkpoint (iteration) saved" in log1 and "Checkpoint (iteration) loaded" in log2
            h1, h2 = history(log1), history(log2)
            ndip = int(re.search(r"Total number of occupied dipoles: (\d+)", log1).group(1))
            cases.append(dict(method=meth, save_args=save_args, load_args=load_args, ndip=ndip,
                              resid_before=[h1[i] for i in sorted(h1)], first_loaded=min(h2),
                              resid_after=[h2[i] for i in sorted(h2)], cross=cross(r2),
                              chp_bytes=os.path.getsize(os.path.join(out_dir, meth + ".chp"))))
            print(meth, ndip, len(h1), min(h2), len(h2), cases[-1]["cross"])
    with open(os.path.join(HERE, "reference_chpoint.json"), "w") as f:
        json.dump(dict(reference="ADDA 1.3b6 sequential build + FFTW-subset shim", setup=dict(grid=6, m=[1.5, 0.1]),
                       eps=1e-10, cases=cases), f, indent=1)


if __name__ == "__main__":
    main(*sys.argv[1:])

"""Generate the fixtures of the tabulated interaction terms (-int igt_so, -int so):

- tests/golden/int_tables.npy: the reference's integral tables input/tables/t1f.dat .. t10f.dat (11928 doubles, read
  with the library's adda_gb300_read_int_tables), so that the GPU machine, which has no reference tree, can build D;
- tests/golden/reference_int_tables.json: runs of the UNMODIFIED reference (ADDA 1.3b6 sequential build from
  oracle/Makefile) with those terms, recorded like tests/golden/make_golden.py records its cases. Small dipoles per
  wavelength keep only nearest neighbours in the tabulated ("close") range; dpl 400-800 brings offsets up to the
  table's radius of 10 lattice units into it.

From the repository root:

    python tests/golden/make_int_tables.py [/path/to/reference/src]
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "a-dda_gb300"))

M = ["-m", "1.1", "0.1"]
ELL = ["-shape", "ellipsoid", "0.5", "1.5"]
# (name, reference arguments, keyword arguments of adda_gb300.Setup + solver options)
CASES = [
    ("igt_so_mgn", ["-int", "igt_so", "-grid", "8"] + M, dict(grid=8, m=1.1 + 0.1j, interaction="igt_so")),
    ("so_mgn", ["-int", "so", "-grid", "8"] + M, dict(grid=8, m=1.1 + 0.1j, interaction="so")),
    ("igt_so_c1", ["-int", "igt_so", "-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-eps", "10"],
     dict(grid=16, m=1.5, dpl=10, interaction="igt_so", eps=1e-10)),
    ("igt_so_dpl600", ["-int", "igt_so", "-grid", "12", "-dpl", "600", "-m", "1.3", "0.05", "-eps", "10"],
     dict(grid=12, m=1.3 + 0.05j, dpl=600, interaction="igt_so", eps=1e-10)),
    ("so_ell_dpl400", ["-int", "so", "-dpl", "400", "-orient", "10", "20", "30", "-eps", "10", "-grid", "12"] + ELL + M,
     dict(grid=12, m=1.1 + 0.1j, dpl=400, interaction="so", shape="ellipsoid", pars=(0.5, 1.5), orient=(10, 20, 30),
          eps=1e-10)),
    ("so_box_dpl800_bicgstab", ["-int", "so", "-shape", "box", "-grid", "10", "-dpl", "800", "-m", "1.4", "0.02",
                                "-iter", "bicgstab", "-eps", "10"],
     dict(grid=10, m=1.4 + 0.02j, dpl=800, interaction="so", shape="box", iter="bicgstab", eps=1e-10)),
]


def main(argv):
    import adda_gb300 as A
    from make_golden import parse_run
    from oracle import oracle as O
    src = argv[0] if argv else O.ref_src_dir()
    binp = O.build_reference(src)
    if not binp:
        raise SystemExit("reference sources not found at " + src)
    tabdir = os.path.join(os.path.dirname(os.path.abspath(src)), "input", "tables")
    tables = A.read_int_tables(tabdir)
    np.save(os.path.join(HERE, "int_tables.npy"), tables)
    results = []
    with tempfile.TemporaryDirectory() as tmp:
        os.symlink(tabdir, os.path.join(tmp, "tables"))  # the reference reads tables/t*f.dat from its working dir
        for name, args, kw in CASES:
            full = args + ["-sym", "no"]
            rundir = os.path.join(tmp, name)
            p = subprocess.run([binp] + full + ["-dir", rundir], cwd=tmp, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError(name + ": " + p.stdout + p.stderr)
            res = parse_run(rundir, p.stdout)
            res.update(name=name, args=full, setup=kw)
            results.append(res)
            print(name, res["ndip"], res["grid"], res["cross"], [len(h) for h in res["resid"].values()])
    with open(os.path.join(HERE, "reference_int_tables.json"), "w") as f:
        json.dump(dict(reference="ADDA 1.3b6 sequential build + FFTW-subset shim", cases=results), f, indent=1,
                  default=lambda z: [z.real, z.imag] if isinstance(z, complex) else z)


if __name__ == "__main__":
    main(sys.argv[1:])

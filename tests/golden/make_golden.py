"""Generate tests/golden/reference_runs.json by running the UNMODIFIED reference (ADDA 1.3b6, sequential build
compiled from its own sources by oracle/Makefile with this project's FFTW-subset shim) on command lines taken from
the reference's own differential test suite (tests/2exec/suite) and its published sample run
(sample/run000_sphere_g16_m1.5).

Each case records what the reference printed: dipole count, box, FFT grid, coupling constants, the RE_ residual
history of each polarisation, and Cext/Cabs from CrossSec-Y/-X. Run from the repository root:

    python tests/golden/make_golden.py [/path/to/reference/src]

This script is the only place that executes the reference; the GPU machine never needs it.
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

M = ["-m", "1.1", "0.1"]
ELL = ["-shape", "ellipsoid", "0.5", "1.5"]
MGN = M + ["-grid", "8"]

# (name, reference arguments, keyword arguments of adda_gb300.Setup + solver options)
CASES = [
    ("sample_default", [], dict(grid=16, m=1.5)),
    ("c1_qmr", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-iter", "qmr", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10)),
    ("c1_bicgstab", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-iter", "bicgstab", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10, iter="bicgstab")),
    ("mgn", MGN, dict(grid=8, m=1.1 + 0.1j)),
    ("mgn_eps10", ["-eps", "10"] + MGN, dict(grid=8, m=1.1 + 0.1j, eps=1e-10)),
    ("mgn_init_zero", ["-init_field", "zero"] + MGN, dict(grid=8, m=1.1 + 0.1j, init="zero")),
    ("mgn_init_inc", ["-init_field", "inc"] + MGN, dict(grid=8, m=1.1 + 0.1j, init="inc")),
    ("mgn_bicgstab", ["-iter", "bicgstab"] + MGN, dict(grid=8, m=1.1 + 0.1j, iter="bicgstab")),
    ("mgn_maxiter3", ["-maxiter", "3"] + MGN, dict(grid=8, m=1.1 + 0.1j, maxiter=3)),
    ("mgn_orient30", ["-orient", "30", "0", "0"] + MGN, dict(grid=8, m=1.1 + 0.1j, orient=(30, 0, 0))),
    ("ell_orient", ["-orient", "10", "20", "30"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), orient=(10, 20, 30))),
    ("pol_cm", ["-pol", "cm"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="cm")),
    ("pol_dgf", ["-pol", "dgf"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="dgf")),
    ("pol_rrc", ["-pol", "rrc"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="rrc")),
    ("pol_ldr_prop", ["-pol", "ldr", "-prop", "1", "2", "3"] + MGN,
     dict(grid=8, m=1.1 + 0.1j, prop=(1, 2, 3))),
    ("pol_ldr_avgpol", ["-pol", "ldr", "avgpol", "-prop", "1", "2", "3"] + MGN,
     dict(grid=8, m=1.1 + 0.1j, prop=(1, 2, 3), avgpol=True)),
    ("prop_mz", ["-prop", "0", "0", "-1"] + MGN, dict(grid=8, m=1.1 + 0.1j, prop=(0, 0, -1))),
    ("prop_x", ["-prop", "1", "0", "0"] + MGN, dict(grid=8, m=1.1 + 0.1j, prop=(1, 0, 0))),
    ("prop_ell", ["-prop", "5", "1", "3"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), prop=(5, 1, 3))),
    ("ell24", ["-grid", "24", "-shape", "ellipsoid", "0.7", "0.8", "-m", "1.4", "0.02", "-orient", "10", "20", "30"],
     dict(grid=24, m=1.4 + 0.02j, shape="ellipsoid", pars=(0.7, 0.8), orient=(10, 20, 30))),
    ("box12", ["-shape", "box", "-grid", "12", "-m", "1.3", "0.05"], dict(grid=12, m=1.3 + 0.05j, shape="box")),
    ("c2_small", ["-grid", "32", "-dpl", "15", "-m", "1.33", "0.01", "-iter", "bicgstab", "-eps", "5"],
     dict(grid=32, m=1.33 + 0.01j, dpl=15, iter="bicgstab")),
    # the other solvers of the reference (-iter bicg|cgnr|csym)
    ("mgn_bicg", ["-iter", "bicg"] + MGN, dict(grid=8, m=1.1 + 0.1j, iter="bicg")),
    ("mgn_cgnr", ["-iter", "cgnr"] + MGN, dict(grid=8, m=1.1 + 0.1j, iter="cgnr")),
    ("mgn_csym", ["-iter", "csym"] + MGN, dict(grid=8, m=1.1 + 0.1j, iter="csym")),
    ("c1_bicg", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-iter", "bicg", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10, iter="bicg")),
    ("c1_cgnr", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-iter", "cgnr", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10, iter="cgnr")),
    ("c1_csym", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-iter", "csym", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10, iter="csym")),
    ("ell_bicg_eps8", ["-iter", "bicg", "-eps", "8"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), iter="bicg", eps=1e-8)),
    ("ell_csym_eps8", ["-iter", "csym", "-eps", "8"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), iter="csym", eps=1e-8)),
    ("mgn_qmr2", ["-iter", "qmr2"] + MGN, dict(grid=8, m=1.1 + 0.1j, iter="qmr2")),
    ("c1_qmr2", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-iter", "qmr2", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10, iter="qmr2")),
    ("ell_qmr2_eps8", ["-iter", "qmr2", "-eps", "8"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), iter="qmr2", eps=1e-8)),
    # scattered fields: the Mueller matrix in the yz plane every 10 degrees (-ntheta 18)
    ("mueller_c1", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-eps", "10", "-ntheta", "18"],
     dict(grid=16, m=1.5, dpl=10, eps=1e-10)),
    ("mueller_ell", ["-orient", "10", "20", "30", "-eps", "10", "-ntheta", "18"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), orient=(10, 20, 30), eps=1e-10)),
    # the other polarizability prescriptions (-pol) and interaction terms (-int)
    ("pol_cldr", ["-pol", "cldr", "-prop", "1", "2", "3"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="cldr", prop=(1, 2, 3))),
    ("pol_fcd", ["-pol", "fcd"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="fcd")),
    ("pol_igt_so", ["-pol", "igt_so"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="igt_so")),
    ("pol_lak", ["-pol", "lak"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="lak")),
    ("pol_so", ["-pol", "so"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="so")),
    ("int_fcd", ["-int", "fcd", "-pol", "fcd"] + MGN, dict(grid=8, m=1.1 + 0.1j, pol="fcd", interaction="fcd")),
    ("int_fcd_st", ["-int", "fcd_st", "-pol", "fcd"] + MGN,
     dict(grid=8, m=1.1 + 0.1j, pol="fcd", interaction="fcd_st")),
    ("c1_fcd", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-int", "fcd", "-pol", "fcd", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10, pol="fcd", interaction="fcd")),
    ("ell_fcd_eps8", ["-int", "fcd", "-pol", "fcd", "-eps", "8"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), pol="fcd", interaction="fcd", eps=1e-8)),
    # WKB initial field (-init_field wkb, incidence along z)
    ("mgn_wkb", ["-init_field", "wkb"] + MGN, dict(grid=8, m=1.1 + 0.1j, init="wkb")),
    ("c1_wkb", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-init_field", "wkb", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10, init="wkb")),
    ("ell_wkb_eps8", ["-init_field", "wkb", "-eps", "8"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), init="wkb", eps=1e-8)),
    ("mgn_bcgs2", ["-iter", "bcgs2"] + MGN, dict(grid=8, m=1.1 + 0.1j, iter="bcgs2")),
    # the static non-local interaction and polarizability (-int/-pol nloc|nloc_av <Rp>, Rp in um; d = 0.57 um here)
    ("int_nloc", ["-int", "nloc", "0.3", "-pol", "nloc", "0.3"] + MGN,
     dict(grid=8, m=1.1 + 0.1j, interaction="nloc", nloc_rp=0.3, pol="nloc", pol_rp=0.3)),
    ("int_nloc_av", ["-int", "nloc_av", "0.5", "-pol", "nloc_av", "0.5"] + MGN,
     dict(grid=8, m=1.1 + 0.1j, interaction="nloc_av", nloc_rp=0.5, pol="nloc_av", pol_rp=0.5)),
    ("int_nloc_small", ["-int", "nloc", "0.1", "-pol", "nloc_av", "0.1"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), interaction="nloc", nloc_rp=0.1, pol="nloc_av",
          pol_rp=0.1)),
    ("int_nloc0", ["-int", "nloc", "0", "-pol", "nloc", "0"] + MGN,
     dict(grid=8, m=1.1 + 0.1j, interaction="nloc", nloc_rp=0.0, pol="nloc", pol_rp=0.0)),
    ("c1_nloc_av", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-int", "nloc_av", "0.2", "-pol", "nloc", "0.2",
                    "-eps", "8"],
     dict(grid=16, m=1.5, dpl=10, interaction="nloc_av", nloc_rp=0.2, pol="nloc", pol_rp=0.2, eps=1e-8)),
    ("c1_bcgs2", ["-grid", "16", "-dpl", "10", "-m", "1.5", "0", "-iter", "bcgs2", "-eps", "5"],
     dict(grid=16, m=1.5, dpl=10, iter="bcgs2")),
    ("ell_bcgs2_eps8", ["-iter", "bcgs2", "-eps", "8"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), iter="bcgs2", eps=1e-8)),
    # Csca and the asymmetry vector from the alldir grid (-Csca -asym; -alldir_inp, written by alldir_file below)
    # (converged solves, -eps 10, so that the integrals compare the quadrature and the fields, not where a solve
    # stopped)
    ("mgn_csca", ["-Csca", "-asym", "-eps", "10"] + MGN, dict(grid=8, m=1.1 + 0.1j, alldir="default", eps=1e-10)),
    ("ell_orient_csca", ["-Csca", "-asym", "-eps", "10", "-orient", "10", "20", "30"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), orient=(10, 20, 30), alldir="default",
          eps=1e-10)),
    ("c1_csca_adapt", ["-Csca", "-asym", "-eps", "10", "-grid", "16", "-dpl", "10", "-m", "1.5", "0"],
     dict(grid=16, m=1.5, dpl=10, alldir="adapt", eps=1e-10)),
    ("ell_csca_part", ["-Csca", "-asym", "-eps", "10", "-prop", "1", "2", "3"] + ELL + MGN,
     dict(grid=8, m=1.1 + 0.1j, shape="ellipsoid", pars=(0.5, 1.5), prop=(1, 2, 3), alldir="part", eps=1e-10)),
] + [("grid%d" % g, ["-grid", str(g), "-size", "8"] + M, dict(grid=g, m=1.1 + 0.1j, size=8.0))
     for g in (2, 4, 6, 10, 12, 18, 20, 24, 30, 32)]


# alldir_params.dat blocks (theta, phi): min, max, Jmin, Jmax, eps, equiv, periodic
ALLDIR = {
    "default": ((0, 180, 2, 6, 0, False, False), (0, 360, 2, 5, 0, True, True)),
    "adapt": ((0, 180, 3, 7, 1e-3, False, False), (0, 360, 2, 5, 1e-4, True, True)),
    "part": ((30, 150, 2, 4, 0, False, False), (0, 180, 1, 3, 0, False, False)),
}


def alldir_file(path, kind):
    with open(path, "w") as f:
        for name, (lo, hi, jmin, jmax, eps, eq, per) in zip(("theta", "phi"), ALLDIR[kind]):
            f.write("%s:\nmin=%g\nmax=%g\nJmin=%d\nJmax=%d\neps=%g\nequiv=%s\nperiodic=%s\n\n" % (
                name, lo, hi, jmin, jmax, eps, "true" if eq else "false", "true" if per else "false"))


def parse_run(rundir, stdout):
    log = open(os.path.join(rundir, "log")).read()
    out = {}
    out["ndip"] = int(re.search(r"Total number of occupied dipoles: (\d+)", log).group(1))
    out["box"] = [int(v) for v in re.search(r"box dimensions: (\d+)x(\d+)x(\d+)", log).groups()]
    out["grid"] = [int(v) for v in re.search(r"The FFT grid is: (\d+)x(\d+)x(\d+)", log).groups()]
    num = r"([-+]?[0-9.]+(?:[eE][-+]?\d+)?)([-+][0-9.]+(?:[eE][-+]?\d+)?)i"
    out["cc"] = [[float(a), float(b)] for a, b in re.findall(r"CoupleConstant:" + num, log)]
    # anisotropic prescriptions print the three diagonal components: CoupleConstant:(a+bi,c+di,e+fi)
    out["cc3"] = [[[float(a), float(b)] for a, b in re.findall(num, grp)]
                  for grp in re.findall(r"CoupleConstant:\(([^)]*)\)", log)]
    hist = {}
    cur = None
    for line in log.splitlines():
        m = re.match(r"here we go, calc ([XY])", line)
        if m:
            cur = m.group(1)
            hist[cur] = []
        m = re.match(r"RE_(\d+) = ([-+0-9.E]+)", line)
        if m and cur:
            hist[cur].append(float(m.group(2)))
    out["resid"] = hist
    cs = {}
    for pol in "YX":
        f = os.path.join(rundir, "CrossSec-" + pol)
        if os.path.exists(f):
            txt = open(f).read()
            cs[pol] = dict(Cext=float(re.search(r"Cext\s*=\s*([-+0-9.eE]+)", txt).group(1)),
                           Cabs=float(re.search(r"Cabs\s*=\s*([-+0-9.eE]+)", txt).group(1)))
            m = re.search(r"Csca\s*=\s*([-+0-9.eE]+)", txt)
            if m:
                cs[pol]["Csca"] = float(m.group(1))
                vec = r"\(([-+0-9.eE]+),([-+0-9.eE]+),([-+0-9.eE]+)\)"
                cs[pol]["Csca.g"] = [float(v) for v in re.search(r"Csca\.g\s*=\s*" + vec, txt).groups()]
                cs[pol]["g"] = [float(v) for v in re.search(r"\ng\s*=\s*" + vec, txt).groups()]
    out["cross"] = cs
    out["maxiter_warning"] = "haven't converged" in stdout + log
    mf = os.path.join(rundir, "mueller")
    if os.path.exists(mf) and "-ntheta" in open(os.path.join(rundir, "log")).read():
        rows = [l.split() for l in open(mf).read().splitlines()[1:] if l.strip()]
        out["mueller"] = [[float(v) for v in r] for r in rows]  # theta, s11 s12 ... s44
    return out


def main(ref_src=None):
    from oracle import oracle as O
    binp = O.build_reference(ref_src)
    if not binp:
        raise SystemExit("reference sources not found at " + (ref_src or O.ref_src_dir()))
    results = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, args, kw in CASES:
            full = args + ["-sym", "no"]
            if "alldir" in kw:
                alldir_file(os.path.join(tmp, name + "_alldir.dat"), kw["alldir"])
                full += ["-alldir_inp", name + "_alldir.dat"]
            rundir = os.path.join(tmp, name)
            p = subprocess.run([binp] + full + ["-dir", rundir], cwd=tmp, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError(name + ": " + p.stdout + p.stderr)
            res = parse_run(rundir, p.stdout)
            res.update(name=name, args=full, setup=kw)
            results.append(res)
            print(name, res["ndip"], res["grid"], res["cross"])
    # the published sample itself (generated by ADDA v1.3b4 on Windows), as printed in the reference tree
    sample = dict(name="published_sample", Cext_Y=135.0449047, Cabs_Y=-2.047466081e-16, niter_Y=22,
                  resid_Y_first=[1.0, 8.4752662637e-01, 8.2113292044e-01, 4.2639057157e-01, 3.0639031825e-01],
                  cc="0.005259037197+1.843854148e-05i")
    with open(os.path.join(HERE, "reference_runs.json"), "w") as f:
        json.dump(dict(reference="ADDA 1.3b6 sequential build + FFTW-subset shim", cases=results,
                       sample=sample), f, indent=1, default=lambda z: [z.real, z.imag] if isinstance(z, complex) else z)


if __name__ == "__main__":
    main(*sys.argv[1:])
